// Allocation-free variant of xd_reorder_and_find_cell_start.
//
// Some callers cannot allocate device memory once they are running: a host
// application that hands out all device memory from its own pool at start-up
// and forbids allocation inside its time loop, or a process held to a fixed
// device-memory budget where a late allocation may fail.  The ordinary entry
// point grows a library workspace with cudaMalloc on demand (the reference's
// thrust sort allocates temporary storage on every call,
// source/mphysics_cuda_def.cu:92-94).  This variant takes its sort scratch
// from the file-scope device array below instead, so it performs no
// allocation at all.
//
// * The array holds the scratch for up to XD_NOALLOC_MAX_ENTRIES entries
//   (about 9.4 MB); it lives in every device that loads the library until the
//   process exits.  Larger sorts are rejected with XD_ERR_CAPACITY.
// * Every call shares the array, which keeps the previous call's contents.
//   The only word that must start at zero (the out-of-range-hash flag) is
//   cleared by each call; every other scratch byte is written before it is
//   read.  Calls whose work overlaps on the GPU (different streams, or
//   different host threads) race on the array: serialise them.
// * In host code the array's name is only a host-side stand-in, so every call
//   takes the device address with cudaGetSymbolAddress, with the caller's
//   device current (a call with n = 0 included), and checks its return code.
//   The address is not cached: after cudaDeviceReset the array has a new one.
// * The library is built without relocatable device code, so this file is a
//   CUDA module of its own.  Under lazy module loading (the default of CUDA
//   12.2 and later) the driver reserves the array's memory only when the
//   module is first used, which is this entry point's first call on a
//   device.  A caller that hands out all device memory from its own pool
//   must therefore make one call on each device before the pool takes its
//   memory -- a call with n = 0 only clears the cell arrays and serves as
//   that set-up -- or run with CUDA_MODULE_LOADING=EAGER.  That first call
//   should also come before any stream capture on the device.  Later calls
//   reserve nothing.
#include <cuda_runtime.h>

#include "xd_grid.cuh"
#include "xd_internal.cuh"

namespace {

// Same layout as xd_grid.cu / xd_sort.cu for n = XD_NOALLOC_MAX_ENTRIES:
// error word (256 B) + alternate keys + alternate values + per-tile digit
// counts (256 x tiles) + scan chunk sums, each rounded up to 256 bytes.
constexpr size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kMax = XD_NOALLOC_MAX_ENTRIES;
constexpr size_t kTiles = (kMax + xd::kSortTile - 1) / xd::kSortTile;
constexpr size_t kHist = 256 * kTiles;
constexpr size_t kChunks = (kHist + 4095) / 4096;
constexpr size_t kScratchBytes = 256 + al256(4 * kMax) + al256(4 * kMax) + al256(4 * kHist) +
                                 al256(4 * kChunks);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch on the current device.
int scratch_address(void** out)
{
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return xd::cuda_status(e, "reorder_noalloc: cudaGetSymbolAddress");
    *out = p;
    return XD_OK;
}

}  // namespace

extern "C" int xd_reorder_and_find_cell_start_noalloc(unsigned* hash, unsigned* index,
                                                      unsigned* cstart, unsigned* cend,
                                                      unsigned* sorted_index, unsigned n,
                                                      unsigned ncell, void* stream)
{
    using namespace xd;
    if (!cstart || !cend) return set_error(XD_ERR_INVALID, "reorder_noalloc: null cell arrays");
    if (ncell == 0) return set_error(XD_ERR_INVALID, "reorder_noalloc: ncell must be > 0");
    if (n > 0 && (!hash || !index || !sorted_index))
        return set_error(XD_ERR_INVALID, "reorder_noalloc: null pointer");
    if ((size_t)n > kMax)
        return set_error(XD_ERR_CAPACITY,
                         "reorder_noalloc: %u entries exceed the fixed scratch's maximum of %u "
                         "(use xd_reorder_and_find_cell_start)", n, (unsigned)kMax);
    if (reorder_scratch_bytes(n) > kScratchBytes)
        return set_error(XD_ERR_CAPACITY, "reorder_noalloc: scratch layout exceeds the fixed array");
    void* scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st != XD_OK) return st;
    return reorder_and_find_cell_start(hash, index, cstart, cend, sorted_index, n, ncell, scratch,
                                       static_cast<cudaStream_t>(stream), true);
}
