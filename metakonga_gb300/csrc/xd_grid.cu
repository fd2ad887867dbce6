// Cell grid: hash, sort, cell ranges (the reference's
// cu_calculateHashAndIndex / cu_calculateHashAndIndexForPolygonSphere /
// cu_reorderDataAndFindCellStart, source/mphysics_cuda_def.cu:58-108).
//
// Integer results are bit-exact with the reference: the cell coordinate is
// floor((p - wo) / cs) with IEEE double division (no reciprocal multiply),
// the sort is stable, and empty cells read cstart = 0xffffffff, cend = 0.
#include <cuda_runtime.h>

#include "xd_grid.cuh"
#include "xd_internal.cuh"

namespace xd {

__global__ void __launch_bounds__(256) k_hash(Params P, unsigned* __restrict__ hash,
                                              unsigned* __restrict__ index,
                                              const double* __restrict__ pos, unsigned n,
                                              unsigned sid)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    d4 p = ld4(pos, id);
    int3 c = grid_pos(P, p.x, p.y, p.z);
    hash[sid + id] = grid_hash(P, c.x, c.y, c.z);
    index[sid + id] = sid + id;
}

// cstart = 0xffffffff, cend = 0 over all ncell cells (def.cu:97-98), with
// 16-byte stores.
__global__ void __launch_bounds__(256) k_fill_cells(uint4* __restrict__ cstart4, uint4* __restrict__ cend4,
                                                    unsigned* __restrict__ cstart,
                                                    unsigned* __restrict__ cend, unsigned ncell)
{
    size_t n4 = ncell / 4;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        cstart4[i] = make_uint4(~0u, ~0u, ~0u, ~0u);
        cend4[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    size_t tail = (size_t)blockIdx.x * blockDim.x + threadIdx.x + n4 * 4;
    if (tail < ncell && tail >= n4 * 4) {
        cstart[tail] = ~0u;
        cend[tail] = 0u;
    }
}

// reorderDataAndFindCellStart_kernel (impl:166-212): a run of equal keys
// [b, e) gives cstart[h] = b, cend[h] = e.  Also writes the sorted keys and
// values back into hash/index (the reference sorts them in place) and
// sorted_index.  A key >= ncell sets *err and is not used as an index.
__global__ void __launch_bounds__(256) k_cell_bounds(const unsigned* __restrict__ skeys,
                                                     const unsigned* __restrict__ svals,
                                                     unsigned* __restrict__ hash,
                                                     unsigned* __restrict__ index,
                                                     unsigned* __restrict__ cstart,
                                                     unsigned* __restrict__ cend,
                                                     unsigned* __restrict__ sorted_index,
                                                     unsigned n, unsigned ncell,
                                                     unsigned* __restrict__ err)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    unsigned h = skeys[id];
    unsigned v = svals[id];
    if (hash != skeys) hash[id] = h;
    if (index != svals) index[id] = v;
    sorted_index[id] = v;
    if (h >= ncell) {
        atomicOr(err, 1u);
        return;
    }
    if (id == 0 || h != skeys[id - 1]) {
        cstart[h] = id;
        if (id > 0) {
            unsigned hp = skeys[id - 1];
            if (hp < ncell) cend[hp] = id;
        }
    }
    if (id == n - 1) cend[h] = id + 1;
}

int launch_cell_bounds_sorted(unsigned* hash, unsigned* index, unsigned* cstart, unsigned* cend,
                              unsigned* sorted_index, unsigned n, unsigned ncell, unsigned* err, cudaStream_t s)
{
    if (n == 0) return XD_OK;
    k_cell_bounds<<<div_up(n, 256), 256, 0, s>>>(hash, index, hash, index, cstart, cend, sorted_index, n, ncell,
                                                 err);
    return launch_status("cell bounds");
}

unsigned key_bits_for(unsigned ncell)
{
    unsigned bits = 0;
    while (bits < 32 && ((ncell - 1u) >> bits) != 0u) ++bits;
    return bits;
}

size_t reorder_scratch_bytes(unsigned n)
{
    return 256 + radix_sort_scratch_bytes(n);
}

int launch_hash(const Params& P, unsigned* hash, unsigned* index, const double* pos, unsigned n,
                unsigned sid, cudaStream_t s)
{
    if (n == 0) return XD_OK;
    k_hash<<<div_up(n, 256), 256, 0, s>>>(P, hash, index, pos, n, sid);
    return launch_status("calculate_hash_and_index");
}

int launch_fill_cells(unsigned* cstart, unsigned* cend, unsigned ncell, cudaStream_t s)
{
    if (ncell == 0) return XD_OK;
    unsigned n4 = ncell / 4 + 1;
    unsigned blocks = div_up(n4, 256);
    if (blocks > 152u * 16u) blocks = 152u * 16u;
    bool aligned = ((reinterpret_cast<uintptr_t>(cstart) | reinterpret_cast<uintptr_t>(cend)) & 15u) == 0;
    if (!aligned) {
        cudaError_t e1 = cudaMemsetAsync(cstart, 0xff, sizeof(unsigned) * (size_t)ncell, s);
        cudaError_t e2 = cudaMemsetAsync(cend, 0, sizeof(unsigned) * (size_t)ncell, s);
        if (e1 != cudaSuccess) return cuda_status(e1, "fill cstart");
        return cuda_status(e2, "fill cend");
    }
    k_fill_cells<<<blocks, 256, 0, s>>>(reinterpret_cast<uint4*>(cstart), reinterpret_cast<uint4*>(cend),
                                        cstart, cend, ncell);
    return launch_status("fill_cells");
}

// scratch layout: [0, 256) error word, then the radix sort's buffers
int reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart, unsigned* cend,
                                unsigned* sorted_index, unsigned n, unsigned ncell, void* scratch,
                                cudaStream_t s, bool check)
{
    if (n == 0) return launch_fill_cells(cstart, cend, ncell, s);
    unsigned* err = static_cast<unsigned*>(scratch);
    void* sort_scratch = static_cast<char*>(scratch) + 256;
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return cuda_status(e, "reorder: clear error word");
    unsigned *sk = nullptr, *sv = nullptr;
    int st = radix_sort_pairs(hash, index, n, key_bits_for(ncell), sort_scratch, s, &sk, &sv);
    if (st != XD_OK) return st;
    st = launch_fill_cells(cstart, cend, ncell, s);
    if (st != XD_OK) return st;
    k_cell_bounds<<<div_up(n, 256), 256, 0, s>>>(sk, sv, hash, index, cstart, cend, sorted_index, n,
                                                 ncell, err);
    st = launch_status("reorder_and_find_cell_start");
    if (st != XD_OK || !check) return st;
    unsigned herr = 0;
    e = cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "reorder: read error word");
    if (herr) return set_error(XD_ERR_INVALID, "reorder: a hash value is >= ncell (%u)", ncell);
    return XD_OK;
}

}  // namespace xd
