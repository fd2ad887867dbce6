// Stable LSD radix sort of 32-bit (key, value) pairs on sm_103a.
//
// Replaces thrust::sort_by_key in cu_reorderDataAndFindCellStart
// (source/mphysics_cuda_def.cu:92-94).  The cell grid's keys only span
// ceil(log2(ncell)) bits (21 for the reference's 128^3 grid), so the sort
// runs ceil(bits / 8) passes of an 8-bit digit.  Each pass is three launches
// with no inter-block waiting:
//   1. k_tile_hist   per-tile digit counts, stored digit-major [256][tiles];
//   2. k_scan_*      exclusive scan of those counts -> each (digit, tile)'s
//                    first output slot;
//   3. k_scatter     stable in-tile ranking with __match_any_sync and a
//                    coalesced read of the tile, then the scatter.
// A tile is 1024 keys: 8 warps x 4 rounds x 32 lanes, visited in index
// order, so equal digits keep their input order and the sort is stable.
#include <cuda_runtime.h>

#include "xd_internal.cuh"

namespace xd {
namespace {

constexpr int kBits = 8;
constexpr int kRadix = 1 << kBits;
constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kRounds = 4;
constexpr int kTile = kThreads * kRounds;   // 1024
static_assert(kTile == (int)kSortTile, "tile size shared with the fixed-scratch entry point");
constexpr int kScanThreads = 1024;
constexpr int kScanChunk = 4096;            // elements per scan block

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__global__ void __launch_bounds__(kThreads) k_tile_hist(const unsigned* __restrict__ keys, unsigned n,
                                                        unsigned shift, unsigned ntiles,
                                                        unsigned* __restrict__ hist)
{
    __shared__ unsigned cnt[kRadix];
    for (int i = threadIdx.x; i < kRadix; i += kThreads) cnt[i] = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const size_t base = (size_t)blockIdx.x * kTile;
    for (int r = 0; r < kRounds; ++r) {
        size_t idx = base + (size_t)r * kThreads + threadIdx.x;
        bool valid = idx < n;
        unsigned d = valid ? ((__ldg(keys + idx) >> shift) & (kRadix - 1)) : kRadix;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        if (valid && (__ffs(peers) - 1) == (int)lane) atomicAdd(&cnt[d], (unsigned)__popc(peers));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kRadix; i += kThreads) hist[(size_t)i * ntiles + blockIdx.x] = cnt[i];
}

// block-wide exclusive scan of one value per thread (1024 threads)
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* warp_sums, unsigned* total)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = warp_sums[lane];
        unsigned s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= (unsigned)o) s += y;
        }
        warp_sums[lane] = s - w;
        if (lane == 31) *total = s;
    }
    __syncthreads();
    return x - v + warp_sums[warp];
}

// Pass 1 of the scan: each block scans kScanChunk elements in place
// (exclusive) and writes its chunk total.
__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(unsigned* __restrict__ data, size_t m,
                                                              unsigned* __restrict__ chunk_sums)
{
    __shared__ unsigned warp_sums[32];
    __shared__ unsigned total;
    const size_t base = (size_t)blockIdx.x * kScanChunk;
    constexpr int per = kScanChunk / kScanThreads;   // 4 consecutive elements per thread
    unsigned v[per];
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < per; ++i) {
        size_t idx = base + (size_t)threadIdx.x * per + i;
        v[i] = idx < m ? data[idx] : 0u;
        s += v[i];
    }
    unsigned off = block_exclusive_scan(s, warp_sums, &total);
#pragma unroll
    for (int i = 0; i < per; ++i) {
        size_t idx = base + (size_t)threadIdx.x * per + i;
        if (idx < m) data[idx] = off;
        off += v[i];
    }
    if (threadIdx.x == 0) chunk_sums[blockIdx.x] = total;
}

// Pass 2: one block scans the chunk totals in place (exclusive), looping
// over them in groups of 1024.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(unsigned* __restrict__ sums, unsigned nchunks)
{
    __shared__ unsigned warp_sums[32];
    __shared__ unsigned total;
    unsigned carry = 0;
    for (unsigned b = 0; b < nchunks; b += kScanThreads) {
        unsigned i = b + threadIdx.x;
        unsigned v = i < nchunks ? sums[i] : 0u;
        unsigned off = block_exclusive_scan(v, warp_sums, &total);
        if (i < nchunks) sums[i] = off + carry;
        carry += total;
        __syncthreads();
    }
}

// Pass 3: add each chunk's offset.
__global__ void __launch_bounds__(kScanThreads) k_scan_add(unsigned* __restrict__ data, size_t m,
                                                           const unsigned* __restrict__ sums)
{
    const unsigned add = sums[blockIdx.x];
    if (add == 0) return;
    const size_t base = (size_t)blockIdx.x * kScanChunk;
    for (int i = threadIdx.x; i < kScanChunk; i += kScanThreads) {
        size_t idx = base + i;
        if (idx < m) data[idx] += add;
    }
}

__global__ void __launch_bounds__(kThreads) k_scatter(const unsigned* __restrict__ kin,
                                                      const unsigned* __restrict__ vin,
                                                      unsigned* __restrict__ kout,
                                                      unsigned* __restrict__ vout, unsigned n,
                                                      unsigned shift, unsigned ntiles,
                                                      const unsigned* __restrict__ offsets)
{
    __shared__ unsigned wcnt[kWarps][kRadix];
    __shared__ unsigned gbase[kRadix];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * kRadix; i += kThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();

    const size_t wbase = (size_t)blockIdx.x * kTile + (size_t)warp * (kRounds * 32);
    const unsigned ltmask = lanemask_lt();
    unsigned key[kRounds], val[kRounds], rank[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        size_t idx = wbase + (size_t)r * 32 + lane;
        bool valid = idx < n;
        key[r] = valid ? __ldg(kin + idx) : 0u;
        val[r] = valid ? __ldg(vin + idx) : 0u;
        unsigned d = valid ? ((key[r] >> shift) & (kRadix - 1)) : kRadix;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        unsigned before = 0;
        if (valid) before = wcnt[warp][d];
        rank[r] = before + __popc(peers & ltmask);
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == (int)lane) wcnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kThreads) {
        unsigned run = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            unsigned c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
        gbase[d] = offsets[(size_t)d * ntiles + blockIdx.x];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        size_t idx = wbase + (size_t)r * 32 + lane;
        if (idx < n) {
            unsigned d = (key[r] >> shift) & (kRadix - 1);
            unsigned dst = gbase[d] + wcnt[warp][d] + rank[r];
            kout[dst] = key[r];
            vout[dst] = val[r];
        }
    }
}

struct SortLayout {
    size_t keys_alt, vals_alt, hist, sums, total;
    unsigned ntiles, nchunks;
    size_t m;
};

SortLayout layout(unsigned n)
{
    SortLayout L;
    L.ntiles = div_up(n ? n : 1u, (unsigned)kTile);
    L.m = (size_t)kRadix * L.ntiles;
    L.nchunks = (unsigned)((L.m + kScanChunk - 1) / kScanChunk);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    L.keys_alt = 0;
    L.vals_alt = L.keys_alt + al(sizeof(unsigned) * (size_t)n);
    L.hist = L.vals_alt + al(sizeof(unsigned) * (size_t)n);
    L.sums = L.hist + al(sizeof(unsigned) * L.m);
    L.total = L.sums + al(sizeof(unsigned) * (size_t)L.nchunks);
    return L;
}

}  // namespace

size_t radix_sort_scratch_bytes(unsigned n) { return layout(n).total; }

// Sorts (keys, vals) by the low key_bits bits.  The result is left either in
// the input arrays or in the scratch's alternate buffers; *out_keys/*out_vals
// point at it.
int radix_sort_pairs(unsigned* keys, unsigned* vals, unsigned n, unsigned key_bits, void* scratch,
                     cudaStream_t s, unsigned** out_keys, unsigned** out_vals)
{
    *out_keys = keys;
    *out_vals = vals;
    if (n <= 1 || key_bits == 0) return XD_OK;
    if (key_bits > 32) key_bits = 32;
    SortLayout L = layout(n);
    char* base = static_cast<char*>(scratch);
    unsigned* kalt = reinterpret_cast<unsigned*>(base + L.keys_alt);
    unsigned* valt = reinterpret_cast<unsigned*>(base + L.vals_alt);
    unsigned* hist = reinterpret_cast<unsigned*>(base + L.hist);
    unsigned* sums = reinterpret_cast<unsigned*>(base + L.sums);
    unsigned *ks = keys, *vs = vals, *kd = kalt, *vd = valt;
    for (unsigned shift = 0; shift < key_bits; shift += kBits) {
        k_tile_hist<<<L.ntiles, kThreads, 0, s>>>(ks, n, shift, L.ntiles, hist);
        k_scan_chunks<<<L.nchunks, kScanThreads, 0, s>>>(hist, L.m, sums);
        k_scan_sums<<<1, kScanThreads, 0, s>>>(sums, L.nchunks);
        k_scan_add<<<L.nchunks, kScanThreads, 0, s>>>(hist, L.m, sums);
        k_scatter<<<L.ntiles, kThreads, 0, s>>>(ks, vs, kd, vd, n, shift, L.ntiles, hist);
        unsigned* t;
        t = ks; ks = kd; kd = t;
        t = vs; vs = vd; vd = t;
    }
    *out_keys = ks;
    *out_vals = vs;
    return launch_status("radix_sort_pairs");
}

}  // namespace xd
