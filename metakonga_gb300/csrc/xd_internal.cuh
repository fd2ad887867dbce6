// Internal device/host helpers of libxdem (not part of the ABI).
//
// Arithmetic convention for the FP64 kernels that must reproduce the
// reference's results: every vector operation is component-wise, left to
// right, exactly as the reference's operators in
// include/mphysics_cuda_impl.cuh:19-63, and the translation units holding
// those kernels are compiled with --fmad=false so no multiply-add is fused.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xdem.h"

namespace xd {

// ---------------------------------------------------------------- vectors
struct d3 {
    double x, y, z;
};

__host__ __device__ __forceinline__ d3 mk(double x, double y, double z) { return d3{ x, y, z }; }
__host__ __device__ __forceinline__ d3 operator+(d3 a, d3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ d3 operator-(d3 a, d3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ d3 operator-(d3 a) { return mk(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ d3 operator*(double s, d3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ d3 operator/(d3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ void operator+=(d3& a, d3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__host__ __device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double length(d3 a) { return sqrt(dot(a, a)); }
__host__ __device__ __forceinline__ d3 cross(d3 a, d3 b)
{
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// packed double3 rows (24-byte stride) and double4 rows
__device__ __forceinline__ d3 ld3(const double* a, size_t i)
{
    const double* p = a + 3 * i;
    return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}
__device__ __forceinline__ d3 ld3rw(const double* a, size_t i)
{
    const double* p = a + 3 * i;
    return mk(p[0], p[1], p[2]);
}
__device__ __forceinline__ void st3(double* a, size_t i, d3 v)
{
    double* p = a + 3 * i;
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
struct d4 {
    double x, y, z, w;
};
__device__ __forceinline__ d4 ld4(const double* a, size_t i)
{
    const double2* p = reinterpret_cast<const double2*>(a + 4 * i);
    double2 lo = __ldg(p), hi = __ldg(p + 1);
    return d4{ lo.x, lo.y, hi.x, hi.y };
}
__host__ __device__ __forceinline__ d3 xyz(const d4& v) { return mk(v.x, v.y, v.z); }
__device__ __forceinline__ d3 ldv(const double* a) { return mk(a[0], a[1], a[2]); }

// ---------------------------------------------------------------- params
// The launch-time copy of device_parameters that every kernel receives by value.
struct Params {
    bool rolling;
    unsigned np;
    unsigned nsphere;
    unsigned ncell;
    unsigned gx, gy, gz;
    double dt;
    double half2dt;
    double cs;
    double cohesion;
    double g[3];
    double wo[3];
};

inline Params to_params(const xd_device_parameters& h)
{
    Params p;
    p.rolling = h.rollingCondition;
    p.np = h.np;
    p.nsphere = h.nsphere;
    p.ncell = h.ncell;
    p.gx = h.grid_size[0];
    p.gy = h.grid_size[1];
    p.gz = h.grid_size[2];
    p.dt = h.dt;
    p.half2dt = h.half2dt;
    p.cs = h.cell_size;
    p.cohesion = h.cohesion;
    for (int i = 0; i < 3; ++i) {
        p.g[i] = h.gravity[i];
        p.wo[i] = h.world_origin[i];
    }
    return p;
}

// calcGridPos (impl:74-83): floor((p - wo) / cs) with IEEE division.
__device__ __forceinline__ int3 grid_pos(const Params& P, double x, double y, double z)
{
    int3 c;
    c.x = (int)floor((x - P.wo[0]) / P.cs);
    c.y = (int)floor((y - P.wo[1]) / P.cs);
    c.z = (int)floor((z - P.wo[2]) / P.cs);
    return c;
}

// calcGridHash (impl:65-72): & (g-1) wrap, 24-bit multiplies.
__device__ __forceinline__ unsigned grid_hash(const Params& P, int cx, int cy, int cz)
{
    unsigned x = (unsigned)cx & (P.gx - 1u);
    unsigned y = (unsigned)cy & (P.gy - 1u);
    unsigned z = (unsigned)cz & (P.gz - 1u);
    return __umul24(__umul24(z, P.gy), P.gx) + __umul24(y, P.gx) + x;
}

// ---------------------------------------------------------------- errors
int set_error(int status, const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);
int launch_status(const char* where);

// shared scratch for the stateless calls (grown on demand)
void* workspace(size_t bytes, int* status);

inline unsigned div_up(unsigned a, unsigned b) { return (a + b - 1) / b; }

// radix sort (xd_sort.cu): keys per tile (8 warps x 4 rounds x 32 lanes)
constexpr unsigned kSortTile = 1024;
size_t radix_sort_scratch_bytes(unsigned n);
int radix_sort_pairs(unsigned* keys, unsigned* vals, unsigned n, unsigned key_bits, void* scratch,
                     cudaStream_t s, unsigned** out_keys, unsigned** out_vals);

}  // namespace xd
