/*
 * Host-emulation prelude for compiling the reference's CUDA kernel header
 * (include/mphysics_cuda_impl.cuh of the xdynamics reference) with g++ as
 * plain C++, so that its FP64 kernels can be executed on the CPU as a pinned
 * oracle.  TEST INFRASTRUCTURE ONLY: nothing here is shipped or measured.
 *
 * What the prelude does:
 *   - CUDA function/variable space qualifiers become empty (kernels turn into
 *     ordinary functions, __constant__ / __shared__ objects into globals);
 *   - blockIdx / threadIdx / blockDim / gridDim become host globals that the
 *     launch emulator (oracle/ref_driver.cpp) sets before each "thread" call;
 *   - __umul24/__mul24 follow the PTX definition (low 32 bits of the product
 *     of the low 24 bits);
 *   - __syncthreads() is a no-op: the emulator runs the threads of a block in
 *     ascending order, which gives the same result as a parallel launch for
 *     every kernel that is emulated (the only barrier-using kernel, the cell
 *     boundary kernel, reads sharedHash[t] that thread t-1 already wrote).
 *   - min/max on floating point follow CUDA's device overloads (fmin/fmax).
 */
#ifndef XD_HOST_PRELUDE_H
#define XD_HOST_PRELUDE_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

using std::abs;
using std::floor;
using std::sqrt;
using std::pow;
using std::log;
using std::atan;
using std::sin;
using std::cos;

#define __device__
#define __host__
#define __global__
#define __constant__
#define __shared__
#define __forceinline__ inline
#define __device_builtin__
#define __builtin_align__(a) __attribute__((aligned(a)))

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef unsigned int uint;

#include "vector_types.h"

extern uint3 blockIdx;
extern uint3 threadIdx;
extern uint3 blockDim;
extern uint3 gridDim;

inline unsigned int __umul24(unsigned int a, unsigned int b)
{
    return (a & 0xffffffu) * (b & 0xffffffu);
}

inline int __mul24(int a, int b)
{
    /* sign-extend the low 24 bits of each operand, keep the low 32 bits */
    long long sa = (long long)((a << 8)) >> 8;
    long long sb = (long long)((b << 8)) >> 8;
    return (int)(unsigned int)(sa * sb);
}

inline void __syncthreads() {}

inline double min(double a, double b) { return std::fmin(a, b); }
inline double max(double a, double b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }

#endif
