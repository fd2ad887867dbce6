/*
 * Host stand-in for CUDA's vector_types.h, used only to compile the
 * reference's kernel header as host C++ for the oracle pin.  Sizes match the
 * CUDA types (double4 = 32 B, double3 = 24 B, float4 = 16 B, float3 = 12 B).
 */
#ifndef XD_REFSHIM_VECTOR_TYPES_H
#define XD_REFSHIM_VECTOR_TYPES_H

struct int3 { int x, y, z; };
struct uint3 { unsigned int x, y, z; };
struct float3 { float x, y, z; };
struct __attribute__((aligned(16))) float4 { float x, y, z, w; };
struct double3 { double x, y, z; };
struct __attribute__((aligned(16))) double4 { double x, y, z, w; };

static inline int3 make_int3(int x, int y, int z) { int3 r = { x, y, z }; return r; }
static inline uint3 make_uint3(unsigned x, unsigned y, unsigned z) { uint3 r = { x, y, z }; return r; }
static inline float3 make_float3(float x, float y, float z) { float3 r = { x, y, z }; return r; }
static inline float4 make_float4(float x, float y, float z, float w) { float4 r = { x, y, z, w }; return r; }
static inline double3 make_double3(double x, double y, double z) { double3 r = { x, y, z }; return r; }
static inline double4 make_double4(double x, double y, double z, double w) { double4 r = { x, y, z, w }; return r; }

#endif
