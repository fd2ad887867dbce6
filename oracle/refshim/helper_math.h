/*
 * Host stand-in for the CUDA-samples helper_math.h (oracle pin build only).
 *
 * Two groups of operators:
 *   1. float3/float4 arithmetic by value, which the reference's FP32 kernels
 *      take from helper_math.h;
 *   2. const-reference overloads of the reference's own double3 operators.
 *      The reference declares them on non-const references (e.g.
 *      `double3 operator+(double3&, double3&)`) and calls them with
 *      temporaries, which only MSVC accepts.  For lvalue arguments overload
 *      resolution still picks the reference's own operator; for temporaries it
 *      picks these, which compute the same expression component by component.
 */
#ifndef XD_REFSHIM_HELPER_MATH_H
#define XD_REFSHIM_HELPER_MATH_H
#include <cmath>
#include "vector_types.h"

/* ---- group 2: double3, const-reference twins (not for the legacy header,
 *      cu_dem_impl.cuh, whose own double3 operators take values) ---- */
#ifndef XD_REFSHIM_LEGACY
inline double dot(const double3& a, const double3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double3 operator-(const double3& a, const double3& b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline double3 operator-(const double3& a) { return make_double3(-a.x, -a.y, -a.z); }
inline double3 operator*(double s, const double3& a) { return make_double3(s * a.x, s * a.y, s * a.z); }
inline double3 operator+(const double3& a, const double3& b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline double3 operator/(const double3& a, double s) { return make_double3(a.x / s, a.y / s, a.z / s); }
inline double length(const double3& a) { return std::sqrt(dot(a, a)); }
#endif

/* ---- group 1: float vectors ---- */
inline float3 make_float3(const float4& a) { return make_float3(a.x, a.y, a.z); }
inline float3 make_float3(float s) { return make_float3(s, s, s); }
inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
inline void operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
inline void operator-=(float3& a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float3 a) { return std::sqrt(dot(a, a)); }
inline float3 cross(float3 a, float3 b) { return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float3 normalize(float3 a) { float inv = 1.0f / std::sqrt(dot(a, a)); return a * inv; }
inline float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

#endif
