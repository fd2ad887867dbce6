// Single-precision twins of the live API (the reference's float kernels,
// mphysics_cuda_impl.cuh:1094-1895, launched by mphysics_cuda_def.cu:254-466):
// velocity-Verlet, cell hash, particle-particle, plane, cube and triangle
// contact forces, and reductionD3 over float3 rows.
//
// Layouts: pos and triangle spheres are float4 rows; vel, acc, omega, alpha,
// force and moment packed float3 rows (12-byte stride); mass and inertia float.
//
// Compiled with --fmad=false.  Each expression follows the reference's float
// kernel in order and type, including the double constants that promote parts
// of getConstant and cohesionForce to double (M_PI / log(rest), the 4.0 and
// 1.0 of the damping coefficient).  Differences from the reference, within a
// few float ulps: CUDA's powf/logf/sqrtf against whatever the reference's
// build used, and the body reaction, which the reference adds with racing
// non-atomic += (impl:1886-1887) and this file sums in a fixed order.
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "xd_grid.cuh"
#include "xd_internal.cuh"

namespace xd {

const Params* params();   // the FP64 parameter block (xd_capi.cu)

namespace {

struct ParamsF {
    unsigned np, nsphere, ncell;
    unsigned gsx, gsy, gsz;   // the FP32 block's grid size (not used by the hash, as in the reference)
    float dt, half2dt, cs, cohesion;
    float g[3], wo[3];
    // calcGridHash (impl:65-72) wraps with the FP64 block's grid size
    unsigned hx, hy, hz;
};

std::mutex g_f_mu;
bool g_have_f = false;
xd_device_parameters_f g_f;

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mkf(float x, float y, float z) { return f3{ x, y, z }; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mkf(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mkf(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator-(f3 a) { return mkf(-a.x, -a.y, -a.z); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mkf(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return mkf(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ void operator+=(f3& a, f3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__device__ __forceinline__ float dotf(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float lenf(f3 a) { return sqrtf(dotf(a, a)); }
__device__ __forceinline__ f3 crossf(f3 a, f3 b)
{
    return mkf(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 ldf3(const float* a, size_t i)
{
    const float* p = a + 3 * i;
    return mkf(p[0], p[1], p[2]);
}
__device__ __forceinline__ void stf3(float* a, size_t i, f3 v)
{
    float* p = a + 3 * i;
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
__device__ __forceinline__ f3 arr3(const float* v) { return mkf(v[0], v[1], v[2]); }

// calcGridPos(float3) (impl:1095-1103) and calcGridHash (impl:65-72)
__device__ __forceinline__ int3 grid_pos_f(const ParamsF& P, float x, float y, float z)
{
    int3 c;
    c.x = (int)floorf((x - P.wo[0]) / P.cs);
    c.y = (int)floorf((y - P.wo[1]) / P.cs);
    c.z = (int)floorf((z - P.wo[2]) / P.cs);
    return c;
}
__device__ __forceinline__ unsigned grid_hash_f(const ParamsF& P, int cx, int cy, int cz)
{
    unsigned x = (unsigned)cx & (P.hx - 1u);
    unsigned y = (unsigned)cy & (P.hy - 1u);
    unsigned z = (unsigned)cz & (P.hz - 1u);
    return __umul24(__umul24(z, P.hy), P.hx) + __umul24(y, P.hx) + x;
}

// getConstant, TCM = 1 (impl:1229-1271), float arguments
struct FcF {
    float kn, vn, ks, vs, mu;
};
__device__ __forceinline__ FcF get_constant_f(float ir, float jr, float im, float jm,
                                              const xd_contact_property_f& cp)
{
    FcF c;
    float Meq = jm ? (im * jm) / (im + jm) : im;
    float Req = jr ? (ir * jr) / (ir + jr) : ir;
    float Eeq = (cp.Ei * cp.Ej) / (cp.Ei * (1 - cp.prj * cp.prj) + cp.Ej * (1 - cp.pri * cp.pri));
    float beta = (float)(M_PI / (double)logf(cp.rest));
    c.kn = (4.0f / 3.0f) * Eeq * sqrtf(Req);
    c.vn = (float)sqrt((4.0 * (double)Meq * (double)c.kn) / (1.0 + (double)(beta * beta)));
    c.ks = c.kn * cp.sratio;
    c.vs = c.vn * cp.sratio;
    c.mu = cp.fric;
    return c;
}

// cohesionForce (impl:1274-1293)
__device__ __forceinline__ float cohesion_f(float ri, float rj, float Ei, float Ej, float pri, float prj,
                                            float coh, float Fn)
{
    float cf = 0.f;
    if (coh) {
        float req = (ri * rj / (ri + rj));
        float Eeq = ((1.0f - pri * pri) / Ei) + ((1.0f - prj * prj) / Ej);
        float rcp = (3.0f * req * (-Fn)) / (4.0f * (1.0f / Eeq));
        float rc = powf(rcp, 1.0f / 3.0f);
        float Ac = (float)(M_PI * (double)rc * (double)rc);
        cf = coh * Ac;
    }
    return cf;
}

// DHSModel (impl:1320-1341): Ft and M are assigned only when the tangential
// slip is non-zero, so they carry over to the next contact of the thread.
__device__ __forceinline__ void dhs_f(const FcF& c, float ir, float jr, float Ei, float Ej, float pri, float prj,
                                      float coh, float cdist, f3 dv, f3 unit, float dt, f3& Ft, f3& Fn, f3& M)
{
    float fsn = -c.kn * powf(cdist, 1.5f);
    float fdn = c.vn * dotf(dv, unit);
    float fca = cohesion_f(ir, jr, Ei, Ej, pri, prj, coh, fsn);
    Fn = (fsn + fca + fdn) * unit;
    f3 e = dv - dotf(dv, unit) * unit;
    float mag_e = lenf(e);
    if (mag_e) {
        f3 sh = e / mag_e;
        float ds = mag_e * dt;
        Ft = fminf(c.ks * ds + c.vs * (dotf(dv, sh)), c.mu * lenf(Fn)) * sh;
        M = crossf(ir * unit, Ft);
    }
}

// ------------------------------------------------------------ integrator

__global__ void __launch_bounds__(256) k_vv_position_f(ParamsF P, float4* __restrict__ pos,
                                                       const float* __restrict__ vel,
                                                       const float* __restrict__ acc, unsigned np)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    f3 v = ldf3(vel, id), a = ldf3(acc, id);
    f3 p = P.dt * v + P.half2dt * a;
    float4 q = pos[id];
    q.x += p.x;
    q.y += p.y;
    q.z += p.z;
    pos[id] = q;
}

__global__ void __launch_bounds__(256) k_vv_velocity_f(ParamsF P, float* __restrict__ vel, float* __restrict__ acc,
                                                       float* __restrict__ omega, float* __restrict__ alpha,
                                                       float* __restrict__ force, float* __restrict__ moment,
                                                       const float* __restrict__ mass,
                                                       const float* __restrict__ iner, unsigned np)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    f3 v = ldf3(vel, id), L = ldf3(acc, id), av = ldf3(omega, id), aa = ldf3(alpha, id);
    float m = mass[id], in = iner[id];
    const float h = 0.5f * P.dt;
    v += h * L;
    av += h * aa;
    L = (1.0f / m) * ldf3(force, id);
    aa = (1.0f / in) * ldf3(moment, id);
    v += h * L;
    av += h * aa;
    stf3(force, id, m * mkf(P.g[0], P.g[1], P.g[2]));
    stf3(moment, id, mkf(0.0f, 0.0f, 0.0f));
    stf3(vel, id, v);
    stf3(omega, id, av);
    stf3(acc, id, L);
    stf3(alpha, id, aa);
}

// ------------------------------------------------------------ cell hash

__global__ void __launch_bounds__(256) k_hash_f(ParamsF P, unsigned* __restrict__ hash, unsigned* __restrict__ index,
                                                const float4* __restrict__ pos, unsigned n, unsigned sid)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    float4 p = pos[id];
    int3 g = grid_pos_f(P, p.x, p.y, p.z);
    hash[sid + id] = grid_hash_f(P, g.x, g.y, g.z);
    index[sid + id] = sid + id;
}

// ------------------------------------------------------------ particle-particle

__global__ void __launch_bounds__(128) k_p2p_f(ParamsF P, const float4* __restrict__ pos,
                                               const float* __restrict__ vel, const float* __restrict__ omega,
                                               float* __restrict__ force, float* __restrict__ moment,
                                               const float* __restrict__ mass, const unsigned* __restrict__ sorted,
                                               const unsigned* __restrict__ cstart,
                                               const unsigned* __restrict__ cend,
                                               const xd_contact_property_f* __restrict__ cpp, unsigned np)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    const xd_contact_property_f cp = *cpp;
    float4 ipos = pos[id];
    f3 ivel = ldf3(vel, id), iomega = ldf3(omega, id);
    int3 gp = grid_pos_f(P, ipos.x, ipos.y, ipos.z);
    float ir = ipos.w, im = mass[id];
    f3 Ft = mkf(0, 0, 0), Fn = mkf(0, 0, 0), M = mkf(0, 0, 0);
    f3 sumF = mkf(0, 0, 0), sumM = mkf(0, 0, 0);
    for (int z = -1; z <= 1; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                unsigned h = grid_hash_f(P, gp.x + x, gp.y + y, gp.z + z);
                unsigned st = cstart[h];
                if (st == 0xffffffffu) continue;
                unsigned en = cend[h];
                for (unsigned j = st; j < en; j++) {
                    unsigned k = sorted[j];
                    if (id == k || k >= np) continue;
                    float4 jpos = pos[k];
                    f3 jvel = ldf3(vel, k), jomega = ldf3(omega, k);
                    float jr = jpos.w, jm = mass[k];
                    f3 rp = mkf(jpos.x - ipos.x, jpos.y - ipos.y, jpos.z - ipos.z);
                    float dist = lenf(rp);
                    float cdist = (ir + jr) - dist;
                    if (cdist > 0) {
                        f3 unit = rp / dist;
                        f3 rv = jvel + crossf(jomega, -jr * unit) - (ivel + crossf(iomega, ir * unit));
                        FcF c = get_constant_f(ir, jr, im, jm, cp);
                        dhs_f(c, ir, jr, cp.Ei, cp.Ej, cp.pri, cp.prj, cp.coh, cdist, rv, unit, P.dt, Ft, Fn, M);
                        sumF += Fn + Ft;
                        sumM += M;
                    }
                }
            }
    f3 f = ldf3(force, id), m = ldf3(moment, id);
    f += sumF;
    m += sumM;
    stf3(force, id, f);
    stf3(moment, id, m);
}

// ------------------------------------------------------------ planes

// particle_plane_contact_detection(float) (impl:1427-1514)
__device__ __forceinline__ float plane_detection_f(const xd_plane_info_f& pe, f3 xp, f3 wp, f3& u, float r)
{
    float a_l1 = powf(wp.x - pe.l1, 2.0f);
    float b_l2 = powf(wp.y - pe.l2, 2.0f);
    float sqa = wp.x * wp.x;
    float sqb = wp.y * wp.y;
    float sqc = wp.z * wp.z;
    float sqr = r * r;
    const f3 xw = arr3(pe.xw), uw = arr3(pe.uw), w2 = arr3(pe.w2), w3 = arr3(pe.w3), w4 = arr3(pe.w4);
    if (fabsf(wp.z) < r && (wp.x > 0 && wp.x < pe.l1) && (wp.y > 0 && wp.y < pe.l2)) {
        f3 dp = xp - xw;
        f3 uu = uw / lenf(uw);
        int pp = -(dotf(dp, uw) < 0 ? -1 : 1);
        u = (float)pp * uu;
        return r - fabsf(dotf(dp, u));
    }
    if (wp.x < 0 && wp.y < 0 && (sqa + sqb + sqc) < sqr) {
        f3 X = xp - xw; float h = lenf(X); u = X / h; return r - h;
    } else if (wp.x > pe.l1 && wp.y < 0 && (a_l1 + sqb + sqc) < sqr) {
        f3 X = xp - w2; float h = lenf(X); u = X / h; return r - h;
    } else if (wp.x > pe.l1 && wp.y > pe.l2 && (a_l1 + b_l2 + sqc) < sqr) {
        f3 X = xp - w3; float h = lenf(X); u = X / h; return r - h;
    } else if (wp.x < 0 && wp.y > pe.l2 && (sqa + b_l2 + sqc) < sqr) {
        f3 X = xp - w4; float h = lenf(X); u = X / h; return r - h;
    }
    f3 X, wj;
    if ((wp.x > 0 && wp.x < pe.l1) && wp.y < 0 && (sqb + sqc) < sqr) {
        X = xp - xw; wj = w2 - xw;
    } else if ((wp.x > 0 && wp.x < pe.l1) && wp.y > pe.l2 && (b_l2 + sqc) < sqr) {
        X = xp - w4; wj = w3 - w4;
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x < 0 && (sqr + sqc) < sqr) {
        X = xp - xw; wj = w4 - xw;
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x > pe.l1 && (a_l1 + sqc) < sqr) {
        X = xp - w2; wj = w3 - w2;
    } else {
        return -1.0f;
    }
    f3 us = wj / lenf(wj);
    f3 hs = X - (dotf(X, us)) * us;
    float h = lenf(hs);
    u = -hs / h;
    return r - h;
}

// plane_contact_force_kernel<1>(float) (impl:1516-1564), planes applied in
// order (cube: six planes, one property)
__global__ void __launch_bounds__(128) k_planes_f(ParamsF P, const xd_plane_info_f* __restrict__ planes,
                                                  unsigned nplanes, const float4* __restrict__ pos,
                                                  const float* __restrict__ vel, const float* __restrict__ omega,
                                                  float* __restrict__ force, float* __restrict__ moment,
                                                  const xd_contact_property_f* __restrict__ cpp,
                                                  const float* __restrict__ mass, unsigned np)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    const xd_contact_property_f cp = *cpp;
    float m = mass[id];
    float4 ipos = pos[id];
    f3 ipos3 = mkf(ipos.x, ipos.y, ipos.z);
    float r = ipos.w;
    f3 ivel = ldf3(vel, id), iomega = ldf3(omega, id);
    f3 fo = ldf3(force, id), mo = ldf3(moment, id);
    for (unsigned w = 0; w < nplanes; ++w) {
        const xd_plane_info_f pe = planes[w];
        f3 Fn = mkf(0, 0, 0), Ft = mkf(0, 0, 0), M = mkf(0, 0, 0);
        f3 dp = ipos3 - arr3(pe.xw);
        f3 unit = mkf(0, 0, 0);
        f3 wp = mkf(dotf(dp, arr3(pe.u1)), dotf(dp, arr3(pe.u2)), dotf(dp, arr3(pe.uw)));
        float cdist = plane_detection_f(pe, ipos3, wp, unit, r);
        if (cdist > 0) {
            f3 dv = -(ivel + crossf(iomega, r * unit));
            FcF c = get_constant_f(r, 0.f, m, 0.f, cp);
            dhs_f(c, 0, 0, 0, 0, 0, 0, cp.coh, cdist, dv, unit, P.dt, Ft, Fn, M);
        }
        fo += Fn + Ft;
        mo += M;
    }
    stf3(force, id, fo);
    stf3(moment, id, mo);
}

// ------------------------------------------------------------ triangles

// closestPtPointTriangle(float) (impl:1718-1774)
__device__ __forceinline__ f3 closest_pt_f(f3 a, f3 b, f3 c, f3 p)
{
    f3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dotf(ab, ap), d2 = dotf(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    f3 bp = p - b;
    float d3 = dotf(ab, bp), d4 = dotf(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = d1 / (d1 - d3);
        return a + v * ab;
    }
    f3 cp = p - c;
    float d5 = dotf(ab, cp), d6 = dotf(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float w = d2 / (d2 - d6);
        return a + w * ac;
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return b + w * (c - b);
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom;
    float w = vc * denom;
    return a + v * ab + w * ac;
}

constexpr int kMaxBodiesF = 8;
constexpr unsigned kPolyThreadsF = 128;

// particle_polygonObject_collision_kernel<1>(float) (impl:1806-1895): the
// particle takes each contact's normal force (and the zero moment of DHS
// with ir = 0) added in contact order; the body's reaction -(Fn + Ft) and its
// moment go to per-block partials in a fixed order.
__global__ void __launch_bounds__(kPolyThreadsF) k_polygon_f(ParamsF P, const xd_polygon_info_f* __restrict__ dpi,
                                                             const xd_polygon_mass_info_f* dpmi,
                                                             const float4* __restrict__ pos,
                                                             const float* __restrict__ vel,
                                                             const float* __restrict__ omega,
                                                             float* __restrict__ force, float* __restrict__ moment,
                                                             const float* __restrict__ mass,
                                                             const unsigned* __restrict__ sorted,
                                                             const unsigned* __restrict__ cstart,
                                                             const unsigned* __restrict__ cend,
                                                             const xd_contact_property_f* __restrict__ cps,
                                                             unsigned np, unsigned nbodies,
                                                             float* __restrict__ partials,
                                                             xd_polygon_mass_info_f* react_atomic)
{
    float react[kMaxBodiesF][6];
#pragma unroll
    for (int b = 0; b < kMaxBodiesF; ++b)
#pragma unroll
        for (int q = 0; q < 6; ++q) react[b][q] = 0.0f;
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < np) {
        float im = mass[id];
        float4 ip4 = pos[id];
        f3 ipos = mkf(ip4.x, ip4.y, ip4.z);
        f3 ivel = ldf3(vel, id), iomega = ldf3(omega, id);
        int3 gp = grid_pos_f(P, ipos.x, ipos.y, ipos.z);
        float ir = ip4.w;
        f3 M = mkf(0, 0, 0), Fn = mkf(0, 0, 0), Ft = mkf(0, 0, 0);
        f3 fo = ldf3(force, id), mo = ldf3(moment, id);
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    unsigned h = grid_hash_f(P, gp.x + x, gp.y + y, gp.z + z);
                    unsigned st = cstart[h];
                    if (st == 0xffffffffu) continue;
                    unsigned en = cend[h];
                    for (unsigned j = st; j < en; j++) {
                        unsigned k = sorted[j];
                        if (k < np) continue;
                        k -= np;
                        const xd_polygon_info_f tri = dpi[k];
                        unsigned pidx = (unsigned)tri.id;
                        const xd_polygon_mass_info_f& pmi = dpmi[pidx];
                        f3 Pv = arr3(tri.P), Qv = arr3(tri.Q), Rv = arr3(tri.R);
                        f3 cpt = closest_pt_f(Pv, Qv, Rv, ipos);
                        f3 po2cp = cpt - arr3(pmi.origin);
                        f3 distVec = ipos - cpt;
                        float dist = lenf(distVec);
                        float cdist = ir - dist;
                        Fn = mkf(0.0f, 0.0f, 0.0f);
                        if (cdist > 0) {
                            f3 qp = Qv - Pv, rp = Rv - Pv;
                            f3 unit = -crossf(qp, rp);
                            unit = unit / lenf(unit);
                            f3 dv = arr3(pmi.vel) + crossf(arr3(pmi.omega), po2cp) - (ivel + crossf(iomega, ir * unit));
                            const xd_contact_property_f cmp = cps[pidx];
                            FcF c = get_constant_f(ir, 0, im, 0, cmp);
                            dhs_f(c, 0, 0, 0, 0, 0, 0, 0, cdist, dv, unit, P.dt, Ft, Fn, M);
                            fo += Fn;
                            mo += M;
                            f3 tot = Fn + Ft;
                            f3 rf = -tot;
                            f3 rm = -crossf(po2cp, tot);
                            if (react_atomic) {
                                // body count unknown to the caller: add as the contact is found
                                atomicAdd(react_atomic[pidx].force + 0, rf.x);
                                atomicAdd(react_atomic[pidx].force + 1, rf.y);
                                atomicAdd(react_atomic[pidx].force + 2, rf.z);
                                atomicAdd(react_atomic[pidx].moment + 0, rm.x);
                                atomicAdd(react_atomic[pidx].moment + 1, rm.y);
                                atomicAdd(react_atomic[pidx].moment + 2, rm.z);
                                continue;
                            }
#pragma unroll
                            for (int b = 0; b < kMaxBodiesF; ++b)
                                if ((unsigned)b == pidx) {
                                    react[b][0] += rf.x; react[b][1] += rf.y; react[b][2] += rf.z;
                                    react[b][3] += rm.x; react[b][4] += rm.y; react[b][5] += rm.z;
                                }
                        }
                    }
                }
        stf3(force, id, fo);
        stf3(moment, id, mo);
    }
    // fixed-order block reduction of the per-thread reactions
    __shared__ float red[kPolyThreadsF];
    for (unsigned b = 0; b < nbodies; ++b)
        for (int q = 0; q < 6; ++q) {
            float v = 0.0f;
#pragma unroll
            for (int bb = 0; bb < kMaxBodiesF; ++bb)
                if ((unsigned)bb == b) v = react[bb][q];
            red[threadIdx.x] = v;
            __syncthreads();
            for (unsigned o = kPolyThreadsF / 2; o > 0; o >>= 1) {
                if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
                __syncthreads();
            }
            if (threadIdx.x == 0) partials[((size_t)blockIdx.x * nbodies + b) * 6 + q] = red[0];
            __syncthreads();
        }
}

__global__ void k_polygon_reaction_f(const float* __restrict__ partials, unsigned nblocks, unsigned nbodies,
                                     xd_polygon_mass_info_f* __restrict__ dpmi)
{
    unsigned t = threadIdx.x;   // one thread per (body, component)
    if (t >= nbodies * 6) return;
    unsigned b = t / 6, q = t % 6;
    float s = 0.0f;
    for (unsigned blk = 0; blk < nblocks; ++blk) s += partials[((size_t)blk * nbodies + b) * 6 + q];
    if (q < 3) dpmi[b].force[q] += s;
    else dpmi[b].moment[q - 3] += s;
}

// ------------------------------------------------------------ reductionD3(float3)

constexpr unsigned kRedThreadsF = 256;

__global__ void __launch_bounds__(kRedThreadsF) k_reduce_f3_partial(const float* __restrict__ in, unsigned n,
                                                                    float* __restrict__ partial)
{
    __shared__ float s[3][kRedThreadsF];
    float a[3] = { 0.f, 0.f, 0.f };
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) a[c] += in[3 * (size_t)i + c];
    for (int c = 0; c < 3; ++c) s[c][threadIdx.x] = a[c];
    __syncthreads();
    for (unsigned o = kRedThreadsF / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 3; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 3) partial[3 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_reduce_f3_final(const float* __restrict__ partial, unsigned nb, float* __restrict__ out)
{
    unsigned c = threadIdx.x;
    if (c >= 3) return;
    float t = 0.f;
    for (unsigned b = 0; b < nb; ++b) t += partial[3 * b + c];
    out[c] = t;
}

// ------------------------------------------------------------ host helpers

bool params_f(ParamsF* out)
{
    std::lock_guard<std::mutex> lk(g_f_mu);
    if (!g_have_f) return false;
    const xd_device_parameters_f& h = g_f;
    ParamsF p;
    p.np = h.np;
    p.nsphere = h.nsphere;
    p.ncell = h.ncell;
    p.gsx = h.grid_size[0];
    p.gsy = h.grid_size[1];
    p.gsz = h.grid_size[2];
    p.dt = h.dt;
    p.half2dt = h.half2dt;
    p.cs = h.cell_size;
    p.cohesion = h.cohesion;
    for (int a = 0; a < 3; ++a) {
        p.g[a] = h.gravity[a];
        p.wo[a] = h.world_origin[a];
    }
    const Params* d = params();
    p.hx = d ? d->gx : 0u;
    p.hy = d ? d->gy : 0u;
    p.hz = d ? d->gz : 0u;
    *out = p;
    return true;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

}  // namespace
}  // namespace xd

using namespace xd;

#define XD_REQUIRE_F(cond, ...)                                     \
    do {                                                            \
        if (!(cond)) return set_error(XD_ERR_INVALID, __VA_ARGS__); \
    } while (0)

#define XD_NEED_PARAMS_F(name)                                                                   \
    ParamsF PF;                                                                                  \
    if (!params_f(&PF))                                                                          \
        return set_error(XD_ERR_STATE, "%s: xd_set_symbolic_parameter_f was not called", name)

extern "C" {

int xd_set_symbolic_parameter_f(const xd_device_parameters_f* h)
{
    XD_REQUIRE_F(h, "set_symbolic_parameter_f: null parameters");
    XD_REQUIRE_F(h->cell_size > 0.0f, "set_symbolic_parameter_f: cell_size must be > 0");
    std::lock_guard<std::mutex> lk(g_f_mu);
    g_f = *h;
    g_have_f = true;
    return XD_OK;
}

int xd_vv_update_position_f(float* pos, const float* vel, const float* acc, unsigned np, void* s)
{
    XD_NEED_PARAMS_F("vv_update_position_f");
    if (np == 0) return XD_OK;
    XD_REQUIRE_F(pos && vel && acc, "vv_update_position_f: null pointer");
    XD_REQUIRE_F(aligned16(pos), "vv_update_position_f: pos must be 16-byte aligned");
    k_vv_position_f<<<div_up(np, 256), 256, 0, S(s)>>>(PF, reinterpret_cast<float4*>(pos), vel, acc, np);
    return launch_status("vv_update_position_f");
}

int xd_vv_update_velocity_f(float* vel, float* acc, float* omega, float* alpha, float* force, float* moment,
                            const float* mass, const float* inertia, unsigned np, void* s)
{
    XD_NEED_PARAMS_F("vv_update_velocity_f");
    if (np == 0) return XD_OK;
    XD_REQUIRE_F(vel && acc && omega && alpha && force && moment && mass && inertia,
                 "vv_update_velocity_f: null pointer");
    k_vv_velocity_f<<<div_up(np, 256), 256, 0, S(s)>>>(PF, vel, acc, omega, alpha, force, moment, mass, inertia,
                                                        np);
    return launch_status("vv_update_velocity_f");
}

int xd_calculate_hash_and_index_f(unsigned* hash, unsigned* index, const float* pos, unsigned np, void* s)
{
    XD_NEED_PARAMS_F("calculate_hash_and_index_f");
    if (np == 0) return XD_OK;
    XD_REQUIRE_F(hash && index && pos, "calculate_hash_and_index_f: null pointer");
    XD_REQUIRE_F(aligned16(pos), "calculate_hash_and_index_f: pos must be 16-byte aligned");
    k_hash_f<<<div_up(np, 256), 256, 0, S(s)>>>(PF, hash, index, reinterpret_cast<const float4*>(pos), np, 0);
    return launch_status("calculate_hash_and_index_f");
}

int xd_calculate_hash_and_index_polysphere_f(unsigned* hash, unsigned* index, unsigned sid, unsigned nsphere,
                                             const float* sphere, void* s)
{
    XD_NEED_PARAMS_F("calculate_hash_and_index_polysphere_f");
    if (nsphere == 0) return XD_OK;
    XD_REQUIRE_F(hash && index && sphere, "calculate_hash_and_index_polysphere_f: null pointer");
    XD_REQUIRE_F(aligned16(sphere), "calculate_hash_and_index_polysphere_f: sphere must be 16-byte aligned");
    k_hash_f<<<div_up(nsphere, 256), 256, 0, S(s)>>>(PF, hash, index, reinterpret_cast<const float4*>(sphere),
                                                      nsphere, sid);
    return launch_status("calculate_hash_and_index_polysphere_f");
}

int xd_reorder_and_find_cell_start_f(unsigned* hash, unsigned* index, unsigned* cstart, unsigned* cend,
                                     unsigned* sorted_index, unsigned n, unsigned ncell, void* s)
{
    return xd_reorder_and_find_cell_start(hash, index, cstart, cend, sorted_index, n, ncell, s);
}

int xd_calculate_p2p_f(int tcm, const float* pos, const float* vel, const float* omega, float* force,
                       float* moment, const float* mass, const unsigned* sorted_index, const unsigned* cstart,
                       const unsigned* cend, const xd_contact_property_f* cp, unsigned np, void* s)
{
    XD_NEED_PARAMS_F("calculate_p2p_f");
    XD_REQUIRE_F(tcm == 1, "calculate_p2p_f: only tcm = 1 (DHS) is provided");
    if (np == 0) return XD_OK;
    XD_REQUIRE_F(pos && vel && omega && force && moment && mass && sorted_index && cstart && cend && cp,
                 "calculate_p2p_f: null pointer");
    XD_REQUIRE_F(aligned16(pos), "calculate_p2p_f: pos must be 16-byte aligned");
    k_p2p_f<<<div_up(np, 128), 128, 0, S(s)>>>(PF, reinterpret_cast<const float4*>(pos), vel, omega, force, moment,
                                                mass, sorted_index, cstart, cend, cp, np);
    return launch_status("calculate_p2p_f");
}

static int planes_f(const char* name, int tcm, const xd_plane_info_f* planes, unsigned nplanes, const float* pos,
                    const float* vel, const float* omega, float* force, float* moment, const float* mass,
                    unsigned np, const xd_contact_property_f* cp, void* s)
{
    XD_NEED_PARAMS_F(name);
    XD_REQUIRE_F(tcm == 1, "%s: only tcm = 1 (DHS) is provided", name);
    if (np == 0) return XD_OK;
    XD_REQUIRE_F(planes && pos && vel && omega && force && moment && mass && cp, "%s: null pointer", name);
    XD_REQUIRE_F(aligned16(pos), "%s: pos must be 16-byte aligned", name);
    k_planes_f<<<div_up(np, 128), 128, 0, S(s)>>>(PF, planes, nplanes, reinterpret_cast<const float4*>(pos), vel,
                                                   omega, force, moment, cp, mass, np);
    return launch_status(name);
}

int xd_plane_contact_force_f(int tcm, const xd_plane_info_f* plane, const float* pos, const float* vel,
                             const float* omega, float* force, float* moment, const float* mass, unsigned np,
                             const xd_contact_property_f* cp, void* s)
{
    return planes_f("plane_contact_force_f", tcm, plane, 1, pos, vel, omega, force, moment, mass, np, cp, s);
}

int xd_cube_contact_force_f(int tcm, const xd_plane_info_f* planes6, const float* pos, const float* vel,
                            const float* omega, float* force, float* moment, const float* mass, unsigned np,
                            const xd_contact_property_f* cp, void* s)
{
    return planes_f("cube_contact_force_f", tcm, planes6, 6, pos, vel, omega, force, moment, mass, np, cp, s);
}

int xd_particle_polygon_collision_f(int tcm, const xd_polygon_info_f* dpi, const float* dsph,
                                    xd_polygon_mass_info_f* dpmi, const float* pos, const float* vel,
                                    const float* omega, float* force, float* moment, const float* mass,
                                    const unsigned* sidx, const unsigned* cstart, const unsigned* cend,
                                    const xd_contact_property_f* cp, unsigned np, unsigned nbodies, void* s)
{
    (void)dsph;   // the reference kernel takes the spheres but reads P, Q, R only
    XD_NEED_PARAMS_F("particle_polygon_collision_f");
    XD_REQUIRE_F(tcm == 1, "particle_polygon_collision_f: only tcm = 1 (DHS) is provided");
    if (np == 0) return XD_OK;
    XD_REQUIRE_F(nbodies <= (unsigned)kMaxBodiesF, "particle_polygon_collision_f: at most %d bodies",
                 kMaxBodiesF);
    XD_REQUIRE_F(dpi && dpmi && pos && vel && omega && force && moment && mass && sidx && cstart && cend && cp,
                 "particle_polygon_collision_f: null pointer");
    XD_REQUIRE_F(aligned16(pos), "particle_polygon_collision_f: pos must be 16-byte aligned");
    const unsigned nb = div_up(np, kPolyThreadsF);
    int st = XD_OK;
    if (nbodies == 0) {
        // nbodies = 0: the reactions are added with atomics (order not fixed)
        k_polygon_f<<<nb, kPolyThreadsF, 0, S(s)>>>(PF, dpi, dpmi, reinterpret_cast<const float4*>(pos), vel,
                                                     omega, force, moment, mass, sidx, cstart, cend, cp, np, 0,
                                                     nullptr, dpmi);
        return launch_status("particle_polygon_collision_f");
    }
    void* ws = workspace(sizeof(float) * 6 * (size_t)nbodies * nb, &st);
    if (!ws) return st;
    float* part = static_cast<float*>(ws);
    k_polygon_f<<<nb, kPolyThreadsF, 0, S(s)>>>(PF, dpi, dpmi, reinterpret_cast<const float4*>(pos), vel, omega,
                                                 force, moment, mass, sidx, cstart, cend, cp, np, nbodies, part,
                                                 nullptr);
    st = launch_status("particle_polygon_collision_f");
    if (st != XD_OK) return st;
    k_polygon_reaction_f<<<1, 64, 0, S(s)>>>(part, nb, nbodies, dpmi);
    return launch_status("particle_polygon_collision_f (reaction)");
}

int xd_reduction_f3(const float* in, unsigned n, float out[3], void* s)
{
    XD_REQUIRE_F(out, "reduction_f3: null output");
    out[0] = out[1] = out[2] = 0.0f;
    if (n == 0) return XD_OK;
    XD_REQUIRE_F(in, "reduction_f3: null input");
    const unsigned nb = std::min(1024u, div_up(n, kRedThreadsF));
    int st = XD_OK;
    void* ws = workspace(sizeof(float) * (3 * (size_t)nb + 4), &st);
    if (!ws) return st;
    float* part = static_cast<float*>(ws);
    float* dout = part + 3 * (size_t)nb;
    k_reduce_f3_partial<<<nb, kRedThreadsF, 0, S(s)>>>(in, n, part);
    k_reduce_f3_final<<<1, 32, 0, S(s)>>>(part, nb, dout);
    st = launch_status("reduction_f3");
    if (st != XD_OK) return st;
    cudaError_t e = cudaMemcpyAsync(out, dout, sizeof(float) * 3, cudaMemcpyDeviceToHost, S(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(S(s));
    return cuda_status(e, "reduction_f3");
}

}  // extern "C"
