// The legacy DEM interface of the reference (include/cu_dem_dec.cuh,
// launchers source/cu_dem_def.cu, kernels include/cu_dem_impl.cuh), restated
// for the parSIM classes that call it.  See include/xdem_legacy.h for the
// layouts and the reference behaviour kept on purpose.
//
// Compiled with --fmad=false.  The vector helpers follow cu_dem_impl.cuh:10-72
// (component-wise, left to right; vector / scalar multiplies by the
// reciprocal), so each expression is evaluated as the reference writes it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/xdem_legacy.h"
#include "xd_grid.cuh"
#include "xd_internal.cuh"

static_assert(sizeof(xd_legacy_parameters) == 144, "legacy device_parameters layout");
static_assert(sizeof(xd_legacy_plane_info) == 160, "legacy device_plane_info layout");
static_assert(sizeof(xd_legacy_polygon) == 144, "cu_polygon layout");
static_assert(sizeof(xd_legacy_mass_info) == 48, "cu_mass_info layout");

namespace xd {
namespace {

std::mutex g_l_mu;
bool g_have_l = false;
xd_legacy_parameters g_l;

struct LP {
    unsigned np, nsp, ncell, gx, gy, gz;
    double dt, half2dt, cs;
    double g[3], wo[3];
    double kn, vn, ks, vs, mu, coh;
};

struct v3 {
    double x, y, z;
};
__device__ __forceinline__ v3 V(double x, double y, double z) { return v3{ x, y, z }; }
__device__ __forceinline__ v3 operator*(double a, v3 b) { return V(a * b.x, a * b.y, a * b.z); }
__device__ __forceinline__ void operator+=(v3& a, v3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__device__ __forceinline__ v3 operator+(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 operator-(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 operator-(v3 a) { return V(-a.x, -a.y, -a.z); }
__device__ __forceinline__ double len(v3 v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b)
{
    return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ v3 operator/(v3 a, double b)
{
    double inv = 1 / b;
    return V(a.x * inv, a.y * inv, a.z * inv);
}
__device__ __forceinline__ v3 ld4(const double* a, size_t i) { return V(a[4 * i], a[4 * i + 1], a[4 * i + 2]); }
__device__ __forceinline__ v3 ld3(const double* a, size_t i) { return V(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
__device__ __forceinline__ v3 ldv(const double* a) { return V(a[0], a[1], a[2]); }
__device__ __forceinline__ void add3(double* a, size_t i, v3 b)
{
    a[3 * i] += b.x;
    a[3 * i + 1] += b.y;
    a[3 * i + 2] += b.z;
}

// calcGridPos / calcGridHash (impl:73-91)
__device__ __forceinline__ unsigned cell_hash(const LP& P, v3 p, int dx, int dy, int dz)
{
    int cx = (int)floor((p.x - P.wo[0]) / P.cs) + dx;
    int cy = (int)floor((p.y - P.wo[1]) / P.cs) + dy;
    int cz = (int)floor((p.z - P.wo[2]) / P.cs) + dz;
    unsigned x = (unsigned)cx & (P.gx - 1u), y = (unsigned)cy & (P.gy - 1u), z = (unsigned)cz & (P.gz - 1u);
    return __umul24(__umul24(z, P.gy), P.gx) + __umul24(y, P.gx) + x;
}

// ------------------------------------------------------------ integrator

__global__ void k_l_vv_position(LP P, double* __restrict__ pos, const double* __restrict__ vel,
                                const double* __restrict__ acc)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= P.np) return;
    v3 p = ld4(pos, id);
    v3 v = ld4(vel, id), a = ld4(acc, id);
    p += P.dt * v + P.half2dt * a;
    pos[4 * (size_t)id] = p.x;
    pos[4 * (size_t)id + 1] = p.y;
    pos[4 * (size_t)id + 2] = p.z;
}

__global__ void k_l_vv_velocity(LP P, double* __restrict__ vel, double* __restrict__ acc, double* __restrict__ omega,
                                double* __restrict__ alpha, const double* __restrict__ force,
                                const double* __restrict__ moment)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= P.np) return;
    const size_t q = 4 * (size_t)id;
    v3 v = ld4(vel, id), a = ld4(acc, id), av = ld4(omega, id), aa = ld4(alpha, id);
    double mass = acc[q + 3], inertia = alpha[q + 3];
    v += 0.5 * P.dt * a;
    av += 0.5 * P.dt * aa;
    a = (1 / mass) * ld3(force, id);
    aa = (1 / inertia) * ld3(moment, id);
    v += 0.5 * P.dt * a;
    av += 0.5 * P.dt * aa;
    vel[q] = v.x; vel[q + 1] = v.y; vel[q + 2] = v.z; vel[q + 3] = 0;
    omega[q] = av.x; omega[q + 1] = av.y; omega[q + 2] = av.z; omega[q + 3] = 0;
    acc[q] = a.x; acc[q + 1] = a.y; acc[q + 2] = a.z; acc[q + 3] = mass;
    alpha[q] = aa.x; alpha[q + 1] = aa.y; alpha[q + 2] = aa.z; alpha[q + 3] = inertia;
}

// ------------------------------------------------------------ grid

__global__ void k_l_hash(LP P, unsigned* __restrict__ hash, unsigned* __restrict__ index,
                         const double* __restrict__ pos)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= P.np + P.nsp) return;
    hash[id] = cell_hash(P, ld4(pos, id), 0, 0, 0);
    index[id] = id;
}

// reorderDataAndFindCellStart_kernel (impl:156-196) over np + nsp entries;
// the neighbour in the sorted list is read directly instead of through
// shared memory (same values)
__global__ void k_l_cell_bounds(LP P, const unsigned* __restrict__ hash, const unsigned* __restrict__ index,
                                unsigned* __restrict__ cstart, unsigned* __restrict__ cend,
                                unsigned* __restrict__ sorted_index)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned tnp = P.np + P.nsp;
    if (id >= tnp) return;
    const unsigned h = hash[id];
    if (id == 0 || h != hash[id - 1]) {
        cstart[h] = id;
        if (id > 0) cend[hash[id - 1]] = id;
    }
    if (id == tnp - 1) cend[h] = id + 1;
    sorted_index[id] = index[id];
}

// ------------------------------------------------------------ particle-particle

// calForce (impl:198-252)
__device__ __forceinline__ bool cal_force(const LP& P, double ir, double jr, v3 ipos, v3 jpos, v3 ivel, v3 jvel,
                                          v3 iomega, v3 jomega, v3& force, v3& moment)
{
    v3 relative_pos = jpos - ipos;
    double dist = len(relative_pos);
    double collid_dist = (ir + jr) - dist;
    if (collid_dist <= 0) {
        if (P.coh == 0) return false;
        double tu = P.coh / P.mu;
        v3 unit = relative_pos / dist;
        v3 relative_vel = jvel + cross(jomega, -jr * unit) - (ivel + cross(iomega, ir * unit));
        double Fn = (-P.kn * pow(-collid_dist, 1.5) + P.vn * dot(relative_vel, unit));
        if (Fn < 0 && Fn > -tu) force += tu * unit;
        v3 e = relative_vel - dot(relative_vel, unit) * unit;
        double mag_e = len(e);
        if (mag_e) {
            v3 s_hat = e / mag_e;
            double ds = mag_e * P.dt;
            double Fs = fmin(P.ks * ds + P.vs * (dot(relative_vel, s_hat)), P.mu * Fn);
            if (Fs < Fn * P.mu + P.coh) moment += cross(ir * unit, (Fn * P.mu + P.coh) * s_hat);
        }
        return false;
    }
    v3 unit = relative_pos / dist;
    v3 relative_vel = jvel + cross(jomega, -jr * unit) - (ivel + cross(iomega, ir * unit));
    v3 single_force = (-P.kn * pow(collid_dist, 1.5) + P.vn * dot(relative_vel, unit)) * unit;
    v3 single_moment = V(0, 0, 0);
    v3 e = relative_vel - dot(relative_vel, unit) * unit;
    double mag_e = len(e);
    if (mag_e) {
        v3 s_hat = e / mag_e;
        double ds = mag_e * P.dt;
        v3 shear_force = fmin(P.ks * ds + P.vs * (dot(relative_vel, s_hat)), P.mu * len(single_force)) * s_hat;
        single_moment = cross(ir * unit, shear_force);
    }
    force += single_force;
    moment += single_moment;
    return true;
}

__global__ void __launch_bounds__(128) k_l_p2p(LP P, const double* __restrict__ pos, const double* __restrict__ vel,
                                               const double* __restrict__ acc, const double* __restrict__ omega,
                                               double* __restrict__ force, double* __restrict__ moment,
                                               const unsigned* __restrict__ sorted, const unsigned* __restrict__ cstart,
                                               const unsigned* __restrict__ cend)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= P.np) return;
    v3 ipos = ld4(pos, id), ivel = ld4(vel, id), iomega = ld4(omega, id);
    double ir = pos[4 * (size_t)id + 3];
    v3 m_force = acc[4 * (size_t)id + 3] * V(P.g[0], P.g[1], P.g[2]);
    v3 m_moment = V(0, 0, 0);
    for (int z = -1; z <= 1; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                unsigned h = cell_hash(P, ipos, x, y, z);
                unsigned st = cstart[h];
                if (st == 0xffffffffu) continue;
                unsigned en = cend[h];
                for (unsigned j = st; j < en; j++) {
                    unsigned k = sorted[j];
                    if (id == k || k >= P.np) continue;
                    cal_force(P, ir, pos[4 * (size_t)k + 3], ipos, ld4(pos, k), ivel, ld4(vel, k), iomega,
                              ld4(omega, k), m_force, m_moment);
                }
            }
    add3(force, id, m_force);
    add3(moment, id, m_moment);
}

// ------------------------------------------------------------ cube

__global__ void __launch_bounds__(128) k_l_cube(LP P, const xd_legacy_plane_info* __restrict__ planes, double kn,
                                                double vn, double ks, double vs, double mu,
                                                const double* __restrict__ pos, const double* __restrict__ vel,
                                                const double* __restrict__ omega, double* __restrict__ force,
                                                double* __restrict__ moment)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= P.np) return;
    double r = pos[4 * (size_t)id + 3];
    v3 ipos = ld4(pos, id), ivel = ld4(vel, id), iomega = ld4(omega, id);
    v3 m_force = V(0, 0, 0), m_moment = V(0, 0, 0);
    for (int i = 0; i < 6; i++) {
        const xd_legacy_plane_info& pl = planes[i];
        v3 xw = ldv(pl.xw), uw = ldv(pl.uw);
        v3 dp = ipos - xw;
        v3 wp = V(dot(dp, ldv(pl.u1)), dot(dp, ldv(pl.u2)), dot(dp, uw));
        if (fabs(wp.z) < r && (wp.x > 0 && wp.x < pl.l1) && (wp.y > 0 && wp.y < pl.l2)) {
            const int sg = dot(ipos - xw, uw) < 0 ? -1 : 1;
            v3 unit = (double)(-sg) * (uw / len(uw));
            double collid_dist = r - fabs(dot(ipos - xw, unit));
            v3 dv = -(ivel + cross(iomega, r * unit));
            v3 single_force = (-kn * pow(collid_dist, 1.5) + vn * dot(dv, unit)) * unit;
            v3 e = dv - dot(dv, unit) * unit;
            double mag_e = len(e);
            if (mag_e) {
                v3 s_hat = e / mag_e;
                double ds = mag_e * P.dt;
                v3 shear_force = fmin(ks * ds + vs * dot(dv, s_hat), mu * len(single_force)) * s_hat;
                m_moment += cross(r * unit, shear_force);
            }
            m_force += single_force;
        }
    }
    add3(force, id, m_force);
    add3(moment, id, m_moment);
}

// ------------------------------------------------------------ shapes

// ClosestPtPointTriangle with the region code wc: 0 vertex, 1 edge, 2 face (impl:380-441)
__device__ __forceinline__ v3 closest_wc(v3 p, v3 a, v3 b, v3 c, int& wc)
{
    v3 ab = b - a, ac = c - a, ap = p - a;
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) { wc = 0; return a; }
    v3 bp = p - b;
    double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) { wc = 0; return b; }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        wc = 1;
        double v = d1 / (d1 - d3);
        return a + v * ab;
    }
    v3 cp = p - c;
    double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) { wc = 0; return c; }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        wc = 1;
        double w = d2 / (d2 - d6);
        return a + w * ac;
    }
    double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        wc = 1;
        double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return b + w * (c - b);
    }
    wc = 2;
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom, w = vc * denom;
    return a + v * ab + w * ac;
}

// isIntersect2Lines (impl:443-452)
__device__ __forceinline__ bool intersect2(double x1, double x2, double x3, double x4, double y1, double y2,
                                           double y3, double y4)
{
    double div = (y4 - y3) * (x2 - x1) - (x4 - x3) * (y2 - y1);
    double t = ((x4 - x3) * (y1 - y3) - (y4 - y3) * (x1 - x3)) / div;
    double s = ((x2 - x1) * (y1 - y3) - (y2 - y1) * (x1 - x3)) / div;
    return (t >= 0 && t <= 1) || (s >= 0 && s <= 1);
}

struct Shape {
    const xd_legacy_mass_info* mi;
    const xd_legacy_polygon* polygons;
    const unsigned* id_set;
    const unsigned* poly_start;
    const unsigned* poly_end;
    double kn, vn, ks, vs, mu;
};

__device__ __forceinline__ v3 shape_force(const LP& P, const Shape& S, double r, double collid_dist, v3 unit, v3 vel,
                                          v3 omega, v3& moment_out)
{
    v3 dv = ldv(S.mi->vel) - (vel + cross(omega, r * unit));
    v3 single_force = (-S.kn * pow(collid_dist, 1.5) + S.vn * dot(dv, unit)) * unit;
    v3 e = dv - dot(dv, unit) * unit;
    double mag_e = len(e);
    if (mag_e) {
        v3 s_hat = e / mag_e;
        double ds = mag_e * P.dt;
        v3 shear_force = fmin(S.ks * ds + S.vs * dot(dv, s_hat), S.mu * len(single_force)) * s_hat;
        moment_out = cross(r * unit, shear_force);
    }
    return single_force;
}

// shpae_hertzian_contact_force_kernel with calculateTriangleParticleContactForce
// (impl:454-526, 676-762): the first face contact through the polygons of
// the vertices in the 27 cells
__global__ void __launch_bounds__(128) k_l_shape_face(LP P, Shape S, bool* __restrict__ isLineContact,
                                                      const double* __restrict__ pos, const double* __restrict__ vel,
                                                      const double* __restrict__ omega, double* __restrict__ force,
                                                      double* __restrict__ moment, const unsigned* __restrict__ sorted,
                                                      const unsigned* __restrict__ cstart,
                                                      const unsigned* __restrict__ cend)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= P.np) return;
    isLineContact[id] = false;
    v3 ipos = ld4(pos, id), ivel = ld4(vel, id), iomega = ld4(omega, id);
    double ir = pos[4 * (size_t)id + 3];
    int count = 0;
    v3 plane_normal = V(0, 0, 0), plane_cp = V(0, 0, 0);   // the last face contact (at most one is kept)
    v3 m_force = V(0, 0, 0), m_moment = V(0, 0, 0);
    for (int z = -1; z <= 1; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                unsigned h = cell_hash(P, ipos, x, y, z);
                unsigned st = cstart[h];
                if (st == 0xffffffffu) continue;
                unsigned en = cend[h];
                for (unsigned j = st; j < en; j++) {
                    unsigned k = sorted[j];
                    if (id == k || k < P.np) continue;
                    const unsigned vtx = k - P.np;
                    for (unsigned q = S.poly_start[vtx]; q < S.poly_end[vtx]; q++) {
                        const xd_legacy_polygon& po = S.polygons[S.id_set[q]];
                        int wc = -1;
                        v3 contact_point = closest_wc(ipos, ldv(po.P), ldv(po.Q), ldv(po.R), wc);
                        v3 sp = ipos - contact_point;
                        double dist = len(sp);
                        v3 p_unit = -ldv(po.N) / len(ldv(po.N));
                        double collid_dist = ir - dist;
                        if (collid_dist <= 0) continue;
                        if (wc != 2) continue;
                        if (count) {
                            v3 ep1 = plane_cp + 10000 * plane_normal;
                            v3 ep2 = contact_point + 10000 * p_unit;
                            if (!intersect2(plane_cp.x, ep1.x, contact_point.x, ep2.x, plane_cp.y, ep1.y,
                                            contact_point.y, ep2.y))
                                continue;
                        }
                        m_force += shape_force(P, S, ir, collid_dist, p_unit, ivel, iomega, m_moment);
                        plane_cp = contact_point;
                        plane_normal = p_unit;
                        ++count;
                        add3(force, id, m_force);
                        add3(moment, id, m_moment);
                        isLineContact[id] = true;
                        return;
                    }
                }
            }
}

// shape_line_or_edge_contact_force_kernel with
// calculateTriangleLineOrEdgeParticleContactForce (impl:528-674): particles
// without a face contact take their first edge or vertex contact
__global__ void __launch_bounds__(128) k_l_shape_edge(LP P, Shape S, bool* __restrict__ isLineContact,
                                                      const double* __restrict__ pos, const double* __restrict__ vel,
                                                      const double* __restrict__ omega, double* __restrict__ force,
                                                      double* __restrict__ moment, const unsigned* __restrict__ sorted,
                                                      const unsigned* __restrict__ cstart,
                                                      const unsigned* __restrict__ cend)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= P.np) return;
    if (isLineContact[id]) return;
    v3 ipos = ld4(pos, id), ivel = ld4(vel, id), iomega = ld4(omega, id);
    double ir = pos[4 * (size_t)id + 3];
    v3 l_moment = V(0, 0, 0);
    for (int z = -1; z <= 1; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                unsigned h = cell_hash(P, ipos, x, y, z);
                unsigned st = cstart[h];
                if (st == 0xffffffffu) continue;
                unsigned en = cend[h];
                for (unsigned j = st; j < en; j++) {
                    unsigned k = sorted[j];
                    if (id == k || k < P.np) continue;
                    const unsigned vtx = k - P.np;
                    for (unsigned q = S.poly_start[vtx]; q < S.poly_end[vtx]; q++) {
                        const xd_legacy_polygon& po = S.polygons[S.id_set[q]];
                        int wc = -1;
                        v3 contact_point = closest_wc(ipos, ldv(po.P), ldv(po.Q), ldv(po.R), wc);
                        v3 sp = ipos - contact_point;
                        double dist = len(sp);
                        v3 s_unit = -sp / dist;
                        double collid_dist = ir - dist;
                        if (collid_dist <= 0) continue;
                        if (wc != 0 && wc != 1) continue;
                        v3 l_force = shape_force(P, S, ir, collid_dist, s_unit, ivel, iomega, l_moment);
                        isLineContact[id] = true;
                        add3(force, id, l_force);
                        add3(moment, id, l_moment);
                        return;
                    }
                }
            }
}

// the shape call's force sum over the particles, in a fixed order
constexpr unsigned kLRed = 256;
__global__ void __launch_bounds__(kLRed) k_l_sum_partial(const double* __restrict__ f, unsigned n,
                                                         double* __restrict__ part)
{
    __shared__ double s[3][kLRed];
    double a[3] = { 0.0, 0.0, 0.0 };
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) a[c] += f[3 * (size_t)i + c];
    for (int c = 0; c < 3; ++c) s[c][threadIdx.x] = a[c];
    __syncthreads();
    for (unsigned o = kLRed / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 3; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 3) part[3 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_l_sum_final(const double* __restrict__ part, unsigned nb, double* __restrict__ out)
{
    unsigned c = threadIdx.x;
    if (c >= 3) return;
    double t = 0.0;
    for (unsigned b = 0; b < nb; ++b) t += part[3 * b + c];
    out[c] = t;
}

// ------------------------------------------------------------ meshes

__global__ void k_l_polygons_position(const double* __restrict__ mpos, const double* __restrict__ A,
                                      const double* __restrict__ lv, unsigned nv, double* __restrict__ pos)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nv) return;
    v3 l = ld3(lv, id);
    double tx = A[0] * l.x + A[1] * l.y + A[2] * l.z;
    double ty = A[3] * l.x + A[4] * l.y + A[5] * l.z;
    double tz = A[6] * l.x + A[7] * l.y + A[8] * l.z;
    pos[3 * (size_t)id] = mpos[0] + tx;
    pos[3 * (size_t)id + 1] = mpos[1] + ty;
    pos[3 * (size_t)id + 2] = mpos[2] + tz;
}

__global__ void k_l_polygons_information(xd_legacy_polygon* __restrict__ polygons, const unsigned* __restrict__ indice,
                                         const double* __restrict__ pos, unsigned ni)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ni) return;
    v3 P = ld3(pos, indice[3 * (size_t)id]), Q = ld3(pos, indice[3 * (size_t)id + 1]),
       R = ld3(pos, indice[3 * (size_t)id + 2]);
    v3 Vv = Q - P, W = R - P, N = cross(Vv, W);
    xd_legacy_polygon& o = polygons[id];
    o.P[0] = P.x; o.P[1] = P.y; o.P[2] = P.z;
    o.Q[0] = Q.x; o.Q[1] = Q.y; o.Q[2] = Q.z;
    o.R[0] = R.x; o.R[1] = R.y; o.R[2] = R.z;
    o.V[0] = Vv.x; o.V[1] = Vv.y; o.V[2] = Vv.z;
    o.W[0] = W.x; o.W[1] = W.y; o.W[2] = W.z;
    o.N[0] = N.x; o.N[1] = N.y; o.N[2] = N.z;
}

__global__ void k_l_mergedata(double* __restrict__ data, const double* __restrict__ pos, unsigned np,
                              const double* __restrict__ vertice, unsigned snp)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np + snp) return;
    double* d = data + 4 * (size_t)id;
    if (id < np) {
        d[0] = pos[4 * (size_t)id];
        d[1] = pos[4 * (size_t)id + 1];
        d[2] = pos[4 * (size_t)id + 2];
        d[3] = pos[4 * (size_t)id + 3];
    } else {
        v3 v = ld3(vertice, id - np);
        d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = -1.0;
    }
}

bool legacy_params(LP* out)
{
    std::lock_guard<std::mutex> lk(g_l_mu);
    if (!g_have_l) return false;
    const xd_legacy_parameters& h = g_l;
    LP p;
    p.np = h.np;
    p.nsp = h.nsp;
    p.ncell = h.ncell;
    p.gx = h.grid_size[0];
    p.gy = h.grid_size[1];
    p.gz = h.grid_size[2];
    p.dt = h.dt;
    p.half2dt = h.half2dt;
    p.cs = h.cell_size;
    for (int a = 0; a < 3; ++a) {
        p.g[a] = h.gravity[a];
        p.wo[a] = h.world_origin[a];
    }
    p.kn = h.kn;
    p.vn = h.vn;
    p.ks = h.ks;
    p.vs = h.vs;
    p.mu = h.mu;
    p.coh = h.cohesive;
    *out = p;
    return true;
}

inline cudaStream_t S_(void* s) { return static_cast<cudaStream_t>(s); }
inline unsigned nblk(unsigned n, unsigned b) { return n ? (n + b - 1) / b : 1u; }

}  // namespace
}  // namespace xd

using namespace xd;

#define XL_REQUIRE(cond, ...)                                       \
    do {                                                            \
        if (!(cond)) return set_error(XD_ERR_INVALID, __VA_ARGS__); \
    } while (0)

#define XL_PARAMS(name)                                                                              \
    LP PL;                                                                                           \
    if (!legacy_params(&PL))                                                                         \
        return set_error(XD_ERR_STATE, "%s: xd_legacy_set_symbolic_parameter was not called", name)

extern "C" {

int xd_legacy_set_symbolic_parameter(const xd_legacy_parameters* h)
{
    XL_REQUIRE(h, "legacy_set_symbolic_parameter: null parameters");
    XL_REQUIRE(h->cell_size > 0.0, "legacy_set_symbolic_parameter: cell_size must be > 0");
    for (int a = 0; a < 3; ++a)
        XL_REQUIRE(h->grid_size[a] && !(h->grid_size[a] & (h->grid_size[a] - 1)),
                   "legacy_set_symbolic_parameter: grid sizes must be powers of two");
    std::lock_guard<std::mutex> lk(g_l_mu);
    g_l = *h;
    g_have_l = true;
    return XD_OK;
}

int xd_legacy_vv_update_position(double* pos, const double* vel, const double* acc, unsigned np, void* s)
{
    (void)np;
    XL_PARAMS("legacy_vv_update_position");
    if (PL.np == 0) return XD_OK;
    XL_REQUIRE(pos && vel && acc, "legacy_vv_update_position: null pointer");
    k_l_vv_position<<<nblk(PL.np, 256), 256, 0, S_(s)>>>(PL, pos, vel, acc);
    return launch_status("legacy_vv_update_position");
}

int xd_legacy_vv_update_velocity(double* vel, double* acc, double* omega, double* alpha, const double* force,
                                 const double* moment, unsigned np, void* s)
{
    (void)np;
    XL_PARAMS("legacy_vv_update_velocity");
    if (PL.np == 0) return XD_OK;
    XL_REQUIRE(vel && acc && omega && alpha && force && moment, "legacy_vv_update_velocity: null pointer");
    k_l_vv_velocity<<<nblk(PL.np, 256), 256, 0, S_(s)>>>(PL, vel, acc, omega, alpha, force, moment);
    return launch_status("legacy_vv_update_velocity");
}

int xd_legacy_calculate_hash_and_index(unsigned* hash, unsigned* index, const double* pos, unsigned np, void* s)
{
    XL_PARAMS("legacy_calculate_hash_and_index");
    XL_REQUIRE(hash && index && pos, "legacy_calculate_hash_and_index: null pointer");
    const unsigned n = PL.np + PL.nsp;
    if (n) k_l_hash<<<nblk(n, 256), 256, 0, S_(s)>>>(PL, hash, index, pos);
    int st = launch_status("legacy_calculate_hash_and_index");
    if (st != XD_OK || np <= 1) return st;
    // the launcher sorts the first np entries (def.cu:65-67), stably by hash
    // wrapped hashes are below gx gy gz
    const unsigned bits = key_bits_for(PL.gx * PL.gy * PL.gz);
    void* ws = workspace(radix_sort_scratch_bytes(np), &st);
    if (!ws) return st;
    unsigned *ok = nullptr, *ov = nullptr;
    st = radix_sort_pairs(hash, index, np, bits, ws, S_(s), &ok, &ov);
    if (st != XD_OK) return st;
    if (ok != hash) {
        cudaError_t e = cudaMemcpyAsync(hash, ok, sizeof(unsigned) * (size_t)np, cudaMemcpyDeviceToDevice, S_(s));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(index, ov, sizeof(unsigned) * (size_t)np, cudaMemcpyDeviceToDevice, S_(s));
        return cuda_status(e, "legacy_calculate_hash_and_index copy-back");
    }
    return XD_OK;
}

int xd_legacy_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart, unsigned* cend,
                                          unsigned* sorted_index, unsigned np, unsigned nc, void* s)
{
    (void)np;
    XL_PARAMS("legacy_reorder_and_find_cell_start");
    XL_REQUIRE(hash && index && cstart && cend && sorted_index, "legacy_reorder_and_find_cell_start: null pointer");
    int st = cuda_status(cudaMemsetAsync(cstart, 0xff, sizeof(unsigned) * (size_t)nc, S_(s)),
                         "legacy_reorder_and_find_cell_start");
    if (st != XD_OK) return st;
    const unsigned n = PL.np + PL.nsp;
    if (n) k_l_cell_bounds<<<nblk(n, 256), 256, 0, S_(s)>>>(PL, hash, index, cstart, cend, sorted_index);
    return launch_status("legacy_reorder_and_find_cell_start");
}

int xd_legacy_calculate_p2p(const double* pos, const double* vel, const double* acc, const double* omega,
                            const double* alpha, double* force, double* moment, const unsigned* sorted_index,
                            const unsigned* cstart, const unsigned* cend, unsigned np, unsigned cRun, void* s)
{
    (void)alpha;
    (void)np;
    (void)cRun;
    XL_PARAMS("legacy_calculate_p2p");
    if (PL.np == 0) return XD_OK;
    XL_REQUIRE(pos && vel && acc && omega && force && moment && sorted_index && cstart && cend,
               "legacy_calculate_p2p: null pointer");
    k_l_p2p<<<nblk(PL.np, 128), 128, 0, S_(s)>>>(PL, pos, vel, acc, omega, force, moment, sorted_index, cstart,
                                                  cend);
    return launch_status("legacy_calculate_p2p");
}

int xd_legacy_cube_hertzian_contact_force(const xd_legacy_plane_info* planes, double kn, double vn, double ks,
                                          double vs, double mu, bool* isLineContact, const double* pos,
                                          const double* vel, const double* omega, double* force, double* moment,
                                          unsigned np, void* s)
{
    (void)isLineContact;
    (void)np;
    XL_PARAMS("legacy_cube_hertzian_contact_force");
    if (PL.np == 0) return XD_OK;
    XL_REQUIRE(planes && pos && vel && omega && force && moment, "legacy_cube_hertzian_contact_force: null pointer");
    k_l_cube<<<nblk(PL.np, 128), 128, 0, S_(s)>>>(PL, planes, kn, vn, ks, vs, mu, pos, vel, omega, force, moment);
    return launch_status("legacy_cube_hertzian_contact_force");
}

int xd_legacy_shape_hertzian_contact_force(const xd_legacy_mass_info* minfo, const xd_legacy_polygon* polygons,
                                           const unsigned* id_set, const unsigned* poly_start,
                                           const unsigned* poly_end, double kn, double vn, double ks, double vs,
                                           double mu, bool* isLineContact, const double* pos, const double* vel,
                                           const double* omega, double* force, double* moment, double* bforce,
                                           unsigned np, const unsigned* sorted_id, const unsigned* cell_start,
                                           const unsigned* cell_end, double out[3], void* s)
{
    (void)bforce;
    XL_REQUIRE(out, "legacy_shape_hertzian_contact_force: null output");
    out[0] = out[1] = out[2] = 0.0;
    XL_PARAMS("legacy_shape_hertzian_contact_force");
    XL_REQUIRE(minfo && polygons && id_set && poly_start && poly_end && isLineContact && pos && vel && omega &&
                   force && moment && sorted_id && cell_start && cell_end,
               "legacy_shape_hertzian_contact_force: null pointer");
    int st = cuda_status(cudaMemsetAsync(force, 0, sizeof(double) * 3 * (size_t)np, S_(s)), "legacy shape");
    if (st == XD_OK) st = cuda_status(cudaMemsetAsync(moment, 0, sizeof(double) * 3 * (size_t)np, S_(s)), "legacy shape");
    if (st != XD_OK) return st;
    Shape S{ minfo, polygons, id_set, poly_start, poly_end, kn, vn, ks, vs, mu };
    if (PL.np) {
        k_l_shape_face<<<nblk(PL.np, 128), 128, 0, S_(s)>>>(PL, S, isLineContact, pos, vel, omega, force, moment,
                                                            sorted_id, cell_start, cell_end);
        k_l_shape_edge<<<nblk(PL.np, 128), 128, 0, S_(s)>>>(PL, S, isLineContact, pos, vel, omega, force, moment,
                                                            sorted_id, cell_start, cell_end);
        st = launch_status("legacy_shape_hertzian_contact_force");
        if (st != XD_OK) return st;
    }
    if (np == 0) return XD_OK;
    const unsigned nb = std::min(1024u, nblk(np, kLRed));
    void* ws = workspace(sizeof(double) * (3 * (size_t)nb + 4), &st);
    if (!ws) return st;
    double* part = static_cast<double*>(ws);
    double* dout = part + 3 * (size_t)nb;
    k_l_sum_partial<<<nb, kLRed, 0, S_(s)>>>(force, np, part);
    k_l_sum_final<<<1, 32, 0, S_(s)>>>(part, nb, dout);
    st = launch_status("legacy_shape_hertzian_contact_force (sum)");
    if (st != XD_OK) return st;
    cudaError_t e = cudaMemcpyAsync(out, dout, sizeof(double) * 3, cudaMemcpyDeviceToHost, S_(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(S_(s));
    return cuda_status(e, "legacy_shape_hertzian_contact_force (sum)");
}

int xd_legacy_update_polygons_position(const double* mpos, const double* A, const double* local_vertice,
                                       unsigned nvertex, double* pos, void* s)
{
    if (nvertex == 0) return XD_OK;
    XL_REQUIRE(mpos && A && local_vertice && pos, "legacy_update_polygons_position: null pointer");
    k_l_polygons_position<<<nblk(nvertex, 256), 256, 0, S_(s)>>>(mpos, A, local_vertice, nvertex, pos);
    return launch_status("legacy_update_polygons_position");
}

int xd_legacy_update_polygons_information(xd_legacy_polygon* polygons, const unsigned* indice, const double* pos,
                                          unsigned ni, void* s)
{
    if (ni == 0) return XD_OK;
    XL_REQUIRE(polygons && indice && pos, "legacy_update_polygons_information: null pointer");
    k_l_polygons_information<<<nblk(ni, 256), 256, 0, S_(s)>>>(polygons, indice, pos, ni);
    return launch_status("legacy_update_polygons_information");
}

int xd_legacy_mergedata(double* data, const double* pos, unsigned np, const double* vertice, unsigned snp,
                        void* s)
{
    if (np + snp == 0) return XD_OK;
    XL_REQUIRE(data && (pos || !np) && (vertice || !snp), "legacy_mergedata: null pointer");
    k_l_mergedata<<<nblk(np + snp, 256), 256, 0, S_(s)>>>(data, pos, np, vertice, snp);
    return launch_status("legacy_mergedata");
}

}  // extern "C"
