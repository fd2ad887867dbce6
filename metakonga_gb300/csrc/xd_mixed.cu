// Mixed-precision scene step: FP64 state and integration, exact integer
// contact decisions, FP32 contact forces.
//
// Per step (same order as dem_simulation::oneStepAnalysis,
// dem_simulation.cpp:447-469):
//   k_mx_integrate  FP64 velocity-Verlet: velocity of step t (from the FP32
//                   contact force + m g) fused with the position of step t+1,
//                   and the particle's cell key in the scene's own grid;
//   radix sort      keys -> permutation (the state is kept in cell order, so
//                   the permutation is close to the identity);
//   k_mx_bounds     cell ranges (only the previous step's cells are cleared);
//   k_mx_reorder    gathers the FP64 state into the new order and builds the
//                   contact view: an FP32 float4 (x, y, z, r) for a cheap
//                   prefilter and int64 fixed-point coordinates (2^-36 m);
//   k_mx_contact    particle-particle forces: FP32 prefilter, then the exact
//                   integer test N = (ri + rj)^2 - |qj - qi|^2 > 0 (no
//                   cancellation), overlap delta = N / (R + |d|) with ~1e-7
//                   relative precision, FP32 Hertz-Mindlin (DHSModel); pairs
//                   within 2e-10 m of touching are decided by the reference's
//                   FP64 expression instead, so pair lists equal the FP64
//                   path's; particles near a wall are appended to a list;
//   k_mx_walls      the listed particles' plane contacts in FP64.
// The grid is the scene's own (not the reference's wrapped 128^3): cell size
// 2 r_max (+0.1 %), padded by one cell on every side, keys clamped inside.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "xd_grid.cuh"
#include "xd_internal.cuh"
#include "xd_mixed.cuh"
#include "xd_physics64.cuh"

namespace xd {

namespace {

constexpr int kMaxPlanes = 16;
constexpr int kFields = 20;   // x y z r vx vy vz wx wy wz ax ay az bx by bz m I 1/m 1/I
enum { FX, FY, FZ, FR, FVX, FVY, FVZ, FWX, FWY, FWZ, FAX, FAY, FAZ, FBX, FBY, FBZ, FM, FI, FIM, FII };
constexpr double kQ = 68719476736.0;          // 2^36 fixed-point units per metre
constexpr float kU = 1.4551915228366852e-11f; // 2^-36 m
constexpr double kGuard = 2e-10;              // metres: FP64 decision inside this band

struct Master {
    double* f[kFields];
    unsigned* id;
};

struct MixParams {
    int gx, gy, gz;
    unsigned n;
    double wo[3];
    double inv_cs;
    float inv_csf;
    double dt, half2dt;
    double g[3];
    float dtf;
    float tol;          // prefilter tolerance (m)
    float c43Eeq, one_b2, sratio, fric;
    double c43Eeq_d, one_b2_d;   // the same constants in FP64 (normal-force recheck)
    long long guard_q;  // guard band in fixed-point units
    int nplanes;
    float pxw[kMaxPlanes][3];   // plane corner relative to the grid origin (FP32)
    float pun[kMaxPlanes][3];   // unit normal (FP32)
    float wall_tol;
};

}  // namespace

struct MixedScene {
    unsigned n = 0, nplanes = 0, ncell = 0;
    int gx = 0, gy = 0, gz = 0;
    double cs = 0.0;
    MixParams P;
    Master m[2];
    int cur = 0;
    // view (sorted order)
    float4* pf = nullptr;
    longlong2* qa = nullptr;
    longlong2* qb = nullptr;
    float4* vf = nullptr;
    float4* vlo = nullptr;   // low parts of the double-float velocity
    float4* wf = nullptr;
    float4* Fc = nullptr;
    float4* Mc = nullptr;
    // grid
    unsigned *keys = nullptr, *vals = nullptr, *prev_keys = nullptr;
    unsigned *cstart = nullptr, *cend = nullptr;
    bool cells_clean = false;      // cstart/cend hold only prev_keys' cells
    void* sort_scratch = nullptr;
    // near-sorted resort buffers
    unsigned *mv_bcount = nullptr, *mv_prefix = nullptr, *mv_key = nullptr, *mv_slot = nullptr;
    unsigned *mv_skey = nullptr, *mv_sslot = nullptr, *mv_sorted = nullptr, *mv_perm = nullptr;
    // walls
    xd_plane_info* planes = nullptr;
    xd_contact_property* cps = nullptr;
    unsigned* wall_list = nullptr;
    unsigned* counters = nullptr;   // [0] wall count, [1] FP64 decisions, [2] FP64 normal forces, [4] movers
    // pair recording
    unsigned* rec_count = nullptr;
    unsigned* rec_pairs = nullptr;
    // host-order transfer buffers
    double* xfer = nullptr;
    bool state_valid_forces = false;   // Fc/Mc hold the forces of the current state
    bool ready = false;                // grid and buffers set up (first upload)
    cudaGraphExec_t graph[2] = { nullptr, nullptr };   // two middle steps, per buffer parity
    bool use_graphs = true;
    unsigned rec_cap_alloc = 0;
    xd_scene_desc desc;
    std::vector<xd_plane_info> host_planes;
    std::vector<xd_contact_property> host_cps;
    std::vector<void*> allocs;
};

namespace {

template <typename T>
int alloc(MixedScene* s, T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * count);
    if (e != cudaSuccess) return cuda_status(e, "mixed scene allocation");
    s->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return XD_OK;
}

// Cell of a position.  The offset from the grid origin is formed in FP64 and
// scaled in FP32: the FP32 rounding (< 3e-7 m over a 4 m box) is far inside
// the 0.1 % margin by which the cell exceeds the largest contact distance, so
// every touching pair still lies in neighbouring cells.
__device__ __forceinline__ unsigned cell_key(const MixParams& P, double x, double y, double z)
{
    int cx = (int)floorf((float)(x - P.wo[0]) * P.inv_csf) + 1;
    int cy = (int)floorf((float)(y - P.wo[1]) * P.inv_csf) + 1;
    int cz = (int)floorf((float)(z - P.wo[2]) * P.inv_csf) + 1;
    cx = min(max(cx, 1), P.gx - 2);
    cy = min(max(cy, 1), P.gy - 2);
    cz = min(max(cz, 1), P.gz - 2);
    return ((unsigned)cz * (unsigned)P.gy + (unsigned)cy) * (unsigned)P.gx + (unsigned)cx;
}

// MODE 0: position only (first step of a call); 1: velocity of step t fused
// with the position of step t+1; 2: velocity only (last step of a call).
template <int MODE>
__global__ void __launch_bounds__(256) k_mx_integrate(MixParams P, Master M,
                                                      const float4* __restrict__ Fc,
                                                      const float4* __restrict__ Mc,
                                                      unsigned* __restrict__ keys,
                                                      unsigned* __restrict__ vals)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double ax = M.f[FAX][i], ay = M.f[FAY][i], az = M.f[FAZ][i];
    double vx = M.f[FVX][i], vy = M.f[FVY][i], vz = M.f[FVZ][i];
    if (MODE != 0) {
        const double im = M.f[FIM][i], iI = M.f[FII][i];
        const float4 f = Fc[i], t = Mc[i];
        // a' = (m g + F_contact) / m = g + F_contact / m (vv_update_velocity_kernel, impl:117-133)
        double nax = fma(im, (double)f.x, P.g[0]);
        double nay = fma(im, (double)f.y, P.g[1]);
        double naz = fma(im, (double)f.z, P.g[2]);
        double nbx = iI * (double)t.x, nby = iI * (double)t.y, nbz = iI * (double)t.z;
        const double h = 0.5 * P.dt;
        vx += h * (ax + nax);
        vy += h * (ay + nay);
        vz += h * (az + naz);
        M.f[FWX][i] += h * (M.f[FBX][i] + nbx);
        M.f[FWY][i] += h * (M.f[FBY][i] + nby);
        M.f[FWZ][i] += h * (M.f[FBZ][i] + nbz);
        M.f[FVX][i] = vx;
        M.f[FVY][i] = vy;
        M.f[FVZ][i] = vz;
        M.f[FAX][i] = ax = nax;
        M.f[FAY][i] = ay = nay;
        M.f[FAZ][i] = az = naz;
        M.f[FBX][i] = nbx;
        M.f[FBY][i] = nby;
        M.f[FBZ][i] = nbz;
    }
    double x = M.f[FX][i], y = M.f[FY][i], z = M.f[FZ][i];
    if (MODE != 2) {
        // vv_update_position_kernel (impl:85-96)
        x += P.dt * vx + P.half2dt * ax;
        y += P.dt * vy + P.half2dt * ay;
        z += P.dt * vz + P.half2dt * az;
        M.f[FX][i] = x;
        M.f[FY][i] = y;
        M.f[FZ][i] = z;
    }
    keys[i] = cell_key(P, x, y, z);
    vals[i] = i;
}

// Gathers the state into the sorted order and builds the contact view.
__global__ void __launch_bounds__(256) k_mx_reorder(MixParams P, Master S, Master D,
                                                    const unsigned* __restrict__ perm,
                                                    float4* __restrict__ pf,
                                                    longlong2* __restrict__ qa,
                                                    longlong2* __restrict__ qb,
                                                    float4* __restrict__ vf,
                                                    float4* __restrict__ vlo,
                                                    float4* __restrict__ wf)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    unsigned o = perm[i];
    double v[kFields];
#pragma unroll
    for (int k = 0; k < kFields; ++k) {
        v[k] = __ldg(S.f[k] + o);
        D.f[k][i] = v[k];
    }
    D.id[i] = __ldg(S.id + o);
    double rx = v[FX] - P.wo[0], ry = v[FY] - P.wo[1], rz = v[FZ] - P.wo[2];
    pf[i] = make_float4((float)rx, (float)ry, (float)rz, (float)v[FR]);
    qa[i] = make_longlong2(__double2ll_rn(rx * kQ), __double2ll_rn(ry * kQ));
    qb[i] = make_longlong2(__double2ll_rn(rz * kQ), __double2ll_rn(v[FR] * kQ));
    const float hx = (float)v[FVX], hy = (float)v[FVY], hz = (float)v[FVZ];
    vf[i] = make_float4(hx, hy, hz, (float)v[FM]);
    vlo[i] = make_float4((float)(v[FVX] - (double)hx), (float)(v[FVY] - (double)hy),
                         (float)(v[FVZ] - (double)hz), 0.f);
    wf[i] = make_float4((float)v[FWX], (float)v[FWY], (float)v[FWZ], 0.f);
}

__global__ void __launch_bounds__(256) k_mx_clear(const unsigned* __restrict__ prev, unsigned n,
                                                  unsigned* __restrict__ cstart,
                                                  unsigned* __restrict__ cend)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned k = prev[i];
    if (i == 0 || prev[i - 1] != k) {
        cstart[k] = 0xffffffffu;
        cend[k] = 0u;
    }
}

__global__ void __launch_bounds__(256) k_mx_bounds(const unsigned* __restrict__ sk, unsigned n,
                                                   unsigned* __restrict__ cstart,
                                                   unsigned* __restrict__ cend,
                                                   unsigned* __restrict__ prev)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned k = sk[i];
    prev[i] = k;
    if (i == 0 || sk[i - 1] != k) cstart[k] = i;
    if (i == n - 1 || sk[i + 1] != k) cend[k] = i + 1;
}

// Reference FP64 contact decision (calculate_p2p_kernel, impl:449-452),
// evaluated without multiply-add contraction like the oracle.
__device__ __forceinline__ double fp64_cdist(const Master& M, unsigned i, unsigned j)
{
    double dx = __dsub_rn(__ldg(M.f[FX] + j), __ldg(M.f[FX] + i));
    double dy = __dsub_rn(__ldg(M.f[FY] + j), __ldg(M.f[FY] + i));
    double dz = __dsub_rn(__ldg(M.f[FZ] + j), __ldg(M.f[FZ] + i));
    double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return __dsub_rn(__dadd_rn(__ldg(M.f[FR] + i), __ldg(M.f[FR] + j)), __dsqrt_rn(d2));
}

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 fk(float x, float y, float z) { return f3{ x, y, z }; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return fk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return fk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return fk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 fcross(f3 a, f3 b)
{
    return fk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Error-free transformations (Knuth's TwoSum, FMA-based TwoProd).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float z = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e)
{
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

// vj - vi of two double-float velocities (hi + lo) as an unevaluated pair
// s + t that keeps the low bits of nearly equal velocities.
__device__ __forceinline__ void df_diff(float ah, float bh, float dlo, float& s, float& t)
{
    float e;
    two_sum(ah, -bh, s, e);
    t = __fadd_rn(e, dlo);
}

// Normal speed (dv . dq) / |dq| in double-float: dv = s + t per component,
// dq the exact integer separation (|dq| < 2^31), D2 = |dq|^2 exact, d0 its
// FP32 square root.  The dot product of a fast tangential velocity with the
// contact normal cancels; here it is carried with ~2^-44 relative error and
// rounded once.
__device__ __forceinline__ float normal_speed(const float s[3], const float t[3], const int dq[3],
                                              float d0, long long D2)
{
    float hi = 0.f, lo = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float qh = __int2float_rn(dq[k]);
        const float ql = __int2float_rn(dq[k] - __float2int_rn(qh));
        float p, pe, ns, e1;
        two_prod(s[k], qh, p, pe);
        two_sum(hi, p, ns, e1);
        hi = ns;
        lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(e1, pe), __fmaf_rn(s[k], ql, __fmul_rn(t[k], qh))));
    }
    float nv, nl;
    two_sum(hi, lo, nv, nl);
    // |dq| = d0 + c with c = (D2 - d0^2) / (2 d0)
    float p, pe;
    two_prod(d0, d0, p, pe);
    const float D2h = __ll2float_rn(D2);
    const float D2l = __ll2float_rn(D2 - __float2ll_rn(D2h));
    const float c = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(D2h, p), pe), D2l), __fmul_rn(2.f, d0));
    // (nv + nl) / (d0 + c)
    const float q0 = __fdiv_rn(nv, d0);
    float qp, qpe;
    two_prod(q0, d0, qp, qpe);
    const float rem = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(nv, qp), qpe), nl), __fmul_rn(q0, c));
    return __fadd_rn(q0, __fdiv_rn(rem, d0));
}

// Per-particle contact state carried across the pairs of one particle (the
// reference keeps Ft and M in the kernel across pairs, impl:426-428).
struct PairAcc {
    f3 Ft, Mm, sumF, sumM;
};

// The force of one contact (i, j) with overlap `delta` (FP32), or, when
// `guard` is set, with the overlap from the reference's FP64 test.
// getConstant TCM = 1 (impl:238-246) and DHSModel (impl:379-401) in FP32, the
// relative velocity formed from double-float velocities, and the two
// cancellation cases (normal force near zero, rolling slip) formed in FP64.
__device__ __forceinline__ void contact_force(const MixParams& P, const Master& M, unsigned i,
                                              unsigned j, float delta, bool guard,
                                              const longlong2& qai, const longlong2& qbi,
                                              const float4& vi4, const float4& vil, const f3& wi,
                                              float ir, float im, const float4* __restrict__ pf,
                                              const longlong2* __restrict__ qa,
                                              const longlong2* __restrict__ qb,
                                              const float4* __restrict__ vf,
                                              const float4* __restrict__ vlo,
                                              const float4* __restrict__ wf,
                                              unsigned* __restrict__ counters, PairAcc& A)
{
    const float dt = P.dtf;
    const longlong2 qaj = __ldg(qa + j), qbj = __ldg(qb + j);
    const long long ddx = qaj.x - qai.x, ddy = qaj.y - qai.y, ddz = qbj.x - qbi.x;
    const long long D2 = ddx * ddx + ddy * ddy + ddz * ddz;
    const float dn = sqrtf((float)D2);
    const float inv = 1.0f / dn;
    const f3 u = fk((float)ddx * inv, (float)ddy * inv, (float)ddz * inv);
    const float4 vj4 = __ldg(vf + j), wj4 = __ldg(wf + j), vjl = __ldg(vlo + j);
    const f3 wj = fk(wj4.x, wj4.y, wj4.z);
    const float jr = __ldg(pf + j).w, jm = vj4.w;
    // vj - vi formed exactly from the double-float velocities
    float dvs[3], dvt[3];
    df_diff(vj4.x, vi4.x, __fsub_rn(vjl.x, vil.x), dvs[0], dvt[0]);
    df_diff(vj4.y, vi4.y, __fsub_rn(vjl.y, vil.y), dvs[1], dvt[1]);
    df_diff(vj4.z, vi4.z, __fsub_rn(vjl.z, vil.z), dvs[2], dvt[2]);
    const f3 dv = fk(dvs[0] + dvt[0], dvs[1] + dvt[1], dvs[2] + dvt[2]);
    // rv = vj + wj x (-rj u) - (vi + wi x (ri u))   (impl:455)
    const f3 wterm = fcross(wj, (-jr) * u) - fcross(wi, ir * u);
    const f3 rv = dv + wterm;
    // rv . u = dv . u (the rotation term is perpendicular to u), in double-float
    const int dqi[3] = { (int)ddx, (int)ddy, (int)ddz };
    const float rvu = normal_speed(dvs, dvt, dqi, dn, D2);
    f3 ev = rv - rvu * u;
    float ee = fdot(ev, ev);
    if (ee < 0.0025f * fdot(wterm, wterm)) {
        // rolling: the rotation term cancels most of the slip; form the slip in
        // FP64 from the FP64 state (FP32 rounding of the terms would dominate)
        atomicAdd(counters + 3, 1u);
        const double dd = sqrt((double)D2);
        const double ux = (double)ddx / dd, uy = (double)ddy / dd, uz = (double)ddz / dd;
        const double ri = __ldg(M.f[FR] + i), rj = __ldg(M.f[FR] + j);
        const double wix = __ldg(M.f[FWX] + i), wiy = __ldg(M.f[FWY] + i), wiz = __ldg(M.f[FWZ] + i);
        const double wjx = __ldg(M.f[FWX] + j), wjy = __ldg(M.f[FWY] + j), wjz = __ldg(M.f[FWZ] + j);
        const double dvx = __ldg(M.f[FVX] + j) - __ldg(M.f[FVX] + i);
        const double dvy = __ldg(M.f[FVY] + j) - __ldg(M.f[FVY] + i);
        const double dvz = __ldg(M.f[FVZ] + j) - __ldg(M.f[FVZ] + i);
        const double rx = dvx - rj * (wjy * uz - wjz * uy) - ri * (wiy * uz - wiz * uy);
        const double ry = dvy - rj * (wjz * ux - wjx * uz) - ri * (wiz * ux - wix * uz);
        const double rz = dvz - rj * (wjx * uy - wjy * ux) - ri * (wix * uy - wiy * ux);
        const double ru = rx * ux + ry * uy + rz * uz;
        ev = fk((float)(rx - ru * ux), (float)(ry - ru * uy), (float)(rz - ru * uz));
        ee = fdot(ev, ev);
    }
    // getConstant, TCM = 1 (impl:238-246)
    const float Meq = (im * jm) / (im + jm);
    const float Req = (ir * jr) / (ir + jr);
    const float kn = P.c43Eeq * sqrtf(Req);
    const float vn = sqrtf((4.0f * Meq * kn) / P.one_b2);
    const float ks = kn * P.sratio, vs = vn * P.sratio;
    // DHSModel (impl:379-401)
    const float fsn = -kn * (delta * sqrtf(delta));
    const float fdn = vn * rvu;
    float fn = fsn + fdn;
    if (fabsf(fn) < 0.03f * fmaxf(fabsf(fsn), fabsf(fdn))) {
        // The elastic and damping terms nearly cancel (the normal force of an
        // unloading contact crossing zero): FP32 rounding of each term would
        // dominate the small sum, so it is formed in FP64 from the FP64 state,
        // with the overlap and normal taken from the FP64 positions.
        atomicAdd(counters + 2, 1u);
        const double px = __ldg(M.f[FX] + j) - __ldg(M.f[FX] + i);
        const double py = __ldg(M.f[FY] + j) - __ldg(M.f[FY] + i);
        const double pz = __ldg(M.f[FZ] + j) - __ldg(M.f[FZ] + i);
        const double dd = sqrt(px * px + py * py + pz * pz);
        const double ux = px / dd, uy = py / dd, uz = pz / dd;
        const double dl = fp64_cdist(M, i, j);
        const double ri = __ldg(M.f[FR] + i), rj = __ldg(M.f[FR] + j);
        const double mi = __ldg(M.f[FM] + i), mj = __ldg(M.f[FM] + j);
        const double vix = __ldg(M.f[FVX] + i), viy = __ldg(M.f[FVY] + i), viz = __ldg(M.f[FVZ] + i);
        const double vjx = __ldg(M.f[FVX] + j), vjy = __ldg(M.f[FVY] + j), vjz = __ldg(M.f[FVZ] + j);
        const double wix = __ldg(M.f[FWX] + i), wiy = __ldg(M.f[FWY] + i), wiz = __ldg(M.f[FWZ] + i);
        const double wjx = __ldg(M.f[FWX] + j), wjy = __ldg(M.f[FWY] + j), wjz = __ldg(M.f[FWZ] + j);
        const double rvx = (vjx - rj * (wjy * uz - wjz * uy)) - (vix + ri * (wiy * uz - wiz * uy));
        const double rvy = (vjy - rj * (wjz * ux - wjx * uz)) - (viy + ri * (wiz * ux - wix * uz));
        const double rvz = (vjz - rj * (wjx * uy - wjy * ux)) - (viz + ri * (wix * uy - wiy * ux));
        const double Meqd = (mi * mj) / (mi + mj), Reqd = (ri * rj) / (ri + rj);
        const double knd = P.c43Eeq_d * sqrt(Reqd);
        const double vnd = sqrt((4.0 * Meqd * knd) / P.one_b2_d);
        fn = (float)(-knd * (dl * sqrt(dl)) + vnd * (rvx * ux + rvy * uy + rvz * uz));
    }
    (void)guard;
    const f3 Fn = fn * u;
    const float mag_e = sqrtf(ee);
    if (mag_e != 0.f) {
        const f3 sh = (1.0f / mag_e) * ev;
        // dv . sh = |e| exactly (sh is the unit slip direction)
        A.Ft = fminf(ks * (mag_e * dt) + vs * mag_e, P.fric * fabsf(fn)) * sh;
        A.Mm = fcross(ir * u, A.Ft);
    }
    A.sumF = A.sumF + (Fn + A.Ft);
    A.sumM = A.sumM + A.Mm;
}

constexpr int kMaxStaged = 20;   // contacts staged per thread in shared memory

// Particle-particle contacts in two phases: (1) the candidate loop -- FP32
// prefilter, exact integer test, FP64 guard band -- stages each contact's
// partner and overlap in shared memory; (2) the force loop runs over the
// staged contacts in the same order.  A particle with more contacts than the
// stage holds finishes the rest by re-scanning its candidates (same order).
template <bool RECORD>
__global__ void __launch_bounds__(256) k_mx_contact(MixParams P, Master M,
                                                    const float4* __restrict__ pf,
                                                    const longlong2* __restrict__ qa,
                                                    const longlong2* __restrict__ qb,
                                                    const float4* __restrict__ vf,
                                                    const float4* __restrict__ vlo,
                                                    const float4* __restrict__ wf,
                                                    const unsigned* __restrict__ keys,
                                                    const unsigned* __restrict__ cstart,
                                                    const unsigned* __restrict__ cend,
                                                    float4* __restrict__ Fc, float4* __restrict__ Mc,
                                                    unsigned* __restrict__ wall_list,
                                                    unsigned* __restrict__ counters,
                                                    unsigned* __restrict__ rec_count,
                                                    unsigned* __restrict__ rec_pairs, unsigned rec_cap)
{
    __shared__ unsigned st_j[kMaxStaged][256];
    __shared__ float st_d[kMaxStaged][256];
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const unsigned tx = threadIdx.x;
    const float4 pi = __ldg(pf + i);
    const longlong2 qai = __ldg(qa + i), qbi = __ldg(qb + i);
    const float ir = pi.w;
    const unsigned key = __ldg(keys + i);
    const int cx = (int)(key % (unsigned)P.gx);
    const int cy = (int)((key / (unsigned)P.gx) % (unsigned)P.gy);
    const int cz = (int)(key / ((unsigned)P.gx * (unsigned)P.gy));
    unsigned ncont = 0;
    // ---- phase 1: candidates
    for (int dz = -1; dz <= 1; ++dz) {
        for (int dy = -1; dy <= 1; ++dy) {
            const unsigned c0 = ((unsigned)(cz + dz) * (unsigned)P.gy + (unsigned)(cy + dy)) * (unsigned)P.gx +
                                (unsigned)(cx - 1);
            const unsigned s = min(min(__ldg(cstart + c0), __ldg(cstart + c0 + 1)), __ldg(cstart + c0 + 2));
            const unsigned e = max(max(__ldg(cend + c0), __ldg(cend + c0 + 1)), __ldg(cend + c0 + 2));
            for (unsigned j = s; j < e; ++j) {
                if (j == i) continue;
                const float4 pj = __ldg(pf + j);
                const float dxf = pj.x - pi.x, dyf = pj.y - pi.y, dzf = pj.z - pi.z;
                const float Rt = ir + pj.w + P.tol;
                if (dxf * dxf + dyf * dyf + dzf * dzf >= Rt * Rt) continue;
                // exact integer test on the fixed-point coordinates
                const longlong2 qaj = __ldg(qa + j), qbj = __ldg(qb + j);
                const long long ddx = qaj.x - qai.x, ddy = qaj.y - qai.y, ddz = qbj.x - qbi.x;
                const long long Rq = qbi.y + qbj.y;
                const long long D2 = ddx * ddx + ddy * ddy + ddz * ddz;
                const long long N = Rq * Rq - D2;
                const long long band = 2 * Rq * P.guard_q;
                float delta;
                if (N > band) {
                    delta = ((float)N / ((float)Rq + sqrtf((float)D2))) * kU;
                } else if (N < -band) {
                    continue;
                } else {
                    atomicAdd(counters + 1, 1u);
                    const double cd = fp64_cdist(M, i, j);
                    if (!(cd > 0)) continue;
                    delta = -(float)cd;     // negative: decided by the FP64 test
                }
                if (RECORD && ncont < rec_cap) rec_pairs[(size_t)i * rec_cap + ncont] = j;
                if (ncont < (unsigned)kMaxStaged) {
                    st_j[ncont][tx] = j;
                    st_d[ncont][tx] = delta;
                }
                ++ncont;
            }
        }
    }
    if (RECORD) rec_count[i] = ncont;
    // ---- phase 2: forces of the staged contacts, in search order
    PairAcc A;
    A.Ft = fk(0.f, 0.f, 0.f);
    A.Mm = fk(0.f, 0.f, 0.f);
    A.sumF = fk(0.f, 0.f, 0.f);
    A.sumM = fk(0.f, 0.f, 0.f);
    if (ncont) {
        const float4 vi4 = __ldg(vf + i), vil = __ldg(vlo + i), wi4 = __ldg(wf + i);
        const f3 wi = fk(wi4.x, wi4.y, wi4.z);
        const float im = vi4.w;
        const unsigned nst = min(ncont, (unsigned)kMaxStaged);
        for (unsigned c = 0; c < nst; ++c) {
            const float d = st_d[c][tx];
            contact_force(P, M, i, st_j[c][tx], fabsf(d), d < 0.f, qai, qbi, vi4, vil, wi, ir, im, pf,
                          qa, qb, vf, vlo, wf, counters, A);
        }
        if (ncont > (unsigned)kMaxStaged) {
            // ---- phase 3 (rare): contacts beyond the stage, by re-scanning
            unsigned k = 0;
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy) {
                    const unsigned c0 = ((unsigned)(cz + dz) * (unsigned)P.gy + (unsigned)(cy + dy)) *
                                            (unsigned)P.gx + (unsigned)(cx - 1);
                    const unsigned s = min(min(__ldg(cstart + c0), __ldg(cstart + c0 + 1)), __ldg(cstart + c0 + 2));
                    const unsigned e = max(max(__ldg(cend + c0), __ldg(cend + c0 + 1)), __ldg(cend + c0 + 2));
                    for (unsigned j = s; j < e; ++j) {
                        if (j == i) continue;
                        const float4 pj = __ldg(pf + j);
                        const float dxf = pj.x - pi.x, dyf = pj.y - pi.y, dzf = pj.z - pi.z;
                        const float Rt = ir + pj.w + P.tol;
                        if (dxf * dxf + dyf * dyf + dzf * dzf >= Rt * Rt) continue;
                        const longlong2 qaj = __ldg(qa + j), qbj = __ldg(qb + j);
                        const long long ddx = qaj.x - qai.x, ddy = qaj.y - qai.y, ddz = qbj.x - qbi.x;
                        const long long Rq = qbi.y + qbj.y;
                        const long long D2 = ddx * ddx + ddy * ddy + ddz * ddz;
                        const long long N = Rq * Rq - D2;
                        const long long band = 2 * Rq * P.guard_q;
                        float delta;
                        if (N > band) {
                            delta = ((float)N / ((float)Rq + sqrtf((float)D2))) * kU;
                        } else if (N < -band) {
                            continue;
                        } else {
                            const double cd = fp64_cdist(M, i, j);
                            if (!(cd > 0)) continue;
                            delta = (float)cd;
                        }
                        if (k++ < (unsigned)kMaxStaged) continue;
                        contact_force(P, M, i, j, delta, false, qai, qbi, vi4, vil, wi, ir, im, pf, qa,
                                      qb, vf, vlo, wf, counters, A);
                    }
                }
        }
    }
    Fc[i] = make_float4(A.sumF.x, A.sumF.y, A.sumF.z, 0.f);
    Mc[i] = make_float4(A.sumM.x, A.sumM.y, A.sumM.z, 0.f);
    // walls: FP32 distance to each plane's supporting plane; near ones go to the FP64 pass
    bool near = false;
    for (int w = 0; w < P.nplanes; ++w) {
        const float hz = (pi.x - P.pxw[w][0]) * P.pun[w][0] + (pi.y - P.pxw[w][1]) * P.pun[w][1] +
                         (pi.z - P.pxw[w][2]) * P.pun[w][2];
        near |= fabsf(hz) < ir + P.wall_tol;
    }
    const unsigned act = __activemask();
    const unsigned ballot = __ballot_sync(act, near);
    if (ballot) {
        const unsigned lane = threadIdx.x & 31u;
        const int leader = __ffs(ballot) - 1;
        unsigned base = 0;
        if ((int)lane == leader) base = atomicAdd(counters, (unsigned)__popc(ballot));
        base = __shfl_sync(act, base, leader);
        if (near) wall_list[base + __popc(ballot & ((1u << lane) - 1u))] = i;
    }
}

// plane_contact_force_kernel<1> (impl:572-621) for the listed particles, all
// planes in order, in FP64; adds to the FP32 contact force.
__global__ void __launch_bounds__(128) k_mx_walls(MixParams P, Master M,
                                                  const xd_plane_info* __restrict__ planes,
                                                  const xd_contact_property* __restrict__ cps,
                                                  const unsigned* __restrict__ wall_list,
                                                  const unsigned* __restrict__ counters,
                                                  float4* __restrict__ Fc)
{
    const unsigned count = counters[0];
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const unsigned i = wall_list[k];
        const double m = M.f[FM][i];
        const d3 ip = mk(M.f[FX][i], M.f[FY][i], M.f[FZ][i]);
        const double r = M.f[FR][i];
        const d3 iv = mk(M.f[FVX][i], M.f[FVY][i], M.f[FVZ][i]);
        const d3 iw = mk(M.f[FWX][i], M.f[FWY][i], M.f[FWZ][i]);
        d3 f = mk(0, 0, 0);
        for (int w = 0; w < P.nplanes; ++w) {
            PlaneD pe = load_plane(planes + w);
            d3 Fn = mk(0, 0, 0), Ft = mk(0, 0, 0), Mo = mk(0, 0, 0);
            d3 dp = ip - pe.xw;
            d3 unit = mk(0, 0, 0);
            d3 wp = mk(dot(dp, pe.u1), dot(dp, pe.u2), dot(dp, pe.uw));
            double cdist = plane_detection(pe, ip, wp, unit, r);
            if (cdist > 0) {
                PairConst pc = load_pair_const(cps + w);
                d3 dv = -(iv + cross(iw, r * unit));
                xd::Fc c = get_constant(pc, r, 0.0, m, 0.0);
                dhs(c, 0, 0, 0, 0, 0, 0, pc.coh, cdist, dv, unit, P.dt, Ft, Fn, Mo);
            }
            f += Fn + Ft;
        }
        float4 o = Fc[i];
        o.x += (float)f.x;
        o.y += (float)f.y;
        o.z += (float)f.z;
        Fc[i] = o;
    }
}

// host-order state <-> master (reference layouts)
__global__ void __launch_bounds__(256) k_mx_load(MixParams P, Master M, const double* __restrict__ pos,
                                                 const double* __restrict__ vel,
                                                 const double* __restrict__ acc,
                                                 const double* __restrict__ omega,
                                                 const double* __restrict__ alpha,
                                                 const double* __restrict__ mass,
                                                 const double* __restrict__ inertia)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    M.f[FX][i] = pos[4 * (size_t)i + 0];
    M.f[FY][i] = pos[4 * (size_t)i + 1];
    M.f[FZ][i] = pos[4 * (size_t)i + 2];
    M.f[FR][i] = pos[4 * (size_t)i + 3];
    for (int a = 0; a < 3; ++a) {
        M.f[FVX + a][i] = vel[3 * (size_t)i + a];
        M.f[FWX + a][i] = omega[3 * (size_t)i + a];
        M.f[FAX + a][i] = acc[3 * (size_t)i + a];
        M.f[FBX + a][i] = alpha[3 * (size_t)i + a];
    }
    double m = mass[i], I = inertia[i];
    M.f[FM][i] = m;
    M.f[FI][i] = I;
    M.f[FIM][i] = 1.0 / m;
    M.f[FII][i] = 1.0 / I;
    M.id[i] = i;
}

__global__ void __launch_bounds__(256) k_mx_store(MixParams P, Master M, double* __restrict__ pos,
                                                  double* __restrict__ vel, double* __restrict__ acc,
                                                  double* __restrict__ omega,
                                                  double* __restrict__ alpha,
                                                  double* __restrict__ force,
                                                  double* __restrict__ moment)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    size_t o = M.id[i];
    pos[4 * o + 0] = M.f[FX][i];
    pos[4 * o + 1] = M.f[FY][i];
    pos[4 * o + 2] = M.f[FZ][i];
    pos[4 * o + 3] = M.f[FR][i];
    double m = M.f[FM][i];
    for (int a = 0; a < 3; ++a) {
        vel[3 * o + a] = M.f[FVX + a][i];
        omega[3 * o + a] = M.f[FWX + a][i];
        acc[3 * o + a] = M.f[FAX + a][i];
        alpha[3 * o + a] = M.f[FBX + a][i];
        force[3 * o + a] = m * P.g[a];
        moment[3 * o + a] = 0.0;
    }
}

__global__ void __launch_bounds__(256) k_mx_store_forces(MixParams P, const unsigned* __restrict__ id,
                                                         const float4* __restrict__ Fc,
                                                         const float4* __restrict__ Mc,
                                                         double* __restrict__ force,
                                                         double* __restrict__ moment)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    size_t o = id[i];
    float4 f = Fc[i], t = Mc[i];
    force[3 * o + 0] = f.x;
    force[3 * o + 1] = f.y;
    force[3 * o + 2] = f.z;
    moment[3 * o + 0] = t.x;
    moment[3 * o + 1] = t.y;
    moment[3 * o + 2] = t.z;
}

__global__ void __launch_bounds__(256) k_mx_keys(MixParams P, Master M, unsigned* __restrict__ keys,
                                                 unsigned* __restrict__ vals)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    keys[i] = cell_key(P, M.f[FX][i], M.f[FY][i], M.f[FZ][i]);
    vals[i] = i;
}

// ---- near-sorted resort ("movers") -----------------------------------------
// The state is in the previous step's cell order, so prev[] (that order's
// keys) is ascending and most particles keep their key.  Sorting (key, slot)
// stably then only needs the movers (key != prev) ranked among themselves;
// every other slot keeps its relative order:
//   position(stayer i) = (i - movers before i) + movers with (key, slot) < (prev[i], i)
//   position(mover m)  = stayers with (prev, slot) < (key_m, slot_m) + rank of m among movers
// which is exactly the stable sort's output.
constexpr int kMvBlock = 1024;     // slots per block in the flag/compact pass (256 threads x 4)

__global__ void __launch_bounds__(256) k_mv_count(const unsigned* __restrict__ keys,
                                                  const unsigned* __restrict__ prev, unsigned n,
                                                  unsigned* __restrict__ bcount)
{
    __shared__ unsigned wsum[8];
    const unsigned base = blockIdx.x * kMvBlock;
    unsigned c = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        unsigned i = base + k * 256 + threadIdx.x;
        if (i < n && keys[i] != prev[i]) ++c;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < 8; ++w) t += wsum[w];
        bcount[blockIdx.x] = t;
    }
}

// exclusive scan of the per-block counts (one block); total movers -> *total
__global__ void __launch_bounds__(1024) k_mv_scan(unsigned* __restrict__ bcount, unsigned nb,
                                                  unsigned* __restrict__ total)
{
    __shared__ unsigned wsum[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (unsigned b0 = 0; b0 < nb; b0 += 1024) {
        unsigned i = b0 + threadIdx.x;
        unsigned v = i < nb ? bcount[i] : 0u;
        unsigned x = v;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (unsigned)o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned w = wsum[lane], t = w;
            for (int o = 1; o < 32; o <<= 1) {
                unsigned y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= (unsigned)o) t += y;
            }
            wsum[lane] = t - w;
        }
        __syncthreads();
        unsigned excl = x - v + wsum[warp] + carry;
        if (i < nb) bcount[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// movers compacted in slot order; mprefix[i] = movers in slots [0, i)
__global__ void __launch_bounds__(256) k_mv_compact(const unsigned* __restrict__ keys,
                                                    const unsigned* __restrict__ prev, unsigned n,
                                                    const unsigned* __restrict__ boff,
                                                    unsigned* __restrict__ mprefix,
                                                    unsigned* __restrict__ mkey,
                                                    unsigned* __restrict__ mslot)
{
    __shared__ unsigned wsum[32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned run = boff[blockIdx.x];
    const unsigned base = blockIdx.x * kMvBlock;
    for (int k = 0; k < 4; ++k) {
        unsigned i = base + k * 256 + threadIdx.x;
        bool mv = i < n && keys[i] != prev[i];
        unsigned bal = __ballot_sync(0xffffffffu, mv);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        unsigned before = 0, all = 0;
        for (int w = 0; w < 8; ++w) {
            unsigned c = wsum[w];
            if (w < (int)warp) before += c;
            all += c;
        }
        unsigned pos = run + before + __popc(bal & ((1u << lane) - 1u));
        if (i < n) mprefix[i] = pos;
        if (mv) {
            mkey[pos] = keys[i];
            mslot[pos] = i;
        }
        if (i == n - 1) mprefix[n] = pos + (mv ? 1u : 0u);
        run += all;
        __syncthreads();
    }
}

__device__ __forceinline__ bool pair_less(unsigned ka, unsigned sa, unsigned kb, unsigned sb)
{
    return ka < kb || (ka == kb && sa < sb);
}

// first index in a[0, n) with a[idx] >= v
__device__ __forceinline__ unsigned lower_bound_u(const unsigned* __restrict__ a, unsigned n, unsigned v)
{
    unsigned lo = 0, hi = n;
    while (lo < hi) {
        unsigned mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Ranks each mover among all movers (shared-memory tiles of the mover set,
// O(M^2) compares: M is a few thousand per step; any M stays correct) and
// places it.  Also writes the sorted mover list for the stayers' searches.
constexpr int kRankTile = 2048;
__global__ void __launch_bounds__(256) k_mv_rank(const unsigned* __restrict__ total,
                                                 const unsigned* __restrict__ mkey,
                                                 const unsigned* __restrict__ mslot,
                                                 const unsigned* __restrict__ prev,
                                                 const unsigned* __restrict__ mprefix, unsigned n,
                                                 unsigned* __restrict__ smkey,
                                                 unsigned* __restrict__ smslot,
                                                 unsigned* __restrict__ skeys,
                                                 unsigned* __restrict__ perm)
{
    __shared__ unsigned tk[kRankTile], ts[kRankTile];
    const unsigned M = *total;
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned base = blockIdx.x * blockDim.x; base < M; base += stride) {
        const unsigned m = base + threadIdx.x;
        const bool act = m < M;
        const unsigned key = act ? mkey[m] : 0u, slot = act ? mslot[m] : 0u;
        unsigned rank = 0;
        for (unsigned t0 = 0; t0 < M; t0 += kRankTile) {
            const unsigned cnt = min((unsigned)kRankTile, M - t0);
            __syncthreads();
            for (unsigned k = threadIdx.x; k < cnt; k += blockDim.x) {
                tk[k] = mkey[t0 + k];
                ts[k] = mslot[t0 + k];
            }
            __syncthreads();
            if (act)
                for (unsigned k = 0; k < cnt; ++k) rank += pair_less(tk[k], ts[k], key, slot) ? 1u : 0u;
        }
        if (act) {
            smkey[rank] = key;
            smslot[rank] = slot;
            const unsigned L = lower_bound_u(prev, n, key);
            const unsigned U = lower_bound_u(prev, n, key + 1u);
            const unsigned cend = max(L, min(U, slot));
            const unsigned pos = (cend - mprefix[cend]) + rank;
            skeys[pos] = key;
            perm[pos] = slot;
        }
    }
}

__global__ void __launch_bounds__(256) k_mv_place(const unsigned* __restrict__ keys,
                                                  const unsigned* __restrict__ prev, unsigned n,
                                                  const unsigned* __restrict__ mprefix,
                                                  const unsigned* __restrict__ total,
                                                  const unsigned* __restrict__ smkey,
                                                  const unsigned* __restrict__ smslot,
                                                  unsigned* __restrict__ skeys,
                                                  unsigned* __restrict__ perm)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned k = prev[i];
    if (keys[i] != k) return;   // a mover: placed by k_mv_rank
    const unsigned M = *total;
    unsigned lo = 0, hi = M;    // movers with (key, slot) < (k, i)
    while (lo < hi) {
        unsigned mid = (lo + hi) >> 1;
        if (pair_less(__ldg(smkey + mid), __ldg(smslot + mid), k, i)) lo = mid + 1;
        else hi = mid;
    }
    const unsigned pos = (i - mprefix[i]) + lo;
    skeys[pos] = k;
    perm[pos] = i;
}

inline unsigned blocks(unsigned n, unsigned t) { return div_up(n ? n : 1u, t); }

}  // namespace

// ------------------------------------------------------------------ host

static int mixed_setup(MixedScene* s, const xd_scene_desc& d, const double* pos_host)
{
    s->n = d.np;
    s->nplanes = d.nplanes;
    // grid from the bounding box of particles and walls
    double lo[3] = { 1e300, 1e300, 1e300 }, hi[3] = { -1e300, -1e300, -1e300 };
    double rmax = 0.0;
    for (unsigned i = 0; i < d.np; ++i) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = fmin(lo[a], pos_host[4 * (size_t)i + a]);
            hi[a] = fmax(hi[a], pos_host[4 * (size_t)i + a]);
        }
        rmax = fmax(rmax, pos_host[4 * (size_t)i + 3]);
    }
    for (unsigned w = 0; w < d.nplanes; ++w) {
        const xd_plane_info& p = d.planes[w];
        const double* pts[4] = { p.xw, p.w2, p.w3, p.w4 };
        for (auto q : pts)
            for (int a = 0; a < 3; ++a) {
                lo[a] = fmin(lo[a], q[a]);
                hi[a] = fmax(hi[a], q[a]);
            }
    }
    if (d.np == 0) {
        for (int a = 0; a < 3; ++a) { lo[a] = 0; hi[a] = 1; }
        rmax = 0.5;
    }
    if (!(rmax > 0.0)) return set_error(XD_ERR_INVALID, "mixed mode: particle radii must be > 0");
    s->cs = 2.0 * rmax * 1.001;
    double margin = 2.0 * s->cs;
    int g[3];
    unsigned long long ncell = 1;
    for (int a = 0; a < 3; ++a) {
        lo[a] -= margin;
        hi[a] += margin;
        g[a] = (int)ceil((hi[a] - lo[a]) / s->cs) + 2;
        ncell *= (unsigned long long)g[a];
    }
    if (ncell > 0x7fffffffull)
        return set_error(XD_ERR_CAPACITY, "mixed mode: grid of %llu cells is too large", ncell);
    s->gx = g[0]; s->gy = g[1]; s->gz = g[2];
    s->ncell = (unsigned)ncell;
    MixParams& P = s->P;
    memset(&P, 0, sizeof(P));
    P.gx = g[0]; P.gy = g[1]; P.gz = g[2];
    P.n = d.np;
    for (int a = 0; a < 3; ++a) {
        P.wo[a] = lo[a];
        P.g[a] = d.params.gravity[a];
    }
    P.inv_cs = 1.0 / s->cs;
    P.inv_csf = (float)P.inv_cs;
    P.dt = d.params.dt;
    P.half2dt = d.params.half2dt;
    P.dtf = (float)d.params.dt;
    P.tol = 4e-6f;
    P.wall_tol = 1e-5f;
    const xd_contact_property& cp = d.cp_pp;
    double Eeq = (cp.Ei * cp.Ej) / (cp.Ei * (1 - cp.prj * cp.prj) + cp.Ej * (1 - cp.pri * cp.pri));
    double beta = M_PI / log(cp.rest);
    P.c43Eeq_d = (4.0 / 3.0) * Eeq;
    P.one_b2_d = 1.0 + beta * beta;
    P.c43Eeq = (float)P.c43Eeq_d;
    P.one_b2 = (float)P.one_b2_d;
    P.sratio = (float)cp.sratio;
    P.fric = (float)cp.fric;
    P.guard_q = (long long)ceil(kGuard * kQ);
    P.nplanes = (int)d.nplanes;
    for (unsigned w = 0; w < d.nplanes; ++w) {
        const xd_plane_info& p = d.planes[w];
        double un = sqrt(p.uw[0] * p.uw[0] + p.uw[1] * p.uw[1] + p.uw[2] * p.uw[2]);
        for (int a = 0; a < 3; ++a) {
            P.pxw[w][a] = (float)(p.xw[a] - lo[a]);
            P.pun[w][a] = (float)(p.uw[a] / un);
        }
    }

    const size_t n = d.np;
    int st = XD_OK;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    for (int b = 0; b < 2; ++b) {
        for (int k = 0; k < kFields; ++k) A(alloc(s, &s->m[b].f[k], n));
        A(alloc(s, &s->m[b].id, n));
    }
    A(alloc(s, &s->pf, n));
    A(alloc(s, &s->qa, n));
    A(alloc(s, &s->qb, n));
    A(alloc(s, &s->vf, n));
    A(alloc(s, &s->vlo, n));
    A(alloc(s, &s->wf, n));
    A(alloc(s, &s->Fc, n));
    A(alloc(s, &s->Mc, n));
    A(alloc(s, &s->keys, n));
    A(alloc(s, &s->vals, n));
    A(alloc(s, &s->prev_keys, n));
    A(alloc(s, &s->cstart, s->ncell));
    A(alloc(s, &s->cend, s->ncell));
    char* scr = nullptr;
    A(alloc(s, &scr, radix_sort_scratch_bytes((unsigned)n)));
    s->sort_scratch = scr;
    A(alloc(s, &s->planes, s->nplanes));
    A(alloc(s, &s->cps, s->nplanes));
    A(alloc(s, &s->wall_list, n));
    A(alloc(s, &s->mv_bcount, div_up((unsigned)(n ? n : 1), 1024u)));
    A(alloc(s, &s->mv_prefix, n + 1));
    A(alloc(s, &s->mv_key, n));
    A(alloc(s, &s->mv_slot, n));
    A(alloc(s, &s->mv_skey, n));
    A(alloc(s, &s->mv_sslot, n));
    A(alloc(s, &s->mv_sorted, n));
    A(alloc(s, &s->mv_perm, n));
    A(alloc(s, &s->counters, 8));
    if (st == XD_OK && s->nplanes) {
        A(cuda_status(cudaMemcpy(s->planes, d.planes, sizeof(xd_plane_info) * s->nplanes, cudaMemcpyHostToDevice), "mixed planes"));
        A(cuda_status(cudaMemcpy(s->cps, d.cp_planes, sizeof(xd_contact_property) * s->nplanes, cudaMemcpyHostToDevice), "mixed planes"));
    }
    return st;
}

int mixed_create(const xd_scene_desc& d, MixedScene** out)
{
    *out = nullptr;
    if (d.ntri) return set_error(XD_ERR_INVALID, "mixed mode: triangle meshes are not supported yet");
    if (d.nplanes > (unsigned)kMaxPlanes)
        return set_error(XD_ERR_INVALID, "mixed mode: at most %d planes", kMaxPlanes);
    if (d.cp_pp.coh != 0.0) return set_error(XD_ERR_INVALID, "mixed mode: cohesion is not supported");
    if (d.nplanes && (!d.planes || !d.cp_planes))
        return set_error(XD_ERR_INVALID, "mixed mode: planes given without arrays");
    MixedScene* s = new (std::nothrow) MixedScene();
    if (!s) return set_error(XD_ERR_NOMEM, "mixed scene: host allocation");
    s->desc = d;
    s->host_planes.assign(d.planes, d.planes + d.nplanes);
    s->host_cps.assign(d.cp_planes, d.cp_planes + d.nplanes);
    s->desc.planes = s->host_planes.data();
    s->desc.cp_planes = s->host_cps.data();
    s->desc.poly = nullptr;
    s->desc.sphere = nullptr;
    s->desc.vlist = nullptr;
    s->desc.pmi = nullptr;
    s->desc.cp_poly = nullptr;
    *out = s;
    return XD_OK;
}

void mixed_destroy(MixedScene* s)
{
    if (!s) return;
    cudaDeviceSynchronize();
    for (int k = 0; k < 2; ++k)
        if (s->graph[k]) cudaGraphExecDestroy(s->graph[k]);
    for (void* p : s->allocs) cudaFree(p);
    delete s;
}

static int ensure_xfer(MixedScene* s)
{
    if (s->xfer) return XD_OK;
    return alloc(s, &s->xfer, (size_t)s->n * (4 + 3 * 6 + 2));
}

int mixed_upload(MixedScene* s, const double* pos, const double* vel, const double* acc,
                 const double* omega, const double* alpha, const double* mass,
                 const double* inertia, cudaStream_t q)
{
    if (!pos || !vel || !acc || !omega || !alpha || !mass || !inertia)
        return set_error(XD_ERR_INVALID, "mixed mode: upload needs pos, vel, acc, omega, alpha, mass, inertia");
    if (!s->ready) {
        int r = mixed_setup(s, s->desc, pos);
        if (r != XD_OK) return r;
        s->ready = true;
    }
    int st = ensure_xfer(s);
    if (st != XD_OK) return st;
    size_t n = s->n;
    double* b = s->xfer;
    double *dpos = b, *dvel = b + 4 * n, *dacc = dvel + 3 * n, *dom = dacc + 3 * n,
           *dal = dom + 3 * n, *dm = dal + 3 * n, *dI = dm + n;
    auto cp = [&](double* d, const double* h, size_t cnt) {
        if (st == XD_OK)
            st = cuda_status(cudaMemcpyAsync(d, h, sizeof(double) * cnt, cudaMemcpyHostToDevice, q), "mixed upload");
    };
    cp(dpos, pos, 4 * n);
    cp(dvel, vel, 3 * n);
    cp(dacc, acc, 3 * n);
    cp(dom, omega, 3 * n);
    cp(dal, alpha, 3 * n);
    cp(dm, mass, n);
    cp(dI, inertia, n);
    if (st != XD_OK) return st;
    s->cur = 0;
    s->cells_clean = false;   // the state is in upload order again: next resort is a full sort
    k_mx_load<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[0], dpos, dvel, dacc, dom, dal, dm, dI);
    st = launch_status("mixed upload");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "mixed upload");
    s->state_valid_forces = false;
    return st;
}

int mixed_download(MixedScene* s, double* pos, double* vel, double* acc, double* omega,
                   double* alpha, double* force, double* moment, cudaStream_t q)
{
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    int st = ensure_xfer(s);
    if (st != XD_OK) return st;
    size_t n = s->n;
    double* b = s->xfer;
    double *dpos = b, *dvel = b + 4 * n, *dacc = dvel + 3 * n, *dom = dacc + 3 * n,
           *dal = dom + 3 * n, *df = dal + 3 * n, *dmo = df + 3 * n;
    // xfer holds 4n + 18n + 2n doubles: pos, vel, acc, omega, alpha, force, moment fit in 22n
    k_mx_store<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[s->cur], dpos, dvel, dacc, dom, dal, df, dmo);
    st = launch_status("mixed download");
    auto cp = [&](double* h, const double* d, size_t cnt) {
        if (st == XD_OK && h)
            st = cuda_status(cudaMemcpyAsync(h, d, sizeof(double) * cnt, cudaMemcpyDeviceToHost, q), "mixed download");
    };
    cp(pos, dpos, 4 * n);
    cp(vel, dvel, 3 * n);
    cp(acc, dacc, 3 * n);
    cp(omega, dom, 3 * n);
    cp(alpha, dal, 3 * n);
    cp(force, df, 3 * n);
    cp(moment, dmo, 3 * n);
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "mixed download");
    return st;
}

// grid + reorder + contacts for the current positions (keys already in s->keys)
static int grid_and_contacts(MixedScene* s, cudaStream_t q, const Phases& ph, bool record,
                             unsigned rec_cap)
{
    const unsigned n = s->n;
    int st;
    unsigned *sk = nullptr, *sv = nullptr;
    ph.begin(2, q);
    if (!s->cells_clean) {
        // no previous order to exploit: full stable radix sort
        st = radix_sort_pairs(s->keys, s->vals, n, key_bits_for(s->ncell), s->sort_scratch, q, &sk, &sv);
        if (st == XD_OK) st = launch_fill_cells(s->cstart, s->cend, s->ncell, q);
        if (st == XD_OK)
            st = cuda_status(cudaMemsetAsync(s->counters + 4, 0, sizeof(unsigned), q), "mixed movers");
    } else {
        const unsigned nb = div_up(n, 1024u);
        unsigned* total = s->counters + 4;
        k_mv_count<<<nb, 256, 0, q>>>(s->keys, s->prev_keys, n, s->mv_bcount);
        k_mv_scan<<<1, 1024, 0, q>>>(s->mv_bcount, nb, total);
        k_mv_compact<<<nb, 256, 0, q>>>(s->keys, s->prev_keys, n, s->mv_bcount, s->mv_prefix,
                                        s->mv_key, s->mv_slot);
        k_mv_rank<<<152 * 2, 256, 0, q>>>(total, s->mv_key, s->mv_slot, s->prev_keys, s->mv_prefix,
                                          n, s->mv_skey, s->mv_sslot, s->mv_sorted, s->mv_perm);
        k_mv_place<<<blocks(n, 256), 256, 0, q>>>(s->keys, s->prev_keys, n, s->mv_prefix, total,
                                                  s->mv_skey, s->mv_sslot, s->mv_sorted, s->mv_perm);
        st = launch_status("mixed near-sorted resort");
        sk = s->mv_sorted;
        sv = s->mv_perm;
        if (st == XD_OK) {
            k_mx_clear<<<blocks(n, 256), 256, 0, q>>>(s->prev_keys, n, s->cstart, s->cend);
            st = launch_status("mixed clear cells");
        }
    }
    if (st == XD_OK) {
        k_mx_bounds<<<blocks(n, 256), 256, 0, q>>>(sk, n, s->cstart, s->cend, s->prev_keys);
        st = launch_status("mixed cell bounds");
        s->cells_clean = true;
    }
    ph.end(2, q);
    if (st != XD_OK) return st;
    ph.begin(6, q);
    const int nxt = 1 - s->cur;
    k_mx_reorder<<<blocks(n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->m[nxt], sv, s->pf, s->qa, s->qb,
                                                s->vf, s->vlo, s->wf);
    st = launch_status("mixed reorder");
    s->cur = nxt;
    ph.end(6, q);
    if (st != XD_OK) return st;
    ph.begin(3, q);
    st = cuda_status(cudaMemsetAsync(s->counters, 0, sizeof(unsigned), q), "mixed counters");
    if (st != XD_OK) return st;
    // prev_keys now holds the sorted keys: the contact kernel reads cell coordinates from it
    if (record)
        k_mx_contact<true><<<blocks(n, 256), 256, 0, q>>>(
            s->P, s->m[s->cur], s->pf, s->qa, s->qb, s->vf, s->vlo, s->wf, s->prev_keys, s->cstart,
            s->cend, s->Fc, s->Mc, s->wall_list, s->counters, s->rec_count, s->rec_pairs, rec_cap);
    else
        k_mx_contact<false><<<blocks(n, 256), 256, 0, q>>>(
            s->P, s->m[s->cur], s->pf, s->qa, s->qb, s->vf, s->vlo, s->wf, s->prev_keys, s->cstart,
            s->cend, s->Fc, s->Mc, s->wall_list, s->counters, nullptr, nullptr, 0);
    st = launch_status("mixed contact");
    ph.end(3, q);
    if (st != XD_OK || !s->nplanes) return st;
    ph.begin(4, q);
    k_mx_walls<<<152 * 4, 128, 0, q>>>(s->P, s->m[s->cur], s->planes, s->cps, s->wall_list, s->counters, s->Fc);
    st = launch_status("mixed walls");
    ph.end(4, q);
    return st;
}

// One middle step: grid, contacts and walls, then the fused velocity/position update.
static int middle_step(MixedScene* s, cudaStream_t q, const Phases& ph, bool last)
{
    const unsigned n = s->n;
    int st = grid_and_contacts(s, q, ph, false, 0);
    if (st != XD_OK) return st;
    ph.begin(0, q);
    if (!last)
        k_mx_integrate<1><<<blocks(n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->Fc, s->Mc, s->keys, s->vals);
    else
        k_mx_integrate<2><<<blocks(n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->Fc, s->Mc, s->keys, s->vals);
    st = launch_status("mixed integrate");
    ph.end(0, q);
    return st;
}

// Captures two middle steps into a graph for the current buffer parity (the
// pair of steps leaves the parity unchanged).  Needs cells_clean.
static int capture_pair(MixedScene* s, cudaStream_t q)
{
    const int parity = s->cur;
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "mixed graph stream");
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int st = cuda_status(e, "mixed graph capture");
    Phases none;
    if (st == XD_OK) st = middle_step(s, cs, none, false);
    if (st == XD_OK) st = middle_step(s, cs, none, false);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    if (st == XD_OK) st = cuda_status(e, "mixed graph capture");
    s->cur = parity;   // capture only recorded the launches
    if (st == XD_OK) st = cuda_status(cudaGraphInstantiate(&s->graph[parity], g, 0), "mixed graph instantiate");
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    (void)q;
    return st;
}

int mixed_step(MixedScene* s, unsigned nsteps, cudaStream_t q, const Phases& ph)
{
    if (nsteps == 0 || s->n == 0) return XD_OK;
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    const unsigned n = s->n;
    const bool graphs = s->use_graphs && ph.fn == nullptr;
    int st;
    if (s->cells_clean && s->n > 1) {
        // The near-sorted resort ranks the movers in O(M^2); after a burst of
        // movers in the previous call, start this one with a full radix sort.
        unsigned prev_movers = 0;
        st = cuda_status(cudaMemcpyAsync(&prev_movers, s->counters + 4, sizeof(unsigned),
                                         cudaMemcpyDeviceToHost, q), "mixed mover count");
        if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "mixed mover count");
        if (st != XD_OK) return st;
        if (prev_movers > s->n / 16 || prev_movers > 65536u) s->cells_clean = false;
    }
    ph.begin(0, q);
    k_mx_integrate<0><<<blocks(n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->Fc, s->Mc, s->keys, s->vals);
    st = launch_status("mixed integrate");
    ph.end(0, q);
    if (st != XD_OK) return st;
    unsigned t = 0;
    if (!s->cells_clean) {
        st = middle_step(s, q, ph, nsteps == 1);
        if (st != XD_OK) return st;
        t = 1;
    }
    // pairs of middle steps as one graph launch; the last step runs directly
    while (graphs && nsteps - t >= 3) {
        if (!s->graph[s->cur]) {
            st = capture_pair(s, q);
            if (st != XD_OK) return st;
        }
        st = cuda_status(cudaGraphLaunch(s->graph[s->cur], q), "mixed graph launch");
        if (st != XD_OK) return st;
        t += 2;   // two reorders: the buffer parity is unchanged
    }
    for (; t < nsteps; ++t) {
        st = middle_step(s, q, ph, t + 1 == nsteps);
        if (st != XD_OK) return st;
    }
    s->state_valid_forces = false;
    return XD_OK;
}

unsigned long long mixed_launches(MixedScene* s, unsigned nsteps)
{
    if (!s || nsteps == 0 || s->n == 0) return 0;
    const unsigned passes = (key_bits_for(s->ncell) + 7) / 8;
    // per step: 5 resort kernels + clear + bounds + reorder + contact (+ walls) + integrate
    const unsigned long long per = 5 + 1 + 1 + 1 + 1 + (s->nplanes ? 1 : 0) + 1;
    unsigned long long total = 1 + per * nsteps;   // + the first position update
    if (!s->cells_clean && s->n > 1) total += 5ull * passes - 5;   // first step: full radix sort
    return total;
}

int mixed_eval_contacts(MixedScene* s, double* force, double* moment, cudaStream_t q)
{
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    int st = ensure_xfer(s);
    if (st != XD_OK) return st;
    Phases none;
    k_mx_keys<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->keys, s->vals);
    st = launch_status("mixed keys");
    if (st == XD_OK) st = grid_and_contacts(s, q, none, false, 0);
    if (st != XD_OK) return st;
    size_t n = s->n;
    double *df = s->xfer, *dm = s->xfer + 3 * n;
    k_mx_store_forces<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[s->cur].id, s->Fc, s->Mc, df, dm);
    st = launch_status("mixed store forces");
    if (st == XD_OK && force)
        st = cuda_status(cudaMemcpyAsync(force, df, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, q), "eval");
    if (st == XD_OK && moment)
        st = cuda_status(cudaMemcpyAsync(moment, dm, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, q), "eval");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "eval");
    return st;
}

int mixed_pair_list(MixedScene* s, unsigned cap_per_particle, unsigned* counts, unsigned* partners,
                    cudaStream_t q)
{
    if (cap_per_particle == 0) return set_error(XD_ERR_INVALID, "pair list: zero capacity");
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    int st = XD_OK;
    if (!s->rec_count) st = alloc(s, &s->rec_count, s->n);
    if (st == XD_OK && s->rec_cap_alloc < cap_per_particle) {
        st = alloc(s, &s->rec_pairs, (size_t)s->n * cap_per_particle);
        s->rec_cap_alloc = cap_per_particle;
    }
    if (st != XD_OK) return st;
    Phases none;
    k_mx_keys<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->keys, s->vals);
    st = launch_status("mixed keys");
    if (st == XD_OK) st = grid_and_contacts(s, q, none, true, cap_per_particle);
    if (st != XD_OK) return st;
    // counts/partners are reported in original particle ids
    size_t n = s->n;
    std::vector<unsigned> ids(n), cnt(n), part((size_t)n * cap_per_particle);
    st = cuda_status(cudaMemcpyAsync(ids.data(), s->m[s->cur].id, 4 * n, cudaMemcpyDeviceToHost, q), "pairs");
    if (st == XD_OK) st = cuda_status(cudaMemcpyAsync(cnt.data(), s->rec_count, 4 * n, cudaMemcpyDeviceToHost, q), "pairs");
    if (st == XD_OK)
        st = cuda_status(cudaMemcpyAsync(part.data(), s->rec_pairs, 4 * n * cap_per_particle, cudaMemcpyDeviceToHost, q), "pairs");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "pairs");
    if (st != XD_OK) return st;
    for (size_t i = 0; i < n; ++i) {
        unsigned o = ids[i];
        counts[o] = cnt[i];
        unsigned c = cnt[i] < cap_per_particle ? cnt[i] : cap_per_particle;
        for (unsigned k = 0; k < c; ++k) partners[(size_t)o * cap_per_particle + k] = ids[part[i * cap_per_particle + k]];
    }
    return XD_OK;
}

int mixed_counters(MixedScene* s, unsigned long long* out, cudaStream_t q)
{
    unsigned c[4] = {};
    int st = cuda_status(cudaMemcpyAsync(c, s->counters, sizeof(c), cudaMemcpyDeviceToHost, q), "counters");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "counters");
    for (int i = 0; i < 4; ++i) out[i] = c[i];
    return st;
}

}  // namespace xd
