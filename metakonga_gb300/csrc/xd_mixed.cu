// Mixed-precision scene step: exact integer contact decisions, FP32 contact
// forces, FP64 positions, double-float velocities.
//
// GB300 issues about 1.6 FP64 operations per clock per SM against about 117
// FP32 FMAs, so FP64 arithmetic in a per-particle kernel costs ~70 FP32
// operations.  The state is laid out so that the bulk kernels do almost none:
//   positions, radii        FP64 (the FP64 guard-band decisions and the
//                           downloaded state are the uploaded bits)
//   velocities, ang. vel.   double-float hi + lo (two FP32, ~48-bit
//                           significand), updated with FP32 arithmetic
//   accelerations           FP32: the contact part a - g, and alpha
//   1/m, 1/I                FP32 (the FP64 mass, by particle id, serves the
//                           FP64 rechecks, the walls and the download)
// The only FP64 operations per particle and step are the position update
// (two adds per axis) and the fixed-point conversion (one FMA per axis).
//
// Per step (dem_simulation::oneStepAnalysis order, dem_simulation.cpp:447-469):
//   k_mx_advance  the velocity-Verlet update in place (velocity of step t from
//                 the contact force, position of step t + 1), the contact view
//                 -- FP32 (x, y, z, r) and int64 fixed point (2^-36 m) -- and
//                 the skin test: cells are 2 r_max + skin wide and every
//                 particle's Verlet list holds the slots within ri + rj + skin
//                 of it at the list build, so both stay valid while no
//                 particle has moved half the skin since;
//   re-binning    only when one has (a CUDA graph conditional node, or the
//                 host between direct launches): cell keys, stable radix sort,
//                 the state permuted into the new cell order, k_lb_fill
//                 (lb[c] = first slot whose key is >= c, for every cell, so a
//                 row of three cells is the slot range [lb[c0], lb[c0 + 3])),
//                 then k_mx_build: the Verlet lists from the neighbour cells in
//                 the reference's order (rows z then y, slots ascending), the
//                 planes in reach, and the heavy list of the particles with
//                 either;
//   k_mx_contact  for the heavy list only (the others keep zero contact
//                 force): particle pairs over the Verlet list -- FP32
//                 prefilter, then the exact integer test
//                 N = (ri + rj)^2 - |qj - qi|^2 > 0 (no cancellation), pairs
//                 within 2e-10 m of touching decided by the reference's FP64
//                 expression so pair lists equal the FP64 path's, FP32
//                 Hertz-Mindlin (DHSModel) in search order (a pair without slip
//                 reuses the previous pair's tangential force, impl:426-428) --
//                 then the planes in reach in FP64.
// The grid is the scene's own (not the reference's wrapped 128^3): padded by
// one cell on every side, keys clamped inside.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
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
constexpr double kQ = 68719476736.0;           // 2^36 fixed-point units per metre
constexpr float kU = 1.4551915228366852e-11f;  // 2^-36 m
constexpr double kGuard = 2e-10;               // metres: FP64 decision inside this band
constexpr double kMagic = 6755399441055744.0;  // 1.5 * 2^52
constexpr unsigned kVerletCap = 48;            // default: neighbours per particle kept in the Verlet list
constexpr unsigned kTriCap = 16;               // default: triangles per particle kept in its list
constexpr float kSkinFactor = 0.1f;            // default: skin width over the largest radius
constexpr unsigned kContactThreads = 64;       // default block size of the contact pass
constexpr unsigned kContactMaxThreads = 128;   // the largest block size a scene may choose
constexpr unsigned kContactMode = 1;           // default pair pass: warp-cooperative
constexpr unsigned kContactWarpsTotal = 152 * 16;   // warps of a full contact grid (every SM, 16 warps each)
constexpr int kMaxBodies = 8;                  // polygon bodies of a mixed scene
constexpr unsigned kGuardBit = 0x80000000u;    // list entry decided by the FP64 test

// Counter words.
enum {
    CN_REBUILD = 0,    // nonzero: this step re-bins (set by k_mx_advance, cleared by k_mx_contact)
    CN_DONE = 1,       // blocks of k_mx_advance finished (last-block hand-off; reset by the last)
    CN_GAPS = 2,       // long gaps of the cell lower-bound array (re-binning)
    CN_HEAVY = 3,      // particles with Verlet neighbours or planes in reach (since the last build)
    CN_DECISIONS = 4,  // FP64 contact decisions (cumulative)
    CN_NORMALS = 5,    // FP64 normal-force rechecks (cumulative)
    CN_SLIPS = 6,      // FP64 slip rechecks (cumulative)
    CN_REBUILDS = 7,   // re-binnings (cumulative)
    CN_RXN = 8,        // blocks of k_rxn_sum done (the last one finishes the sum)
    CN_HTRI = 9,       // listed particles with walls (planes, triangles) in reach: hlist[0, CN_HTRI)
    CN_HBACK = 10,     // the other listed particles: hlist[n - CN_HBACK, n)
    CN_WALLS = 11,     // wall contacts decided by the FP64 region test (cumulative)
    CN_VINC = 12,      // Verlet lists over their capacity at the last build (the pass searches the cells)
    CN_TINC = 13,      // triangle lists over their capacity at the last build
    CN_VSUM = 14,      // Verlet-list entries at the last build
    CN_TSUM = 15,      // triangle-list entries at the last build
    kCounters = 16
};

struct Master {
    double *x, *y, *z, *r;   // FP64 positions and radii
    float4* vh;              // velocity hi; .w = 1/m
    float4* vl;              // velocity lo; .w unused
    float4* wh;              // angular velocity hi; .w = 1/I
    float4* wl;              // angular velocity lo; .w = particle id (bits)
    float4* ab;              // contact acceleration a - g; .w = alpha.x
    float2* b2;              // alpha.y, alpha.z
};

struct MixParams {
    int gx, gy, gz;
    unsigned n;
    unsigned gxy;        // gx * gy: key offset of one cell in z
    double wo[3];        // grid origin, a multiple of 2^-36 m
    double qoff[3];      // 1.5 * 2^52 - wo * 2^36 (fixed-point offsets)
    double g[3];
    double dt;
    float csf, inv_csf;
    float half_skin;     // a particle keeps its cell while within half the skin of it
    float rmaxf;         // largest radius
    int small_q;         // 2 r_max < 2^-6 m: a touching pair's fixed-point separation and radius sum fit
                         // in 32 bits (their FP32 values then come from 32-bit conversions)
    float vcut;          // Verlet list: pairs within ri + rj + vcut are listed
    float disp2;         // squared displacement that forces re-binning
    float inv_gx, inv_gxy;   // 1 / gx, 1 / (gx gy) for the key decode
    float dtf, hf, half2dtf;
    float gf[3];
    float2 dt_df;        // dt as double-float
    float2 G1[3];        // dt * g, double-float (gravity's velocity increment)
    float2 G2[3];        // dt^2 / 2 * g, double-float
    float tol;           // prefilter tolerance (m)
    float c43Eeq, one_b2, sratio, fric;
    double c43Eeq_d, one_b2_d;   // the same constants in FP64 (rechecks)
    float2 c43Eeq_p, one_b2_p;   // and as float pairs (hi + lo)
    // cohesionForce (impl:259-279): coh and its Eeq = (1 - pri^2)/Ei + (1 - prj^2)/Ej
    float coh, coh_eeq;
    double coh_d, coh_eeq_d;
    long long guard_q;   // guard band in fixed-point units
    int nplanes;
    float pxw[kMaxPlanes][3];   // plane corner relative to the grid origin (FP32)
    float pun[kMaxPlanes][3];   // unit normal (FP32)
    double pl_c43Eeq[kMaxPlanes], pl_one_b2[kMaxPlanes];   // getConstant's pair constants per plane
    double pl_sratio[kMaxPlanes], pl_fric[kMaxPlanes];
    float wall_tol;
    int rolling;         // rollingCondition: rotation terms in the relative velocity
    unsigned ntri, nbodies;
    unsigned vcap, tcap; // Verlet-list and triangle-list capacities per particle
    float tri_reach;     // a triangle is registered in every cell within this of its box
    double pb_c43Eeq[kMaxBodies], pb_one_b2[kMaxBodies];   // getConstant's terms per polygon body
    double pb_sratio[kMaxBodies], pb_fric[kMaxBodies];
};

// Per-plane record of the contact pass (written whenever the planes are
// set): the corner xw and the unit normal uw / |uw| in FP64 (a face contact's
// distance is (x - xw) . n, impl:557-560), and the edge directions and
// lengths in FP32 for the region test.
struct __align__(16) PlaneRec {
    double xw[3];
    double n[3];
    float u1[3], u2[3];
    float l1, l2;
};

}  // namespace

struct MixedScene {
    // n: the particles that take part in a step (P.n); cap: the particles
    // held.  They differ only under an emitter: slots [n, cap) then hold the
    // particles not yet emitted, in id order (no re-binning touches them).
    unsigned n = 0, cap = 0, nplanes = 0, ncell = 0;
    // tuning (xd_scene_set_tuning, before the first upload)
    float skin_factor = kSkinFactor;
    unsigned vcap = kVerletCap, tcap = kTriCap, cthreads = kContactThreads;
    unsigned cmode = kContactMode;   // 0: a thread per listed particle; 1: warp-cooperative pairs
    unsigned active_req = ~0u;    // active count set before the first upload
    bool emitted = false;         // the particle count has changed since the graphs were made
    unsigned version = 0;         // raised whenever the step graphs are dropped (parameters changed)
    int gx = 0, gy = 0, gz = 0;
    double cs = 0.0;
    MixParams P;
    Master m[2];                  // m[0] the state in cell order; m[1] scratch for re-binning
    int cur = 0;
    double* mass0 = nullptr;   // FP64 mass by particle id (rechecks, walls, download)
    // contact view (sorted order)
    float4* pf = nullptr;
    longlong2* qa = nullptr;
    longlong2* qb = nullptr;
    float4* pr = nullptr;         // quantisation residuals of x, y, z and r (metres)
    float4* Fc = nullptr;
    float4* Mc = nullptr;
    // Verlet lists (slots of the current cell order, rebuilt with the cells)
    unsigned* hlist = nullptr;    // particles with neighbours or planes in reach
    unsigned short* wmask = nullptr;   // planes in reach of each particle
    unsigned* vcount = nullptr;   // Verlet neighbours per particle (| kIncomplete: overflow)
    unsigned* vlist = nullptr;    // [vcap][n]: neighbour slots in search order
    float4* pref = nullptr;       // FP32 positions at the last list build
    // triangle meshes (FP64, world frame) and their polygon bodies
    unsigned ntri = 0, nbodies = 0;
    xd_polygon_info* poly = nullptr;
    double* sphere = nullptr;     // circumcentres (written by the mesh update)
    double* vlist_body = nullptr; // body-frame vertices [ntri][9]
    xd_polygon_mass_info* pmi = nullptr;
    float* tri_ref = nullptr;     // vertices at the last build, FP32 relative to the grid origin
    float4* tbound = nullptr;     // bounding sphere of each triangle at the last build (same frame)
    TriRec* trec = nullptr;       // the contact pass's triangle records of the current pose
    unsigned* tcells = nullptr;   // cells per triangle, then their exclusive scan [ntri + 1]
    unsigned* tpk = nullptr;      // (cell, triangle) pairs [tpair_cap]: keys, triangles
    unsigned* tpt = nullptr;
    unsigned tpair_cap = 0;
    void* tsort_scratch = nullptr;
    unsigned* tpk_sorted = nullptr;   // the sort's outputs (fixed for the scene)
    unsigned* tpt_sorted = nullptr;
    unsigned* tcount = nullptr;   // triangles in reach per particle (| kIncomplete: overflow)
    unsigned* tlist = nullptr;    // [tcap][n]: triangle ids in id order
    double* rxn = nullptr;        // reaction on the bodies per particle [nbodies][6][n]
    double* rxn_part = nullptr;   // block partials of its fixed-order sum
    bool bodies_dirty = false;
    bool tri_table_dirty = true;   // the triangles' cell table is to be built before the next step
    std::vector<xd_polygon_info> host_poly;
    std::vector<double> host_sphere, host_vlist;
    std::vector<xd_polygon_mass_info> host_pmi;
    std::vector<xd_contact_property> host_cppoly;
    // grid
    unsigned *keys = nullptr, *vals = nullptr, *prev_keys = nullptr;
    unsigned* lb = nullptr;       // ncell + 1 entries
    uint4* gaps = nullptr;
    unsigned gap_cap = 0;
    bool cells_clean = false;     // prev_keys holds the current order's assigned keys
    void* sort_scratch = nullptr;
    unsigned* perm = nullptr;     // re-binning: new slot -> old slot (the sort's value output)
    unsigned* sorted_keys = nullptr;
    // walls
    xd_plane_info* planes = nullptr;
    PlaneRec* prec = nullptr;     // the contact pass's plane records
    xd_contact_property* cps = nullptr;
    unsigned* counters = nullptr;
    // pair recording
    unsigned* rec_count = nullptr;
    unsigned* rec_pairs = nullptr;
    // host-order transfer buffers
    double* xfer = nullptr;
    bool ready = false;                // grid and buffers set up (first upload)
    cudaGraphExec_t graph[5] = {};   // first step; 1, 2, 4 and 8 middle steps
    // tangential-spring history (an extension): [s * n + slot] tables in the
    // state's slot order, permuted with the particles at re-binning
    unsigned hslots = 0;
    unsigned* hkey = nullptr;
    double* hdelta = nullptr;
    unsigned* hkey2 = nullptr;
    double* hdelta2 = nullptr;
    unsigned long long* hoverflow = nullptr;
    unsigned passes = 0;          // radix passes of one re-binning
    bool use_graphs = true;
    bool kinematic = false;   // bodies moved by their own vel and omega every step
    unsigned rec_cap_alloc = 0;
    xd_scene_desc desc;
    std::vector<xd_plane_info> host_planes;
    std::vector<xd_contact_property> host_cps;
    std::vector<void*> allocs;
    unsigned long long bytes = 0;   // device memory held
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
    s->bytes += sizeof(T) * count;
    *p = static_cast<T*>(q);
    return XD_OK;
}

inline unsigned blocks(unsigned n, unsigned t) { return div_up(n ? n : 1u, t); }

// ---- FP32 helpers ----------------------------------------------------------

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 fk(float x, float y, float z) { return f3{ x, y, z }; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return fk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return fk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return fk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 fadd_rn(f3 a, f3 b)
{
    return fk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
// a x b with every product and difference rounded on its own
__device__ __forceinline__ f3 fcross_rn(f3 a, f3 b)
{
    return fk(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
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
// s + e = a + b exactly for |a| >= |b| (Dekker's FastTwoSum)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// Double-float numbers hi + lo (|lo| <= ulp(hi) / 2): Dekker/Knuth pair
// arithmetic, ~2^-48 relative rounding per operation.
struct dfl {
    float hi, lo;
};
__device__ __forceinline__ dfl df_add(dfl a, dfl b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    dfl r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ dfl df_add_f(dfl a, float b)
{
    float s, e;
    two_sum(a.hi, b, s, e);
    e = __fadd_rn(e, a.lo);
    dfl r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b)
{
    float p, e;
    two_prod(a.hi, b.hi, p, e);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    dfl r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ dfl df_of(float2 v) { return dfl{ v.x, v.y }; }
__device__ __forceinline__ double df_to_d(float hi, float lo) { return (double)hi + (double)lo; }
__host__ inline float2 df_split(double v)
{
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
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
// dq the exact integer separation (|dq| < 2^31), D2 = |dq|^2 exact, D2h its
// FP32 rounding, d0 the FP32 square root of that.  The dot product of a fast
// tangential velocity with the contact normal cancels; here it is carried
// with ~2^-44 relative error and rounded once.
__device__ __forceinline__ float normal_speed(const float s[3], const float t[3], const int dq[3],
                                              float d0, long long D2, float D2h, float& q0_out, float& q1_out,
                                              float& c_out)
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
    // D2h: D2 rounded to FP32 (the caller's, for d0)
    const float D2l = __ll2float_rn(D2 - __float2ll_rn(D2h));
    const float c = __fadd_rn(__fsub_rn(__fsub_rn(D2h, p), pe), D2l) / __fmul_rn(2.f, d0);
    // (nv + nl) / (d0 + c)
    const float q0 = nv / d0;   // any close quotient: its residual is exact below
    float qp, qpe;
    two_prod(q0, d0, qp, qpe);
    const float rem = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(nv, qp), qpe), nl), __fmul_rn(q0, c));
    q0_out = q0;
    q1_out = rem / d0;
    c_out = c;
    return __fadd_rn(q0, q1_out);
}

// ---- pair arithmetic for the rolling slip ---------------------------------

__device__ __forceinline__ dfl df_make(float a, float b)
{
    dfl r;
    two_sum(a, b, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ dfl df_neg(dfl a) { return dfl{ -a.hi, -a.lo }; }
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

// 1 / (d0 + c) as a pair: r0 = 1 / d0 refined by one Newton step (the
// residual 1 - d0 r0 of a rounded reciprocal is exact in one FMA).
__device__ __forceinline__ dfl df_inv(float d0, float c)
{
    const float r0 = 1.0f / d0;   // refined by the Newton step
    const float res = __fsub_rn(__fmaf_rn(-d0, r0, 1.0f), __fmul_rn(c, r0));
    dfl r;
    fast_two_sum(r0, __fmul_rn(r0, res), r.hi, r.lo);
    return r;
}

// A fixed-point length (units of 2^-36 m, |q| < 2^44) as an exact pair.
__device__ __forceinline__ dfl q_to_df(long long q)
{
    return df_make(__fmul_rn(__int2float_rn((int)(q >> 20)), 0x1p-16f),
                   __fmul_rn(__int2float_rn((int)(q & 0xfffff)), 0x1p-36f));
}

// The slip e = rv - (rv . u) u of a pair in pair arithmetic (about 2^-44 of
// its terms), rounded once: rv = dv - W x u with W = rj wj + ri wi
// (impl:455), dv = s + t exact, u = dq / |dq| from the exact integer
// separation (|dq| = d0 + c), the radii from their fixed-point values, the
// angular velocities from their hi/lo pairs, and the normal speed q0 + q1.
// Used where the FP32 rotation term's rounding could matter (rolling).
__device__ __noinline__ f3 slip_pair(const float s[3], const float t[3], const int dq[3], float d0, float c,
                                     float q0, float q1, long long qri, long long qrj, float4 wih, float4 wil,
                                     float4 wjh, float4 wjl)
{
    const dfl inv = df_inv(d0, c);
    dfl u[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float qh = __int2float_rn(dq[k]);
        const float ql = __int2float_rn(dq[k] - __float2int_rn(qh));
        u[k] = df_mul(df_make(qh, ql), inv);
    }
    const dfl ri = q_to_df(qri), rj = q_to_df(qrj);
    const dfl W[3] = { df_add(df_mul(rj, dfl{ wjh.x, wjl.x }), df_mul(ri, dfl{ wih.x, wil.x })),
                       df_add(df_mul(rj, dfl{ wjh.y, wjl.y }), df_mul(ri, dfl{ wih.y, wil.y })),
                       df_add(df_mul(rj, dfl{ wjh.z, wjl.z }), df_mul(ri, dfl{ wih.z, wil.z })) };
    const dfl wu[3] = { df_sub(df_mul(W[1], u[2]), df_mul(W[2], u[1])),
                        df_sub(df_mul(W[2], u[0]), df_mul(W[0], u[2])),
                        df_sub(df_mul(W[0], u[1]), df_mul(W[1], u[0])) };
    const dfl rvu = df_make(q0, q1);
    float e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const dfl v = df_sub(df_sub(df_make(s[k], t[k]), wu[k]), df_mul(rvu, u[k]));
        e[k] = __fadd_rn(v.hi, v.lo);
    }
    return fk(e[0], e[1], e[2]);
}

// a / b and sqrt(a) in pair arithmetic (one correction step each).  This
// file is compiled with approximate FP32 division and square root
// (-prec-div=false -prec-sqrt=false, about 2 ulp): every quotient and root
// in the pair helpers is a first guess whose residual is formed exactly and
// corrected, and the plain FP32 force terms carry error bounds (kTermErr,
// kRotErr) well above that.
__device__ __forceinline__ dfl df_div(dfl a, dfl b)
{
    const float q1 = a.hi / b.hi;
    const dfl r = df_sub(a, df_mul(b, dfl{ q1, 0.f }));
    dfl q;
    fast_two_sum(q1, r.hi / b.hi, q.hi, q.lo);
    return q;
}
__device__ __forceinline__ dfl df_sqrt(dfl a)
{
    if (!(a.hi > 0.f)) return dfl{ 0.f, 0.f };
    const float s0 = sqrtf(a.hi);
    float p, pe;
    two_prod(s0, s0, p, pe);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
    dfl q;
    fast_two_sum(s0, r / __fmul_rn(2.f, s0), q.hi, q.lo);
    return q;
}
// an FP64 value as a float pair
__device__ __forceinline__ dfl d_to_df(double x)
{
    const float h = __double2float_rn(x);
    return dfl{ h, __double2float_rn(x - (double)h) };
}

// The normal force -kn d^1.5 + vn (dv . u) of pair (i, j) in pair arithmetic
// (about 2^-44 of its terms), for contacts whose FP32 terms nearly cancel:
// the overlap (ri + rj) - |xj - xi| from the FP64 positions and radii (the
// reference's expression, impl:449-452), getConstant's Req and Meq from the
// FP64 radii and masses (impl:238-246), the normal speed q0 + q1.  No
// cohesion (the cohesive recheck is FP64).
__device__ __noinline__ float normal_pair(const MixParams& P, const Master& M, const double* __restrict__ mass0,
                                          unsigned i, unsigned j, unsigned idi, unsigned idj, float q0, float q1)
{
    const dfl X = d_to_df(__ldg(M.x + j) - __ldg(M.x + i));
    const dfl Y = d_to_df(__ldg(M.y + j) - __ldg(M.y + i));
    const dfl Z = d_to_df(__ldg(M.z + j) - __ldg(M.z + i));
    const dfl d = df_sqrt(df_add(df_add(df_mul(X, X), df_mul(Y, Y)), df_mul(Z, Z)));
    const dfl ri = d_to_df(__ldg(M.r + i)), rj = d_to_df(__ldg(M.r + j));
    const dfl rs = df_add(ri, rj);
    const dfl delta = df_sub(rs, d);
    const dfl mi = d_to_df(__ldg(mass0 + idi)), mj = d_to_df(__ldg(mass0 + idj));
    const dfl Req = df_div(df_mul(ri, rj), rs);
    const dfl Meq = df_div(df_mul(mi, mj), df_add(mi, mj));
    const dfl kn = df_mul(df_of(P.c43Eeq_p), df_sqrt(Req));
    const dfl vn = df_sqrt(df_div(df_mul(df_mul(dfl{ 4.f, 0.f }, Meq), kn), df_of(P.one_b2_p)));
    const dfl fsn = df_neg(df_mul(kn, df_mul(delta, df_sqrt(delta))));
    const dfl fn = df_add(fsn, df_mul(vn, df_make(q0, q1)));
    return __fadd_rn(fn.hi, fn.lo);
}

// ---- fixed point and the contact view --------------------------------------

// round((x - wo) * 2^36), ties to even, in one FMA: x * 2^36 + (1.5 * 2^52 -
// wo * 2^36) lies in [2^52, 2^53), where FP64 numbers are spaced 1 apart, so
// the rounded sum's low bits are the integer.  Needs |x - wo| < 2^15 m.
__device__ __forceinline__ long long fixed_q(double x, double off)
{
    return __double_as_longlong(__fma_rn(x, kQ, off)) - __double_as_longlong(kMagic);
}

// FP32 value of a fixed-point coordinate (|q| < 2^51), from two exact 32-bit
// conversions (the 64-bit integer conversions run on the FP64 pipe).
__device__ __forceinline__ float q_to_f(long long q)
{
    return __fmaf_rn(__int2float_rn((int)(q >> 20)), 0x1p-16f,
                     __fmul_rn(__int2float_rn((int)(q & 0xfffff)), 0x1p-36f));
}

// The quantisation residual x - (wo + q 2^-36) in metres of a fixed-point
// coordinate formed as t = fma(x, 2^36, off): the FMA's rounding error,
// recovered by a second FMA (off - t is exact: both lie in [2^52, 2^53)).
__device__ __forceinline__ float fixed_residual(double x, double off, long long q)
{
    const double t = __longlong_as_double(q + __double_as_longlong(kMagic));
    return (float)__fma_rn(x, kQ, off - t) * 0x1p-36f;
}

// The contact view of slot i: FP32 position and radius (pf), the int64 fixed
// point (qa, qb) that decides contacts exactly, and the residuals of the
// fixed point (pr) that restore the FP64 positions' overlap and normal to
// about 1e-18 m in the force.
__device__ __forceinline__ float4 write_view(const MixParams& P, unsigned i, double x, double y,
                                             double z, double r, float4* __restrict__ pf,
                                             longlong2* __restrict__ qa, longlong2* __restrict__ qb,
                                             float4* __restrict__ pr)
{
    const long long qx = fixed_q(x, P.qoff[0]), qy = fixed_q(y, P.qoff[1]), qz = fixed_q(z, P.qoff[2]);
    const long long qr = fixed_q(r, kMagic);
    qa[i] = make_longlong2(qx, qy);
    qb[i] = make_longlong2(qz, qr);
    pr[i] = make_float4(fixed_residual(x, P.qoff[0], qx), fixed_residual(y, P.qoff[1], qy),
                        fixed_residual(z, P.qoff[2], qz), fixed_residual(r, kMagic, qr));
    const float4 v = make_float4(q_to_f(qx), q_to_f(qy), q_to_f(qz), (float)r);
    pf[i] = v;
    return v;
}

// Planes within reach of a particle: FP32 distance to each plane's supporting
// plane against r + pad (the finite plane is never nearer).
__device__ __forceinline__ unsigned near_planes(const MixParams& P, const float4& p, float pad)
{
    unsigned mask = 0;
    for (int w = 0; w < P.nplanes; ++w) {
        const float hz = (p.x - P.pxw[w][0]) * P.pun[w][0] + (p.y - P.pxw[w][1]) * P.pun[w][1] +
                         (p.z - P.pxw[w][2]) * P.pun[w][2];
        if (fabsf(hz) < p.w + pad) mask |= 1u << w;
    }
    return mask;
}

// Cell key of a position relative to the grid origin (FP32).  Interior cells
// only: keys are clamped to [1, g - 2] on every axis.
__device__ __forceinline__ unsigned cell_key(const MixParams& P, float x, float y, float z)
{
    int cx = (int)floorf(x * P.inv_csf) + 1;
    int cy = (int)floorf(y * P.inv_csf) + 1;
    int cz = (int)floorf(z * P.inv_csf) + 1;
    cx = min(max(cx, 1), P.gx - 2);
    cy = min(max(cy, 1), P.gy - 2);
    cz = min(max(cz, 1), P.gz - 2);
    return ((unsigned)cz * (unsigned)P.gy + (unsigned)cy) * (unsigned)P.gx + (unsigned)cx;
}

// Appends v to list (counter *cnt) for the lanes where take is set, one
// atomic per warp.  Every lane of the warp calls it.
template <typename T>
__device__ __forceinline__ void warp_append(bool take, const T& v, T* __restrict__ list,
                                            unsigned* __restrict__ cnt)
{
    const unsigned bal = __ballot_sync(0xffffffffu, take);
    if (!bal) return;
    const unsigned lane = threadIdx.x & 31u;
    const int leader = __ffs(bal) - 1;
    unsigned base = 0;
    if ((int)lane == leader) base = atomicAdd(cnt, (unsigned)__popc(bal));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) list[base + __popc(bal & ((1u << lane) - 1u))] = v;
}

// Adds one to a diagnostic counter for each lane that calls it, one atomic
// per group of converged lanes (a shared address would otherwise serialise
// every lane's increment).
__device__ __forceinline__ void count_one(unsigned* c)
{
    const unsigned m = __activemask();
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(c, (unsigned)__popc(m));
}

// Adds v of each converged lane to a diagnostic counter, one atomic per group.
__device__ __forceinline__ void count_add(unsigned* c, unsigned v)
{
    const unsigned m = __activemask();
    const unsigned t = __reduce_add_sync(m, v);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1) && t) atomicAdd(c, t);
}

// ---- integration -----------------------------------------------------------
//
// Velocity Verlet as the reference splits it (vv_update_position_kernel
// impl:85-96, vv_update_velocity_kernel impl:117-133), with a = g + F / m:
//   MODE 0  position of step t + 1 from (v, a) of step t (first step of a call)
//   MODE 1  velocity of step t from the step's contact force, then the
//           position of step t + 1
//   MODE 2  velocity only (last step of a call)
//   MODE 3  no update (contacts of the current state)

// Cell coordinates of a key: FP32 reciprocal estimates, each off by at most
// one (the quotient is below 2^16), then corrected.
__device__ __forceinline__ void decode_key(const MixParams& P, unsigned key, unsigned& cx, unsigned& cy,
                                           unsigned& cz)
{
    cz = (unsigned)((float)key * P.inv_gxy);
    if (cz * P.gxy > key) --cz;
    else if ((cz + 1u) * P.gxy <= key) ++cz;
    const unsigned rem = key - cz * P.gxy;
    cy = (unsigned)((float)rem * P.inv_gx);
    if (cy * (unsigned)P.gx > rem) --cy;
    else if ((cy + 1u) * (unsigned)P.gx <= rem) ++cy;
    cx = rem - cy * (unsigned)P.gx;
}

// Velocity update of one particle (MODE 1 and 2): v += dt g + h (a_c + a_c'),
// w += h (alpha + alpha'), with a_c' = F / m and alpha' = M / I.
__device__ __forceinline__ void kick(const MixParams& P, float4& vh, float4& vl, float4& wh,
                                     float4& wl, float4& ab, float2& b2, const float4& f,
                                     const float4& t)
{
    const float im = vh.w, iI = wh.w;
    const float ax = f.x * im, ay = f.y * im, az = f.z * im;
    const float bx = t.x * iI, by = t.y * iI, bz = t.z * iI;
    dfl v;
    v = df_add_f(df_add(dfl{ vh.x, vl.x }, df_of(P.G1[0])), P.hf * (ab.x + ax));
    vh.x = v.hi; vl.x = v.lo;
    v = df_add_f(df_add(dfl{ vh.y, vl.y }, df_of(P.G1[1])), P.hf * (ab.y + ay));
    vh.y = v.hi; vl.y = v.lo;
    v = df_add_f(df_add(dfl{ vh.z, vl.z }, df_of(P.G1[2])), P.hf * (ab.z + az));
    vh.z = v.hi; vl.z = v.lo;
    v = df_add_f(dfl{ wh.x, wl.x }, P.hf * (ab.w + bx));
    wh.x = v.hi; wl.x = v.lo;
    v = df_add_f(dfl{ wh.y, wl.y }, P.hf * (b2.x + by));
    wh.y = v.hi; wl.y = v.lo;
    v = df_add_f(dfl{ wh.z, wl.z }, P.hf * (b2.y + bz));
    wh.z = v.hi; wl.z = v.lo;
    ab = make_float4(ax, ay, az, bx);
    b2 = make_float2(by, bz);
}

// x += dt v + dt^2/2 (g + a_c): the increment in double-float, added in FP64.
__device__ __forceinline__ double drift(const MixParams& P, double x, float vhi, float vlo, int k,
                                        float ac)
{
    dfl inc = df_mul(df_of(P.dt_df), dfl{ vhi, vlo });
    inc = df_add(inc, df_of(P.G2[k]));
    inc = df_add_f(inc, P.half2dtf * ac);
    return __dadd_rn(x, __dadd_rn((double)inc.hi, (double)inc.lo));
}

// k_mx_advance: one step of the state in place (MODE as above), the contact
// view, then the skin test on the new position: every particle must stay
// within half the skin of its position at the last list build (pref); one
// that does not sets CN_REBUILD.  The last block to finish passes the flag to
// the graph's conditional node (use_cond), one caller as the conditional
// requires.
// One slot of the advance (MODE 0: drift; MODE 1: kick with the last
// contact forces, then drift), its contact view, and whether it has left half
// the skin since the last build.
template <int MODE>
__device__ __forceinline__ bool advance_one(const MixParams& P, const Master& M, const float4* __restrict__ Fc,
                                            const float4* __restrict__ Mc, const float4* __restrict__ pref,
                                            float4* __restrict__ pf, longlong2* __restrict__ qa,
                                            longlong2* __restrict__ qb, float4* __restrict__ pr,
                                            const unsigned i)
{
    double x = M.x[i], y = M.y[i], z = M.z[i];
    const double r = M.r[i];
    if (MODE == 0 || MODE == 1) {
        float4 vh = M.vh[i], vl = M.vl[i], ab = M.ab[i];
        if (MODE == 1) {
            float4 wh = M.wh[i], wl = M.wl[i];
            float2 b2 = M.b2[i];
            kick(P, vh, vl, wh, wl, ab, b2, Fc[i], Mc[i]);
            M.vh[i] = vh;
            M.vl[i] = vl;
            M.wh[i] = wh;
            M.wl[i] = wl;
            M.ab[i] = ab;
            M.b2[i] = b2;
        }
        x = drift(P, x, vh.x, vl.x, 0, ab.x);
        y = drift(P, y, vh.y, vl.y, 1, ab.y);
        z = drift(P, z, vh.z, vl.z, 2, ab.z);
        M.x[i] = x;
        M.y[i] = y;
        M.z[i] = z;
    }
    const float4 v = write_view(P, i, x, y, z, r, pf, qa, qb, pr);
    const float4 r0 = pref[i];
    const float dx = v.x - r0.x, dy = v.y - r0.y, dz = v.z - r0.z;
    return !(dx * dx + dy * dy + dz * dz < P.disp2);
}

template <int MODE>
__global__ void __launch_bounds__(256) k_mx_advance(MixParams P, Master M, const float4* __restrict__ Fc,
                                                    const float4* __restrict__ Mc,
                                                    const float4* __restrict__ pref,
                                                    float4* __restrict__ pf, longlong2* __restrict__ qa,
                                                    longlong2* __restrict__ qb, float4* __restrict__ pr,
                                                    unsigned* __restrict__ counters,
                                                    cudaGraphConditionalHandle cond, int use_cond)
{
    __shared__ bool last;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool out = i < P.n && advance_one<MODE>(P, M, Fc, Mc, pref, pf, qa, qb, pr, i);
    // only the flag must be visible to the last block: the lanes that set it
    // fence; the state and view writes need no ordering here
    if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31u) == 0) {
        atomicOr(counters + CN_REBUILD, 1u);
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counters + CN_DONE, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const unsigned f = atomicOr(counters + CN_REBUILD, 0u) ? 1u : 0u;
        // the handle's default (0, assigned at every graph launch) stands
        // unless a re-binning is due
        if (use_cond && f) cudaGraphSetConditional(cond, 1u);
        counters[CN_DONE] = 0;
    }
}

// Re-binning, 1: the cell key of every slot's current position.
__global__ void __launch_bounds__(256) k_mx_keys(MixParams P, const float4* __restrict__ pf,
                                                 unsigned* __restrict__ keys, unsigned* __restrict__ vals)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const float4 p = pf[i];
    keys[i] = cell_key(P, p.x, p.y, p.z);
    vals[i] = i;
}

// Re-binning, 2: the state in the new order (perm: new slot -> old slot) into D.
__global__ void __launch_bounds__(256) k_mx_permute(MixParams P, Master S, Master D,
                                                    const unsigned* __restrict__ perm)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const unsigned o = __ldg(perm + i);
    D.x[i] = __ldg(S.x + o);
    D.y[i] = __ldg(S.y + o);
    D.z[i] = __ldg(S.z + o);
    D.r[i] = __ldg(S.r + o);
    D.vh[i] = __ldg(S.vh + o);
    D.vl[i] = __ldg(S.vl + o);
    D.wh[i] = __ldg(S.wh + o);
    D.wl[i] = __ldg(S.wl + o);
    D.ab[i] = __ldg(S.ab + o);
    D.b2[i] = __ldg(S.b2 + o);
}

// Re-binning, 3: back into the state arrays, with the contact view.
__global__ void __launch_bounds__(256) k_mx_copyback(MixParams P, Master S, Master D,
                                                     float4* __restrict__ pf, longlong2* __restrict__ qa,
                                                     longlong2* __restrict__ qb, float4* __restrict__ pr)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const double x = S.x[i], y = S.y[i], z = S.z[i], r = S.r[i];
    D.x[i] = x;
    D.y[i] = y;
    D.z[i] = z;
    D.r[i] = r;
    D.vh[i] = S.vh[i];
    D.vl[i] = S.vl[i];
    D.wh[i] = S.wh[i];
    D.wl[i] = S.wl[i];
    D.ab[i] = S.ab[i];
    D.b2[i] = S.b2[i];
    write_view(P, i, x, y, z, r, pf, qa, qb, pr);
}

// MODE 2: velocity only, in place (the last step of a call).
__device__ __forceinline__ void finish_one(const MixParams& P, const Master& M, const float4* __restrict__ Fc,
                                           const float4* __restrict__ Mc, const unsigned i)
{
    float4 vh = M.vh[i], vl = M.vl[i], wh = M.wh[i], wl = M.wl[i], ab = M.ab[i];
    float2 b2 = M.b2[i];
    kick(P, vh, vl, wh, wl, ab, b2, Fc[i], Mc[i]);
    M.vh[i] = vh;
    M.vl[i] = vl;
    M.wh[i] = wh;
    M.wl[i] = wl;
    M.ab[i] = ab;
    M.b2[i] = b2;
}

__global__ void __launch_bounds__(256) k_mx_finish(MixParams P, Master M, const float4* __restrict__ Fc,
                                                   const float4* __restrict__ Mc)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.n) finish_one(P, M, Fc, Mc, i);
}

// ---- cell lower bounds -----------------------------------------------------
//
// lb[c] for c in (sk[t-1], sk[t]] is t (lb[0..sk[0]] = 0, lb(sk[n-1]..ncell] = n).
// Each slot fills the gap of empty cells before its own: short gaps by the
// thread, medium ones by its warp, long ones by every block (k_lb_long).
constexpr unsigned kGapThread = 16, kGapWarp = 4096;

__global__ void __launch_bounds__(256) k_lb_fill(const unsigned* __restrict__ sk, unsigned n,
                                                 unsigned ncell, unsigned* __restrict__ lb,
                                                 unsigned* __restrict__ prev,
                                                 uint4* __restrict__ gaps,
                                                 unsigned* __restrict__ counters)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;   // slots 0 .. n
    const unsigned lane = threadIdx.x & 31u;
    if (t == 0) atomicAdd(counters + CN_REBUILDS, 1u);
    unsigned lo = 1, hi = 0;
    if (t <= n) {
        const unsigned kc = t < n ? sk[t] : ncell;
        if (t < n) prev[t] = kc;
        lo = t == 0 ? 0u : sk[t - 1] + 1u;
        hi = kc;
    }
    const unsigned len = hi >= lo ? hi - lo + 1u : 0u;
    if (len && len <= kGapThread)
        for (unsigned c = lo; c <= hi; ++c) lb[c] = t;
    unsigned pend = __ballot_sync(0xffffffffu, len > kGapThread && len <= kGapWarp);
    while (pend) {
        const int src = __ffs(pend) - 1;
        const unsigned glo = __shfl_sync(0xffffffffu, lo, src);
        const unsigned ghi = __shfl_sync(0xffffffffu, hi, src);
        const unsigned gv = __shfl_sync(0xffffffffu, t, src);
        for (unsigned c = glo + lane; c <= ghi; c += 32) lb[c] = gv;
        pend &= pend - 1u;
    }
    if (len > kGapWarp) gaps[atomicAdd(counters + CN_GAPS, 1u)] = make_uint4(lo, hi, t, 0u);
}

__global__ void __launch_bounds__(256) k_lb_long(const uint4* __restrict__ gaps,
                                                 const unsigned* __restrict__ counters,
                                                 unsigned* __restrict__ lb)
{
    const unsigned m = counters[CN_GAPS];
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned g = 0; g < m; ++g) {
        const uint4 G = gaps[g];
        for (unsigned c = G.x + blockIdx.x * blockDim.x + threadIdx.x; c <= G.y; c += stride) lb[c] = G.z;
    }
}

// ---- contacts --------------------------------------------------------------

// Reference FP64 contact decision (calculate_p2p_kernel, impl:449-452),
// evaluated without multiply-add contraction like the oracle.
__device__ __noinline__ double fp64_cdist(const Master& M, unsigned i, unsigned j)
{
    double dx = __dsub_rn(__ldg(M.x + j), __ldg(M.x + i));
    double dy = __dsub_rn(__ldg(M.y + j), __ldg(M.y + i));
    double dz = __dsub_rn(__ldg(M.z + j), __ldg(M.z + i));
    double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return __dsub_rn(__dadd_rn(__ldg(M.r + i), __ldg(M.r + j)), __dsqrt_rn(d2));
}

// The exact test of a candidate pair that passed the FP32 prefilter: the
// integer separation against the radii, and the FP64 guard band.  Returns 0
// (no contact), 1 (contact) or 2 (contact decided by the FP64 test).
template <bool COUNT>
__device__ __forceinline__ int exact_touch_q(const MixParams& P, const Master& M, unsigned i, unsigned j,
                                             const longlong2& qai, const longlong2& qbi, const longlong2& qaj,
                                             const longlong2& qbj, unsigned* __restrict__ counters)
{
    const long long ddx = qaj.x - qai.x, ddy = qaj.y - qai.y, ddz = qbj.x - qbi.x;
    const long long Rq = qbi.y + qbj.y;
    const long long N = Rq * Rq - (ddx * ddx + ddy * ddy + ddz * ddz);
    const long long band = 2 * Rq * P.guard_q;
    if (N > band) return 1;
    if (N < -band) return 0;
    if (COUNT) count_one(counters + CN_DECISIONS);
    return fp64_cdist(M, i, j) > 0 ? 2 : 0;
}

template <bool COUNT>
__device__ __forceinline__ int exact_touch(const MixParams& P, const Master& M, unsigned i, unsigned j,
                                           const longlong2& qai, const longlong2& qbi,
                                           const longlong2* __restrict__ qa,
                                           const longlong2* __restrict__ qb,
                                           unsigned* __restrict__ counters)
{
    return exact_touch_q<COUNT>(P, M, i, j, qai, qbi, __ldg(qa + j), __ldg(qb + j), counters);
}

// The candidate test of pair (i, j): FP32 prefilter, then the exact test.
template <bool COUNT>
__device__ __forceinline__ int touch(const MixParams& P, const Master& M, unsigned i, unsigned j,
                                     const float4& pi, const longlong2& qai, const longlong2& qbi,
                                     const float4* __restrict__ pf, const longlong2* __restrict__ qa,
                                     const longlong2* __restrict__ qb, unsigned* __restrict__ counters)
{
    const float4 pj = __ldg(pf + j);
    const float dxf = pj.x - pi.x, dyf = pj.y - pi.y, dzf = pj.z - pi.z;
    const float Rt = pi.w + P.tol + pj.w;
    if (fmaf(dxf, dxf, fmaf(dyf, dyf, dzf * dzf)) >= Rt * Rt) return 0;
    return exact_touch<COUNT>(P, M, i, j, qai, qbi, qa, qb, counters);
}

// Visits the contacts of slot i in the reference's order (neighbour rows z
// then y, each row's slots ascending): fn(j, guard) for every touching j.
// Candidates pass an FP32 prefilter, then the exact integer test; pairs in
// the guard band are decided by fp64_cdist.
template <bool COUNT, typename Fn>
__device__ __forceinline__ void for_each_contact(const MixParams& P, const Master& M, unsigned i,
                                                 const float4& pi, const longlong2& qai,
                                                 const longlong2& qbi, unsigned key,
                                                 const float4* __restrict__ pf,
                                                 const longlong2* __restrict__ qa,
                                                 const longlong2* __restrict__ qb,
                                                 const unsigned* __restrict__ lb,
                                                 unsigned* __restrict__ counters, Fn fn)
{
    // row (dz, dy) starts at cell key - 1 + dy gx + dz gx gy; the next row's
    // bounds are loaded while this row's candidates are visited
    unsigned c0 = key - 1u - (unsigned)P.gx - P.gxy;
    unsigned s = __ldg(lb + c0), e = __ldg(lb + c0 + 3);
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        const unsigned c1 = (r % 3 == 2) ? c0 - 2u * (unsigned)P.gx + P.gxy : c0 + (unsigned)P.gx;
        unsigned sn = 0, en = 0;
        if (r < 8) {
            sn = __ldg(lb + c1);
            en = __ldg(lb + c1 + 3);
        }
        for (unsigned j = s; j < e; ++j) {
            if (j == i) continue;
            const int t = touch<COUNT>(P, M, i, j, pi, qai, qbi, pf, qa, qb, counters);
            if (t) fn(j, t == 2);
        }
        s = sn;
        e = en;
        c0 = c1;
    }
}

constexpr unsigned kIncomplete = 0x80000000u;   // vcount flag: the list is not complete

// ---- triangle meshes ---------------------------------------------------------
//
// At a re-binning every triangle is registered in each cell that its
// bounding box, widened by the reach of the largest particle, overlaps;
// each particle then lists the triangles of its cell whose closest point is
// within r + skin (FP64), in triangle-id order.  Meshes move only between
// calls (xd_scene_set_bodies); the mesh update then compares the vertices
// with those of the last build and raises CN_REBUILD past half the skin.

// The interior cells a triangle's widened bounding box covers, and its
// vertices in FP32 relative to the grid origin.
__device__ __forceinline__ void tri_box(const MixParams& P, const xd_polygon_info* __restrict__ t,
                                        int lo[3], int hi[3], float v[9])
{
    const double* V[3] = { t->P, t->Q, t->R };
    const int g[3] = { P.gx, P.gy, P.gz };
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float mn = 3.0e38f, mx = -3.0e38f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float c = (float)(__ldg(V[k] + a) - P.wo[a]);
            v[3 * k + a] = c;
            mn = fminf(mn, c);
            mx = fmaxf(mx, c);
        }
        lo[a] = min(max((int)floorf((mn - P.tri_reach) * P.inv_csf) + 1, 1), g[a] - 2);
        hi[a] = min(max((int)floorf((mx + P.tri_reach) * P.inv_csf) + 1, 1), g[a] - 2);
    }
}

// Cells per triangle (tcells[ntri] = 0 for the scan) and the build vertices.
__global__ void __launch_bounds__(256) k_tri_count(MixParams P, const xd_polygon_info* __restrict__ poly,
                                                   unsigned* __restrict__ tcells,
                                                   float* __restrict__ tri_ref, float4* __restrict__ tbound)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > P.ntri) return;
    if (t == P.ntri) {
        tcells[t] = 0;
        return;
    }
    int lo[3], hi[3];
    float v[9];
    tri_box(P, poly + t, lo, hi, v);
    for (int k = 0; k < 9; ++k) tri_ref[9 * (size_t)t + k] = v[k];
    // bounding sphere for the list build: centroid and farthest vertex
    const float gx = (v[0] + v[3] + v[6]) * (1.f / 3.f), gy = (v[1] + v[4] + v[7]) * (1.f / 3.f),
                gz = (v[2] + v[5] + v[8]) * (1.f / 3.f);
    float rb = 0.f;
    for (int k = 0; k < 3; ++k) {
        const float dx = v[3 * k] - gx, dy = v[3 * k + 1] - gy, dz = v[3 * k + 2] - gz;
        rb = fmaxf(rb, sqrtf(dx * dx + dy * dy + dz * dz));
    }
    tbound[t] = make_float4(gx, gy, gz, rb);
    tcells[t] = (unsigned)((hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1));
}

// In-place exclusive scan of m values, one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan1(unsigned* __restrict__ a, unsigned m)
{
    __shared__ unsigned wsum[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (unsigned b0 = 0; b0 < m; b0 += 1024) {
        const unsigned i = b0 + threadIdx.x;
        const unsigned v = i < m ? a[i] : 0u;
        unsigned x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (unsigned)o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            const unsigned w = wsum[lane];
            unsigned t = w;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= (unsigned)o) t += y;
            }
            wsum[lane] = t - w;
        }
        __syncthreads();
        const unsigned excl = x - v + wsum[warp] + carry;
        if (i < m) a[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
}

// The (cell key, triangle) pairs, cells in key order per triangle.
__global__ void __launch_bounds__(256) k_tri_fill(MixParams P, const xd_polygon_info* __restrict__ poly,
                                                  const unsigned* __restrict__ toff, unsigned cap,
                                                  unsigned* __restrict__ tpk, unsigned* __restrict__ tpt)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.ntri) return;
    int lo[3], hi[3];
    float v[9];
    tri_box(P, poly + t, lo, hi, v);
    unsigned k = toff[t];
    for (int z = lo[2]; z <= hi[2]; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x, ++k)
                if (k < cap) {
                    tpk[k] = ((unsigned)z * (unsigned)P.gy + (unsigned)y) * (unsigned)P.gx + (unsigned)x;
                    tpt[k] = t;
                }
}

// Unused pair slots sort to the end (key = ncell, past every cell).
__global__ void __launch_bounds__(256) k_tri_pad(const unsigned* __restrict__ toff, unsigned ntri,
                                                 unsigned cap, unsigned ncell, unsigned* __restrict__ tpk,
                                                 unsigned* __restrict__ tpt)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap || i < toff[ntri]) return;
    tpk[i] = ncell;
    tpt[i] = 0;
}

// First index in a[0, m) with a[idx] >= v.
__device__ __forceinline__ unsigned lower_bound_u(const unsigned* __restrict__ a, unsigned m, unsigned v)
{
    unsigned lo = 0, hi = m;
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ d3 tri_vertex(const double* v) { return mk(__ldg(v), __ldg(v + 1), __ldg(v + 2)); }

// Squared distance from the origin to triangle abc in FP32 (the closest-point
// regions of Ericson, Real-Time Collision Detection 5.1.5, with the query
// point at the origin).  The distance is continuous across the regions, so a
// region misjudged by rounding moves it by rounding only.  face: the closest
// point is inside the face with every barycentric coordinate above 1e-5, far
// beyond the FP32 rounding, so the FP64 region test of the reference takes its
// face branch as well.
__device__ __forceinline__ float tri_dist2_f(float ax, float ay, float az, float bx, float by, float bz, float cx,
                                             float cy, float cz, bool& face)
{
    face = false;
    const float abx = bx - ax, aby = by - ay, abz = bz - az;
    const float acx = cx - ax, acy = cy - ay, acz = cz - az;
    const float d1 = -(abx * ax + aby * ay + abz * az), d2 = -(acx * ax + acy * ay + acz * az);
    if (d1 <= 0.f && d2 <= 0.f) return ax * ax + ay * ay + az * az;
    const float d3 = -(abx * bx + aby * by + abz * bz), d4 = -(acx * bx + acy * by + acz * bz);
    if (d3 >= 0.f && d4 <= d3) return bx * bx + by * by + bz * bz;
    const float vc = d1 * d4 - d3 * d2;
    float qx, qy, qz;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
        const float v = d1 / (d1 - d3);
        qx = ax + v * abx;
        qy = ay + v * aby;
        qz = az + v * abz;
        return qx * qx + qy * qy + qz * qz;
    }
    const float d5 = -(abx * cx + aby * cy + abz * cz), d6 = -(acx * cx + acy * cy + acz * cz);
    if (d6 >= 0.f && d5 <= d6) return cx * cx + cy * cy + cz * cz;
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
        const float w = d2 / (d2 - d6);
        qx = ax + w * acx;
        qy = ay + w * acy;
        qz = az + w * acz;
        return qx * qx + qy * qy + qz * qz;
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
        const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        qx = bx + w * (cx - bx);
        qy = by + w * (cy - by);
        qz = bz + w * (cz - bz);
        return qx * qx + qy * qy + qz * qz;
    }
    const float den = 1.f / (va + vb + vc);
    const float v = vb * den, w = vc * den;
    face = va * den > 1e-5f && v > 1e-5f && w > 1e-5f;
    qx = ax + v * abx + w * acx;
    qy = ay + v * aby + w * acy;
    qz = az + v * abz + w * acz;
    return qx * qx + qy * qy + qz * qz;
}

// Per particle: the triangles of its cell within r + skin, in id order.  The
// test is FP32 (vertices and centre relative to the grid origin, rounded
// within about 1e-7 m) with a 1e-5 m margin: a list may hold a triangle just
// out of reach (the contact pass decides each contact exactly), never miss
// one within it.
__global__ void __launch_bounds__(256) k_tri_build(MixParams P, const float4* __restrict__ pf,
                                                   const unsigned* __restrict__ keys,
                                                   const unsigned* __restrict__ tpk,
                                                   const unsigned* __restrict__ tpt, unsigned cap,
                                                   const float* __restrict__ tri_ref,
                                                   const float4* __restrict__ tbound,
                                                   unsigned* __restrict__ tcount, unsigned* __restrict__ tlist,
                                                   unsigned* __restrict__ counters)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const unsigned key = __ldg(keys + i);
    const unsigned b = lower_bound_u(tpk, cap, key), e = lower_bound_u(tpk, cap, key + 1u);
    const float4 p = __ldg(pf + i);
    const float lim = p.w + P.vcut + 1e-5f;
    const unsigned n = P.n;
    unsigned c = 0;
    for (unsigned k = b; k < e; ++k) {
        const unsigned t = __ldg(tpt + k);
        // the triangle's bounding sphere first
        const float4 bs = __ldg(tbound + t);
        const float sx = bs.x - p.x, sy = bs.y - p.y, sz = bs.z - p.z;
        if (sqrtf(sx * sx + sy * sy + sz * sz) - bs.w > lim) continue;
        const float* v = tri_ref + 9 * (size_t)t;
        bool face;
        const float d2 = tri_dist2_f(__ldg(v) - p.x, __ldg(v + 1) - p.y, __ldg(v + 2) - p.z, __ldg(v + 3) - p.x,
                                     __ldg(v + 4) - p.y, __ldg(v + 5) - p.z, __ldg(v + 6) - p.x,
                                     __ldg(v + 7) - p.y, __ldg(v + 8) - p.z, face);
        if (d2 < lim * lim || !(d2 < 3.0e38f)) {
            if (c < P.tcap) tlist[(size_t)c * n + i] = t;
            ++c;
        }
    }
    tcount[i] = c > P.tcap ? (P.tcap | kIncomplete) : c;
    if (c > P.tcap) count_one(counters + CN_TINC);
    count_add(counters + CN_TSUM, min(c, P.tcap));
}

// Verlet list build (steps that re-bin the cells), one thread per particle:
// the nine neighbour rows' slot ranges, trimmed to the cells within reach,
// are staged in shared memory and visited as one flattened loop (rows z then
// y, slots ascending: the reference's order); every j with
// |pj - pi| < ri + rj + vcut (FP32) is listed.  More than P.vcap marks the
// list incomplete (the contact pass then searches the cells).  Also records
// the build positions for the skin test, each particle's planes in reach
// (within r + skin), zero contact force, and the list of the particles with
// neighbours or planes in reach -- the only ones the contact pass visits until
// the next build.
__global__ void __launch_bounds__(256) k_mx_build(MixParams P, const float4* __restrict__ pf,
                                                  const unsigned* __restrict__ keys,
                                                  const unsigned* __restrict__ lb,
                                                  unsigned* __restrict__ vcount,
                                                  unsigned* __restrict__ vlist,
                                                  float4* __restrict__ pref,
                                                  unsigned short* __restrict__ wmask,
                                                  const unsigned* __restrict__ tcount,
                                                  double* __restrict__ rxn,
                                                  unsigned* __restrict__ hlist,
                                                  float4* __restrict__ Fc, float4* __restrict__ Mc,
                                                  unsigned* __restrict__ counters)
{
    __shared__ uint2 rows[9][256];
    const unsigned tid = threadIdx.x;
    const unsigned i = blockIdx.x * blockDim.x + tid;
    bool heavy = false, tri = false;
    if (i < P.n) {
        const float4 pi = __ldg(pf + i);
        pref[i] = pi;
        Fc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        Mc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (unsigned q = 0; q < 6 * P.nbodies; ++q) rxn[(size_t)q * P.n + i] = 0.0;
        const unsigned wm = near_planes(P, pi, P.wall_tol + P.vcut);
        wmask[i] = (unsigned short)wm;
        const unsigned key = __ldg(keys + i);
        // Neighbour cells out of reach are skipped: particles assigned to the
        // cell below on an axis lie at most half a skin above its top face, so
        // none of them is within ri + r_max + vcut of i when i is farther than
        // that above it; likewise above.
        unsigned cx, cy, cz;
        decode_key(P, key, cx, cy, cz);
        const float reach = pi.w + P.rmaxf + P.vcut + P.half_skin;
        const float bx = (float)((int)cx - 1) * P.csf, by = (float)((int)cy - 1) * P.csf,
                    bz = (float)((int)cz - 1) * P.csf;
        const bool lox = pi.x - bx < reach, hix = bx + P.csf - pi.x < reach;
        const bool loy = pi.y - by < reach, hiy = by + P.csf - pi.y < reach;
        const bool loz = pi.z - bz < reach, hiz = bz + P.csf - pi.z < reach;
        const unsigned x0 = key - (lox ? 1u : 0u), x1 = key + (hix ? 2u : 1u);
        unsigned left = 0;   // candidates over all rows
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            const int dy = r % 3 - 1, dz = r / 3 - 1;
            const bool use = (dy < 0 ? loy : dy > 0 ? hiy : true) && (dz < 0 ? loz : dz > 0 ? hiz : true);
            const unsigned off = (unsigned)dy * (unsigned)P.gx + (unsigned)dz * P.gxy;
            // cell indices wrap in 32-bit unsigned arithmetic before indexing
            const unsigned c0 = x0 + off, c1 = x1 + off;
            const uint2 b = use ? make_uint2(__ldg(lb + c0), __ldg(lb + c1)) : make_uint2(0u, 0u);
            rows[r][tid] = b;
            left += b.y - b.x;
        }
        const unsigned n = P.n;
        const float rt0 = pi.w + P.vcut;
        unsigned nv = 0, r = 0;
        uint2 b = rows[0][tid];
        unsigned j = b.x;
        for (; left; --left, ++j) {
            if (j == b.y) {   // next non-empty row (one exists while candidates are left)
                do {
                    b = rows[++r][tid];
                } while (b.x == b.y);
                j = b.x;
            }
            const float4 pj = __ldg(pf + j);
            const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
            const float Rt = rt0 + pj.w;
            if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) >= Rt * Rt || j == i) continue;
            if (nv < P.vcap) vlist[(size_t)nv * n + i] = j;
            ++nv;
        }
        vcount[i] = nv > P.vcap ? (P.vcap | kIncomplete) : nv;
        if (nv > P.vcap) count_one(counters + CN_VINC);
        count_add(counters + CN_VSUM, min(nv, P.vcap));
        tri = (P.ntri && __ldg(tcount + i) != 0u) || wm != 0u;   // walls in reach
        heavy = nv > 0 || tri;
    }
    // the spheres with walls (planes or triangles) in reach first, the others
    // from the end: the wall pass takes the front of the list, and in the
    // per-particle pass the warps run the wall work side by side instead of
    // on a few lanes each
    warp_append(heavy && tri, i, hlist, counters + CN_HTRI);
    const unsigned bal = __ballot_sync(0xffffffffu, heavy && !tri);
    if (bal) {
        const unsigned lane = threadIdx.x & 31u;
        const int leader = __ffs(bal) - 1;
        unsigned base = 0;
        if ((int)lane == leader) base = atomicAdd(counters + CN_HBACK, (unsigned)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (heavy && !tri) hlist[P.n - 1u - (base + __popc(bal & ((1u << lane) - 1u)))] = i;
    }
    const unsigned hb = __ballot_sync(0xffffffffu, heavy);
    if (hb && (threadIdx.x & 31u) == 0) atomicAdd(counters + CN_HEAVY, (unsigned)__popc(hb));
}

// Per-particle contact state carried across the pairs of one particle (the
// reference keeps Ft and M in the kernel across pairs, impl:426-428).
struct PairAcc {
    f3 Ft, Mm, sumF, sumM;
};

// One pair contact's terms: the normal force, and -- when its slip is not
// zero -- the tangential force and moment that replace the carried ones.
struct PairOut {
    f3 Fn, Ft, Mm;
    bool slip;
};

// Own data of particle i for its force loop.
struct Own {
    unsigned i;
    longlong2 qa, qb;
    float4 vh, vl;
    f3 w;
    float r, im;   // radius, 1/m
    float wfloor;  // m g: the smallest force scale of the particle's contacts
    float4 pr;     // residuals of its fixed-point position and radius (metres)
};

// When an FP32 contact force term is re-formed in FP64.  The per-particle
// force error is judged against max(sum_c |F_c|, m g); each contact's FP32
// error is kept below kForceTol of its own scale max(|Fn|, m g), so that the
// handful of contacts of a particle stay well inside the 2e-5 gate.
//  * normal force: the FP32 terms carry about kTermErr of the largest term;
//  * slip: the FP32 rotation term w x r u carries about kRotErr of its
//    terms' size |w| r (not of its value: a spin about the normal leaves a
//    small cross product of large terms); below the Coulomb cap the
//    tangential force moves by (ks dt + vs) times that, at the cap its
//    direction turns by that over |e|.
constexpr float kForceTol = 2e-6f;
constexpr float kTermErr = 5e-7f;
constexpr float kRotErr = 7e-7f;

__device__ __forceinline__ bool normal_needs_fp64(float term_max, float fn_abs, float wfloor)
{
    return kTermErr * term_max > kForceTol * fmaxf(fn_abs, wfloor);
}

__device__ __forceinline__ bool slip_needs_fp64(float wt, float ee, float lin, float mu, float fn_abs, float wfloor)
{
    if (!(wt > 0.f)) return false;
    const float me = sqrtf(ee);
    const float scale = kForceTol * fmaxf(fn_abs, wfloor);
    if (lin * me >= mu * fn_abs) return kRotErr * wt * mu * fn_abs > scale * me;   // at the cap
    return kRotErr * wt * lin > scale;
}

// The force of one contact (i, j).  getConstant TCM = 1 (impl:238-246) and
// DHSModel (impl:379-401) in FP32: the overlap from the exact integer
// separation (or the reference's FP64 expression for guard-band pairs), the
// relative velocity from the double-float velocities, and the two
// cancellation cases (normal force near zero, rolling slip) formed in FP64.
// HIST: 0 the reference's DHS; 1 tangential springs kept in the table (an
// extension, formed in FP64 from the FP32 normal, slip and normal force);
// 2 the same read-only (diagnostic evaluation).
// OUT: the contact's terms go to *o instead of the running sums in A (the
// warp-cooperative pass sums them in list order afterwards; see accumulate).
template <int HIST, bool OUT = false>
__device__ __forceinline__ void contact_force(const MixParams& P, const Master& M, const Own& I,
                                              unsigned j, bool guard, const double* __restrict__ mass0,
                                              const float4* __restrict__ pf,
                                              const longlong2* __restrict__ qa,
                                              const longlong2* __restrict__ qb,
                                              const float4* __restrict__ pr,
                                              unsigned* __restrict__ counters, PairAcc& A,
                                              const HistTable& ht, HistState& hs, PairOut* o = nullptr)
{
    const unsigned i = I.i;
    const float dt = P.dtf;
    const longlong2 qaj = __ldg(qa + j), qbj = __ldg(qb + j);
    const long long ddx = qaj.x - I.qa.x, ddy = qaj.y - I.qa.y, ddz = qbj.x - I.qb.x;
    const long long D2 = ddx * ddx + ddy * ddy + ddz * ddz;
    const float D2f = (float)D2;
    const float dn = sqrtf(D2f);
    // 64-bit integer conversions issue on the FP64 pipe: values that fit in
    // 32 bits (a touching pair's separation and radius sum when 2 r_max <
    // 2^-6 m) take the 32-bit ones, which round the same
    float fdx, fdy, fdz;
    if (P.small_q) {
        fdx = __int2float_rn((int)ddx);
        fdy = __int2float_rn((int)ddy);
        fdz = __int2float_rn((int)ddz);
    } else {
        fdx = (float)ddx;
        fdy = (float)ddy;
        fdz = (float)ddz;
    }
    float delta;
    if (guard) {
        delta = (float)fp64_cdist(M, i, j);
    } else {
        const long long Rq = I.qb.y + qbj.y;
        const float fRq = P.small_q ? __int2float_rn((int)Rq) : (float)Rq;
        delta = ((float)(Rq * Rq - D2) / (fRq + dn)) * kU;
    }
    const float inv = 1.0f / dn;
    const f3 u = fk(fdx * inv, fdy * inv, fdz * inv);
    // The fixed point's residuals restore the FP64 positions: the overlap
    // gains (e_ri + e_rj) - u . (e_j - e_i) (the 2^-36 m grid alone would move
    // a light contact's overlap by up to ~3e-11 m, a part in 1e5 of 3e-6 m)
    const float4 ej = __ldg(pr + j);
    const f3 de = fk(ej.x - I.pr.x, ej.y - I.pr.y, ej.z - I.pr.z);
    const float ude = fdot(u, de);
    if (!guard) delta += (I.pr.w + ej.w) - ude;
    const float4 vj4 = __ldg(M.vh + j), vjl = __ldg(M.vl + j), wj4 = __ldg(M.wh + j);
    const f3 wj = fk(wj4.x, wj4.y, wj4.z);
    const float jr = __ldg(pf + j).w, jim = vj4.w;
    const float ir = I.r;
    // vj - vi formed exactly from the double-float velocities
    float dvs[3], dvt[3];
    df_diff(vj4.x, I.vh.x, __fsub_rn(vjl.x, I.vl.x), dvs[0], dvt[0]);
    df_diff(vj4.y, I.vh.y, __fsub_rn(vjl.y, I.vl.y), dvs[1], dvt[1]);
    df_diff(vj4.z, I.vh.z, __fsub_rn(vjl.z, I.vl.z), dvs[2], dvt[2]);
    const f3 dv = fk(dvs[0] + dvt[0], dvs[1] + dvt[1], dvs[2] + dvt[2]);
    // rv = vj + wj x (-rj u) - (vi + wi x (ri u)), or vj - vi without rolling (impl:455)
    const f3 wterm = P.rolling ? fcross(wj, (-jr) * u) - fcross(I.w, ir * u) : fk(0.f, 0.f, 0.f);
    const f3 rv = dv + wterm;
    // rv . u = dv . u (the rotation term is perpendicular to u), in double-float
    const int dqi[3] = { (int)ddx, (int)ddy, (int)ddz };
    float rq0, rq1, rqc;
    float rvu = normal_speed(dvs, dvt, dqi, dn, D2, D2f, rq0, rq1, rqc);
    {
        // and the normal's turn (de - (u . de) u) / |d| in the normal speed
        const float cr = (fdot(dv, de) - rvu * ude) * (inv * (1.0f / kU));
        rq1 += cr;
        rvu = rq0 + rq1;
    }
    f3 ev = rv - rvu * u;
    float ee = fdot(ev, ev);
    // getConstant, TCM = 1 (impl:238-246)
    const float Meq = 1.0f / (I.im + jim);   // m_i m_j / (m_i + m_j)
    const float Req = (ir * jr) / (ir + jr);
    const float kn = P.c43Eeq * sqrtf(Req);
    const float vn = sqrtf((4.0f * Meq * kn) / P.one_b2);
    const float ks = kn * P.sratio, vs = vn * P.sratio;
    // DHSModel (impl:379-401)
    const float fsn = -kn * (delta * sqrtf(delta));
    const float fdn = vn * rvu;
    float fca = 0.f;
    if (P.coh != 0.f) {
        // cohesionForce (impl:259-279): coh pi rc^2, rc^3 = 3 Req (-fsn) Eeq / 4
        const float rc = cbrtf((3.0f * Req * (-fsn)) / (4.0f * (1.0f / P.coh_eeq)));
        fca = P.coh * (3.14159265358979f * rc * rc);
    }
    float fn = fsn + fca + fdn;
    if (normal_needs_fp64(fmaxf(fmaxf(fabsf(fsn), fabsf(fdn)), fca), fabsf(fn), I.wfloor)) {
        // The elastic, (cohesive) and damping terms nearly cancel (the
        // normal force of an unloading contact crossing zero): FP32 rounding
        // of each term would dominate the small sum, so it is formed again
        // in pair arithmetic (in FP64 with cohesion), with the overlap from
        // the FP64 positions.
        count_one(counters + CN_NORMALS);
        const unsigned idi = __float_as_uint(__ldg(M.wl + i).w), idj = __float_as_uint(__ldg(M.wl + j).w);
        if (P.coh == 0.f) {
            fn = normal_pair(P, M, mass0, i, j, idi, idj, rq0, rq1);
        } else {
            const double dl = fp64_cdist(M, i, j);
            const double ri = __ldg(M.r + i), rj = __ldg(M.r + j);
            const double mi = __ldg(mass0 + idi), mj = __ldg(mass0 + idj);
            const double Meqd = (mi * mj) / (mi + mj), Reqd = (ri * rj) / (ri + rj);
            const double knd = P.c43Eeq_d * sqrt(Reqd);
            const double vnd = sqrt((4.0 * Meqd * knd) / P.one_b2_d);
            const double fsnd = -knd * (dl * sqrt(dl));
            const double rc = pow((3.0 * Reqd * (-fsnd)) / (4.0 * (1.0 / P.coh_eeq_d)), 1.0 / 3.0);
            const double fcad = P.coh_d * (M_PI * rc * rc);
            // rv . u = dv . u (the rotation term is perpendicular to u)
            fn = (float)(fsnd + fcad + vnd * ((double)rq0 + (double)rq1));
        }
    }
    // The slip in FP64 where the FP32 rounding of the rotation term (about
    // kRotErr of |w x r|) could move the tangential force by more than
    // kForceTol of the contact's force scale max(|Fn|, m_i g): a sliding
    // contact (Coulomb cap) whose slip nearly cancels, or a fast spin.
    if (P.rolling && slip_needs_fp64(sqrtf(fdot(I.w, I.w)) * ir + sqrtf(fdot(wj, wj)) * jr, ee, ks * dt + vs, P.fric,
                                     fabsf(fn), I.wfloor)) {
        count_one(counters + CN_SLIPS);
        ev = slip_pair(dvs, dvt, dqi, dn, rqc, rq0, rq1, I.qb.y, qbj.y, make_float4(I.w.x, I.w.y, I.w.z, 0.f),
                       __ldg(M.wl + i), wj4, __ldg(M.wl + j));
        ee = fdot(ev, ev);
    }
    // products and sums rounded one by one (no contraction into the sums), so
    // that the per-particle and the warp-cooperative pair passes, which sum
    // these terms in different places, give the same bits
    const f3 Fn = fk(__fmul_rn(fn, u.x), __fmul_rn(fn, u.y), __fmul_rn(fn, u.z));
    if (HIST) {
        // the partner's key is its original index
        const unsigned key = __float_as_uint(__ldg(M.wl + j).w);
        d3 d;
        int sl = -1;
        if (HIST == 1) sl = hist_slot(ht, hs, i, key, d);
        else hist_peek(ht, i, key, d);
        xd::Fc c;
        c.kn = kn;
        c.vn = vn;
        c.ks = ks;
        c.vs = vs;
        c.mu = P.fric;
        d3 Ftd, Md;
        hist_tangential(c, (double)ir, mk(ev.x, ev.y, ev.z), mk(u.x, u.y, u.z), P.dt, mk(Fn.x, Fn.y, Fn.z), d,
                        Ftd, Md);
        if (HIST == 1) hist_store(ht, sl, i, d);
        A.Ft = fk((float)Ftd.x, (float)Ftd.y, (float)Ftd.z);
        A.Mm = fk((float)Md.x, (float)Md.y, (float)Md.z);
    } else {
        const float mag_e = sqrtf(ee);
        if (OUT) {
            o->Fn = Fn;
            o->slip = mag_e != 0.f;
        }
        if (mag_e != 0.f) {
            const float ie = 1.0f / mag_e;
            const f3 sh = fk(__fmul_rn(ie, ev.x), __fmul_rn(ie, ev.y), __fmul_rn(ie, ev.z));
            // dv . sh = |e| exactly (sh is the unit slip direction)
            const float ft = fminf(ks * (mag_e * dt) + vs * mag_e, P.fric * fabsf(fn));
            const f3 Ft = fk(__fmul_rn(ft, sh.x), __fmul_rn(ft, sh.y), __fmul_rn(ft, sh.z));
            const f3 Mm = fcross_rn(fk(__fmul_rn(ir, u.x), __fmul_rn(ir, u.y), __fmul_rn(ir, u.z)), Ft);
            if (OUT) {
                o->Ft = Ft;
                o->Mm = Mm;
                return;
            }
            A.Ft = Ft;
            A.Mm = Mm;
        }
        if (OUT) return;
    }
    A.sumF = fadd_rn(A.sumF, fadd_rn(Fn, A.Ft));
    A.sumM = fadd_rn(A.sumM, A.Mm);
}

// Adds one contact's terms to the particle's sums, as contact_force does in
// its own loop: a contact with zero slip keeps the tangential force and
// moment of the one before it (impl:390-400).
__device__ __forceinline__ void accumulate(PairAcc& A, const PairOut& o)
{
    if (o.slip) {
        A.Ft = o.Ft;
        A.Mm = o.Mm;
    }
    A.sumF = fadd_rn(A.sumF, fadd_rn(o.Fn, A.Ft));
    A.sumM = fadd_rn(A.sumM, A.Mm);
}

// Contact forces of the particles on the heavy list (the others keep the
// zero force of the last build): the particle pairs of the Verlet list (or,
// for an incomplete list, of the neighbour cells) in search order -- FP32
// prefilter, exact integer test, FP64 guard band, FP32 Hertz-Mindlin -- then
// plane_contact_force_kernel<1> (impl:572-621) for the planes in reach, in
// FP64, in plane order (the others are out of reach and add exactly zero).
// Block 0 clears CN_REBUILD for the next step's skin test.


// Entry t of the listed particles: the ones with triangles in reach fill the
// list from the front (front of them), the others from the end.
__device__ __forceinline__ unsigned list_index(unsigned t, unsigned front, unsigned n)
{
    return t < front ? t : n - 1u - (t - front);
}

// The pointers of one scene the contact pass reads and writes.
struct ContactArgs {
    Master M;
    const float4* pf;
    const longlong2* qa;
    const longlong2* qb;
    const float4* pr;
    const unsigned* keys;
    const unsigned* lb;
    const unsigned* vcount;
    const unsigned* vlist;
    const unsigned* hlist;
    const unsigned short* wmask;
    const xd_plane_info* planes;
    const PlaneRec* prec;
    const double* mass0;
    const xd_polygon_info* poly;
    const TriRec* trec;
    const xd_polygon_mass_info* pmi;
    const unsigned* tcount;
    const unsigned* tlist;
    const unsigned* tpk;
    const unsigned* tpt;
    unsigned tcap;
    double* rxn;
    float4* Fc;
    float4* Mc;
    unsigned* counters;
    unsigned* rec_count;
    unsigned* rec_pairs;
    unsigned rec_cap;
    HistTable ht;
    int rxn_on;
};

// ---- wall contacts in FP32 ------------------------------------------------

// Metres: a wall contact whose FP64 plane distance is within this of touching
// is decided by the reference's FP64 region test (the plane distance and the
// reference's closest-point chain differ by a few 1e-16 m).
constexpr double kWallGuard = 1e-13;

// One wall contact's force: DHSModel (impl:379-401) with Req = r, Meq = m and
// no particle moment, as the plane and polygon kernels call it (ir = 0).
// cd: the overlap (FP64), u: the unit normal (FP64), dvd: the relative
// velocity without the particle's rotation term, in FP64 (wall velocity
// minus the particle's); the rotation term -(w x r u) is added in FP32 (it
// is perpendicular to u, so the normal speed dv . u is dvd . u, formed in
// FP64: a sliding sphere's dv is nearly perpendicular to u).  Ft is in/out:
// the polygon kernel keeps it across triangles when a slip is exactly zero.
// The normal force and the rolling slip are formed again in FP64 when their
// FP32 terms nearly cancel, as for particle pairs.
struct WallK {
    float kn, vn, ks, vs, mu;
    const double* c43Eeq;   // getConstant's FP64 terms (for the rechecks)
    const double* one_b2;
};

__device__ __forceinline__ WallK wall_constants(const double* c43Eeq, const double* one_b2, double sratio,
                                                double fric, float rf, float mf)
{
    WallK k;
    k.kn = (float)*c43Eeq * sqrtf(rf);
    k.vn = sqrtf((4.0f * mf * k.kn) / (float)*one_b2);
    k.ks = k.kn * (float)sratio;
    k.vs = k.vn * (float)sratio;
    k.mu = (float)fric;
    k.c43Eeq = c43Eeq;
    k.one_b2 = one_b2;
    return k;
}

// One wall contact's terms: the normal force and, when the slip is not zero,
// the tangential force (else the one carried from the contact before stays).
struct WallOut {
    f3 Fn, Ft;
    bool slip;
};

__device__ __forceinline__ WallOut wall_force(const MixParams& P, const WallK& k, double cd, d3 u, d3 dvd, double r,
                                              double m, float rf, float wfloor, const float4& wh, const float4& wl,
                                              unsigned* __restrict__ counters)
{
    const float df = (float)cd;
    const f3 uf = fk((float)u.x, (float)u.y, (float)u.z);
    const double rvu_d = dvd.x * u.x + dvd.y * u.y + dvd.z * u.z;
    const float rvu = (float)rvu_d;
    const f3 wterm = P.rolling ? fcross(fk(wh.x, wh.y, wh.z), (-rf) * uf) : fk(0.f, 0.f, 0.f);
    const f3 dvf = fk((float)dvd.x, (float)dvd.y, (float)dvd.z) + wterm;
    f3 ev = dvf - rvu * uf;
    float ee = fdot(ev, ev);
    const float fsn = -k.kn * (df * sqrtf(df));
    const float fdn = k.vn * rvu;
    float fn = fsn + fdn;
    if (normal_needs_fp64(fmaxf(fabsf(fsn), fabsf(fdn)), fabsf(fn), wfloor)) {
        // the terms nearly cancel: formed again in pair arithmetic
        count_one(counters + CN_NORMALS);
        const dfl R = d_to_df(r), D = d_to_df(cd);
        const dfl kn = df_mul(d_to_df(*k.c43Eeq), df_sqrt(R));
        const dfl vn = df_sqrt(df_div(df_mul(df_mul(dfl{ 4.f, 0.f }, d_to_df(m)), kn), d_to_df(*k.one_b2)));
        const dfl f = df_add(df_neg(df_mul(kn, df_mul(D, df_sqrt(D)))), df_mul(vn, d_to_df(rvu_d)));
        fn = __fadd_rn(f.hi, f.lo);
    }
    if (P.rolling && slip_needs_fp64(sqrtf(wh.x * wh.x + wh.y * wh.y + wh.z * wh.z) * rf, ee, k.ks * P.dtf + k.vs,
                                     k.mu, fabsf(fn), wfloor)) {
        // the rotation term cancels most of the slip
        count_one(counters + CN_SLIPS);
        const d3 iw = mk(df_to_d(wh.x, wl.x), df_to_d(wh.y, wl.y), df_to_d(wh.z, wl.z));
        const d3 dv = dvd - cross(iw, r * u);
        const double dn = dot(dv, u);
        ev = fk((float)(dv.x - dn * u.x), (float)(dv.y - dn * u.y), (float)(dv.z - dn * u.z));
        ee = fdot(ev, ev);
    }
    WallOut o;
    // products rounded one by one, so that the per-particle and the
    // cooperative wall passes, which add these terms in different places,
    // give the same bits
    o.Fn = fk(__fmul_rn(fn, uf.x), __fmul_rn(fn, uf.y), __fmul_rn(fn, uf.z));
    const float mag_e = sqrtf(ee);
    o.slip = mag_e != 0.f;
    if (o.slip) {
        // dv . s = |e| (s the unit slip direction)
        const float ft = fminf(k.ks * (mag_e * P.dtf) + k.vs * mag_e, k.mu * fabsf(fn));
        const float ie = 1.0f / mag_e;
        o.Ft = fk(__fmul_rn(ft, __fmul_rn(ie, ev.x)), __fmul_rn(ft, __fmul_rn(ie, ev.y)),
                  __fmul_rn(ft, __fmul_rn(ie, ev.z)));
    }
    return o;
}

// The wall data of particle i that its wall contacts read.
struct WallOwn {
    float4 pi, vh, vl, wh, wl;
    d3 ip, iv;
    double r, m;
    float mf, wfloor;
};

__device__ __forceinline__ WallOwn load_wall_own(const MixParams& P, const ContactArgs& C, unsigned i)
{
    const Master& M = C.M;
    WallOwn o;
    o.pi = __ldg(C.pf + i);
    o.vh = __ldg(M.vh + i);
    o.vl = __ldg(M.vl + i);
    o.wh = __ldg(M.wh + i);
    o.wl = __ldg(M.wl + i);
    o.m = __ldg(C.mass0 + __float_as_uint(o.wl.w));
    o.mf = (float)o.m;
    o.wfloor = o.mf * sqrtf(P.gf[0] * P.gf[0] + P.gf[1] * P.gf[1] + P.gf[2] * P.gf[2]);
    o.ip = mk(__ldg(M.x + i), __ldg(M.y + i), __ldg(M.z + i));
    o.r = __ldg(M.r + i);
    o.iv = mk(df_to_d(o.vh.x, o.vl.x), df_to_d(o.vh.y, o.vl.y), df_to_d(o.vh.z, o.vl.z));
    return o;
}

// One wall candidate's result: kind 0 none, 1 plane, 2 triangle (of body b,
// po2cp its contact point from the body's origin, FP32).
struct WallRes {
    unsigned kind, b;
    WallOut o;
    f3 po2cp;
};

constexpr unsigned kWallPlane = 0x80000000u;   // candidate code: plane w is kWallPlane | w, triangle t is t

// Wall candidate `code` of particle i: plane_contact_force_kernel<1>
// (impl:572-621) for a plane, particle_polygonObject_collision_kernel<1>
// (impl:923-1021) for a triangle.  A contact whose closest point is clearly
// inside the face in the FP32 region test (relative to the sphere centre)
// is found by one FP64 plane distance; every other contact, and any within
// kWallGuard of touching, by the reference's FP64 region test, rounded per
// operation, so every contact decision is the reference's.
__device__ __forceinline__ WallRes wall_eval(const MixParams& P, const ContactArgs& C, const WallOwn& w,
                                             unsigned code)
{
    unsigned* __restrict__ counters = C.counters;
    const float rf = w.pi.w;
    WallRes res;
    res.kind = 0;
    if (code & kWallPlane) {
        const unsigned pw = code & ~kWallPlane;
        const PlaneRec* pr = C.prec + pw;
        const d3 dp = w.ip - mk(__ldg(pr->xw), __ldg(pr->xw + 1), __ldg(pr->xw + 2));
        const float dx = (float)dp.x, dy = (float)dp.y, dz = (float)dp.z;
        const float wx = dx * __ldg(pr->u1) + dy * __ldg(pr->u1 + 1) + dz * __ldg(pr->u1 + 2);
        const float wy = dx * __ldg(pr->u2) + dy * __ldg(pr->u2 + 1) + dz * __ldg(pr->u2 + 2);
        const float l1 = __ldg(&pr->l1), l2 = __ldg(&pr->l2);
        const float mg = 1e-6f * (fabsf(dx) + fabsf(dy) + fabsf(dz) + l1 + l2);
        double cd = -1.0;
        d3 unit;
        bool exact = true;
        if (wx > mg && wx < l1 - mg && wy > mg && wy < l2 - mg) {
            // inside the rectangle: the face region (impl:557-560)
            const d3 n = mk(__ldg(pr->n), __ldg(pr->n + 1), __ldg(pr->n + 2));
            const double h = dp.x * n.x + dp.y * n.y + dp.z * n.z;
            cd = w.r - fabs(h);
            if (cd < -kWallGuard) return res;
            if (cd > kWallGuard && fabs(h) > 1e-12) {
                exact = false;
                unit = h < 0.0 ? n : -n;
            }
        }
        if (exact) {
            count_one(counters + CN_WALLS);
            const PlaneD pe = load_plane(C.planes + pw);
            cd = plane_detection(pe, w.ip, plane_coords(pe, w.ip), unit, w.r);
            if (!(cd > 0)) return res;
        }
        const WallK k = wall_constants(P.pl_c43Eeq + pw, P.pl_one_b2 + pw, P.pl_sratio[pw], P.pl_fric[pw], rf, w.mf);
        res.kind = 1;
        res.o = wall_force(P, k, cd, unit, -w.iv, w.r, w.m, rf, w.wfloor, w.wh, w.wl, counters);
        return res;
    }
    const unsigned t = code;
    const TriRec* tr = C.trec + t;
    const d3 sp = w.ip - mk(__ldg(tr->p), __ldg(tr->p + 1), __ldg(tr->p + 2));   // x - P
    const float sx = (float)sp.x, sy = (float)sp.y, sz = (float)sp.z;
    const float qx = __ldg(tr->q) - sx, qy = __ldg(tr->q + 1) - sy, qz = __ldg(tr->q + 2) - sz;
    const float cx = __ldg(tr->r) - sx, cy = __ldg(tr->r + 1) - sy, cz = __ldg(tr->r + 2) - sz;
    bool face;
    const float d2f = tri_dist2_f(-sx, -sy, -sz, qx, qy, qz, cx, cy, cz, face);
    {
        // out of reach by more than the FP32 error: no contact in FP64 either
        const float span = fabsf(sx) + fabsf(sy) + fabsf(sz) + fabsf(qx) + fabsf(qy) + fabsf(qz) + fabsf(cx) +
                           fabsf(cy) + fabsf(cz);
        const float lim = rf + 1e-6f + 1e-5f * span;
        if (d2f > lim * lim && d2f < 3.0e38f) return res;
    }
    const d3 u = mk(__ldg(tr->n), __ldg(tr->n + 1), __ldg(tr->n + 2));
    double cd = -1.0;
    d3 cpt;
    bool exact = true;
    if (face) {
        const double h = sp.x * u.x + sp.y * u.y + sp.z * u.z;   // n . (x - P)
        cd = w.r - fabs(h);
        if (cd < -kWallGuard) return res;
        if (cd > kWallGuard) {
            exact = false;
            cpt = w.ip - h * u;
        }
    }
    if (exact) {
        count_one(counters + CN_WALLS);
        const xd_polygon_info* tri = C.poly + t;
        cpt = closest_pt_triangle(tri_vertex(tri->P), tri_vertex(tri->Q), tri_vertex(tri->R), w.ip);
        cd = rn::sub(w.r, rn::length(rn::sub(w.ip, cpt)));
        if (!(cd > 0)) return res;
    }
    const unsigned b = __ldg(&tr->body);
    // getConstant with the body's hoisted material terms (Meq = m, Req = r)
    const WallK k = wall_constants(P.pb_c43Eeq + b, P.pb_one_b2 + b, P.pb_sratio[b], P.pb_fric[b], rf, w.mf);
    const xd_polygon_mass_info* body = C.pmi + b;
    const d3 po2cp = cpt - tri_vertex(body->origin);
    const d3 pvel = tri_vertex(body->vel), pom = tri_vertex(body->omega);
    // a body at rest: the wall velocity is zero, and so is every term of it
    const bool moving = pvel.x != 0.0 || pvel.y != 0.0 || pvel.z != 0.0 || pom.x != 0.0 || pom.y != 0.0 ||
                        pom.z != 0.0;
    const d3 dvd = !moving ? -w.iv : (P.rolling ? (pvel + cross(pom, po2cp)) - w.iv : pvel - w.iv);
    res.kind = 2;
    res.b = b;
    res.o = wall_force(P, k, cd, u, dvd, w.r, w.m, rf, w.wfloor, w.wh, w.wl, counters);
    res.po2cp = fk((float)po2cp.x, (float)po2cp.y, (float)po2cp.z);
    return res;
}

// The reaction of a particle's run of triangle contacts on one body, added
// to the particle's slots of rxn when the body changes and at the end
// (consecutive contacts on the same body are summed in registers first: the
// slots are read and written once per run instead of once per contact).
struct RxnAcc {
    unsigned b;
    double v[6];
};

__device__ __forceinline__ void rxn_flush(const ContactArgs& C, unsigned n, unsigned i, RxnAcc& a)
{
    if (a.b == 0xffffffffu) return;
    double* rb = C.rxn + (size_t)a.b * 6 * n + i;
#pragma unroll
    for (int q = 0; q < 6; ++q) rb[(size_t)q * n] += a.v[q];
    a.b = 0xffffffffu;
}

// Adds one wall result to particle i's wall force f, in candidate order: a
// plane starts from Ft = 0 (each plane is its own launch in the reference);
// triangles carry Ft from one to the next when a slip is exactly zero; the
// reaction on the triangle's body (-fc and -(po2cp x fc)) goes to the run
// accumulator a.
__device__ __forceinline__ void wall_add(const ContactArgs& C, unsigned n, unsigned i, const WallRes& r, f3& f,
                                         f3& Ftri, RxnAcc& a)
{
    if (r.kind == 0) return;
    f3 Ft;
    if (r.kind == 1) {
        Ft = r.o.slip ? r.o.Ft : fk(0.f, 0.f, 0.f);
    } else {
        if (r.o.slip) Ftri = r.o.Ft;
        Ft = Ftri;
    }
    const f3 fc = fadd_rn(r.o.Fn, Ft);
    f = fadd_rn(f, fc);
    if (r.kind == 2 && C.rxn_on) {
        if (a.b != r.b) {
            rxn_flush(C, n, i, a);
            a.b = r.b;
#pragma unroll
            for (int q = 0; q < 6; ++q) a.v[q] = 0.0;
        }
        const f3 rm = fcross_rn(fc, r.po2cp);   // -(po2cp x fc)
        a.v[0] -= (double)fc.x;
        a.v[1] -= (double)fc.y;
        a.v[2] -= (double)fc.z;
        a.v[3] += (double)rm.x;
        a.v[4] += (double)rm.y;
        a.v[5] += (double)rm.z;
    }
}

// The wall contacts of listed particle i (the reference's DHS model, no
// history): its planes in reach (plane_contact_force_kernel<1>,
// impl:572-621; each plane starts from Ft = 0, as each is its own launch
// there), then its triangles (particle_polygonObject_collision_kernel<1>,
// impl:923-1021; Ft kept across triangles, the normal from the face winding,
// the wall velocity of the body at the contact point, the reaction summed per
// particle into rxn).  A contact whose closest point is clearly inside the
// face in the FP32 region test (relative to the sphere centre) is found by
// one FP64 plane distance; every other contact, and any within kWallGuard of
// touching, by the reference's FP64 region test, rounded per operation, so
// every contact decision is the reference's.  The forces are FP32
// (wall_force).
__device__ __forceinline__ f3 walls_fp32(const MixParams& P, const ContactArgs& C, const unsigned i, const float4 pi,
                                      const unsigned wm, const unsigned tc)
{
    const WallOwn w = load_wall_own(P, C, i);
    f3 f = fk(0.f, 0.f, 0.f), Ftri = fk(0.f, 0.f, 0.f);
    RxnAcc ra;
    ra.b = 0xffffffffu;
    for (unsigned mask = wm; mask; mask &= mask - 1u)
        wall_add(C, P.n, i, wall_eval(P, C, w, kWallPlane | (unsigned)(__ffs(mask) - 1)), f, Ftri, ra);
    if (tc) {
        const unsigned n = P.n;
        const bool listed = !(tc & kIncomplete);
        unsigned kb = 0, ke = tc;
        if (!listed) {
            const unsigned key = __ldg(C.keys + i);
            kb = lower_bound_u(C.tpk, C.tcap, key);
            ke = lower_bound_u(C.tpk, C.tcap, key + 1u);
        }
        for (unsigned kk = kb; kk < ke; ++kk) {
            const unsigned t = listed ? __ldg(C.tlist + (size_t)kk * n + i) : __ldg(C.tpt + kk);
            wall_add(C, n, i, wall_eval(P, C, w, t), f, Ftri, ra);
        }
        rxn_flush(C, n, i, ra);
    }
    return f;
}

// The contact pass of one listed particle (slot i): its Verlet-list pairs,
// planes and triangles, summed in a fixed order into Fc/Mc.
template <bool RECORD, int HIST>
__device__ __forceinline__ void contact_entry(const MixParams& P, const ContactArgs& C, const unsigned i)
{
    const Master& M = C.M;
    const float4* __restrict__ pf = C.pf;
    const longlong2* __restrict__ qa = C.qa;
    const longlong2* __restrict__ qb = C.qb;
    const unsigned* __restrict__ keys = C.keys;
    const unsigned* __restrict__ lb = C.lb;
    const unsigned* __restrict__ vcount = C.vcount;
    const unsigned* __restrict__ vlist = C.vlist;
    const unsigned short* __restrict__ wmask = C.wmask;
    const xd_plane_info* __restrict__ planes = C.planes;
    const double* __restrict__ mass0 = C.mass0;
    const xd_polygon_info* __restrict__ poly = C.poly;
    const xd_polygon_mass_info* __restrict__ pmi = C.pmi;
    const unsigned* __restrict__ tcount = C.tcount;
    const unsigned* __restrict__ tlist = C.tlist;
    const unsigned* __restrict__ tpk = C.tpk;
    const unsigned* __restrict__ tpt = C.tpt;
    const unsigned tcap = C.tcap;
    double* __restrict__ rxn = C.rxn;
    float4* __restrict__ Fc = C.Fc;
    float4* __restrict__ Mc = C.Mc;
    unsigned* __restrict__ counters = C.counters;
    unsigned* __restrict__ rec_count = C.rec_count;
    unsigned* __restrict__ rec_pairs = C.rec_pairs;
    const unsigned rec_cap = C.rec_cap;
    const HistTable& ht = C.ht;
    const int rxn_on = C.rxn_on;
    const unsigned n = P.n;
    const float4 pi = __ldg(pf + i);
    // the particle's own data is loaded when first needed: most listed
    // particles have neighbours within the skin but no contact
    Own I;
    I.i = i;
    I.r = pi.w;
    bool have_q = false, have_v = false;
    PairAcc A;
    A.Ft = fk(0.f, 0.f, 0.f);
    A.Mm = fk(0.f, 0.f, 0.f);
    A.sumF = fk(0.f, 0.f, 0.f);
    A.sumM = fk(0.f, 0.f, 0.f);
    unsigned nc = 0;
    HistState hs;
    if (HIST == 1) hist_begin(ht, i, hs);
    auto add = [&](unsigned j, bool guard) {
        if (!have_v) {
            I.vh = __ldg(M.vh + i);
            I.vl = __ldg(M.vl + i);
            const float4 w4 = __ldg(M.wh + i);
            I.w = fk(w4.x, w4.y, w4.z);
            I.im = I.vh.w;
            I.wfloor = sqrtf(P.gf[0] * P.gf[0] + P.gf[1] * P.gf[1] + P.gf[2] * P.gf[2]) / I.im;
            I.pr = __ldg(C.pr + i);
            have_v = true;
        }
        contact_force<HIST>(P, M, I, j, guard, mass0, pf, qa, qb, C.pr, counters, A, ht, hs);
        if (RECORD && nc < rec_cap) rec_pairs[(size_t)i * rec_cap + nc] = j;
        ++nc;
    };
    const unsigned vc = __ldg(vcount + i);
    if (!(vc & kIncomplete)) {
        const float rt0 = pi.w + P.tol;
        for (unsigned k = 0; k < vc; ++k) {
            const unsigned j = __ldg(vlist + (size_t)k * n + i);
            const float4 pj = __ldg(pf + j);
            const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
            const float Rt = rt0 + pj.w;
            if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) >= Rt * Rt) continue;
            if (!have_q) {
                I.qa = __ldg(qa + i);
                I.qb = __ldg(qb + i);
                have_q = true;
            }
            const int c = exact_touch<true>(P, M, i, j, I.qa, I.qb, qa, qb, counters);
            if (c) add(j, c == 2);
        }
    } else {
        I.qa = __ldg(qa + i);
        I.qb = __ldg(qb + i);
        for_each_contact<true>(P, M, i, pi, I.qa, I.qb, __ldg(keys + i), pf, qa, qb, lb, counters, add);
    }
    float4 F = make_float4(A.sumF.x, A.sumF.y, A.sumF.z, 0.f);
    // planes in reach: an FP32 distance to the supporting plane first (the
    // finite plane is never nearer), the reference's FP64 test after it
    unsigned wm = __ldg(wmask + i);
    for (unsigned mask = wm; mask; mask &= mask - 1u) {
        const int w = __ffs(mask) - 1;
        const float hz = (pi.x - P.pxw[w][0]) * P.pun[w][0] + (pi.y - P.pxw[w][1]) * P.pun[w][1] +
                         (pi.z - P.pxw[w][2]) * P.pun[w][2];
        if (!(fabsf(hz) < pi.w + P.tol)) wm &= ~(1u << w);
    }
    if (HIST == 0) {
        const unsigned tc0 = P.ntri ? __ldg(tcount + i) : 0u;
        if (wm || tc0) {
            const f3 fw = walls_fp32(P, C, i, pi, wm, tc0);
            F.x += fw.x;
            F.y += fw.y;
            F.z += fw.z;
        }
        Fc[i] = F;
        Mc[i] = make_float4(A.sumM.x, A.sumM.y, A.sumM.z, 0.f);
        if (RECORD) rec_count[i] = nc;
        return;
    }
    if (wm) {
        const float4 vh = __ldg(M.vh + i), vl = __ldg(M.vl + i);
        const float4 wl = __ldg(M.wl + i), wh = __ldg(M.wh + i);
        const double m = __ldg(mass0 + __float_as_uint(wl.w));
        const d3 ip = mk(__ldg(M.x + i), __ldg(M.y + i), __ldg(M.z + i));
        const double r = __ldg(M.r + i);
        const d3 iv = mk(df_to_d(vh.x, vl.x), df_to_d(vh.y, vl.y), df_to_d(vh.z, vl.z));
        const d3 iw = mk(df_to_d(wh.x, wl.x), df_to_d(wh.y, wl.y), df_to_d(wh.z, wl.z));
        d3 f = mk(0, 0, 0);
        for (unsigned mask = wm; mask; mask &= mask - 1u) {
            const int w = __ffs(mask) - 1;
            PlaneD pe = load_plane(planes + w);
            d3 Fn = mk(0, 0, 0), Ft = mk(0, 0, 0), Mo = mk(0, 0, 0);
            d3 dp = ip - pe.xw;
            d3 unit = mk(0, 0, 0);
            d3 wp = mk(dot(dp, pe.u1), dot(dp, pe.u2), dot(dp, pe.uw));
            double cdist = plane_detection(pe, ip, wp, unit, r);
            if (cdist > 0) {
                d3 dv = P.rolling ? -(iv + cross(iw, r * unit)) : -iv;
                // getConstant with the plane's hoisted material terms (Meq = m, Req = r)
                xd::Fc c;
                c.kn = P.pl_c43Eeq[w] * sqrt(r);
                c.vn = sqrt((4.0 * m * c.kn) / P.pl_one_b2[w]);
                c.ks = c.kn * P.pl_sratio[w];
                c.vs = c.vn * P.pl_sratio[w];
                c.mu = P.pl_fric[w];
                if (HIST) {
                    Fn = normal_force(c, 0, 0, 0, 0, 0, 0, 0.0, cdist, dv, unit);
                    d3 d;
                    int sl = -1;
                    if (HIST == 1) sl = hist_slot(ht, hs, i, kHistPlane | (unsigned)w, d);
                    else hist_peek(ht, i, kHistPlane | (unsigned)w, d);
                    hist_tangential(c, 0.0, dv, unit, P.dt, Fn, d, Ft, Mo);
                    if (HIST == 1) hist_store(ht, sl, i, d);
                } else {
                    dhs(c, 0, 0, 0, 0, 0, 0, 0.0, cdist, dv, unit, P.dt, Ft, Fn, Mo);
                }
            }
            f += Fn + Ft;
        }
        F.x += (float)f.x;
        F.y += (float)f.y;
        F.z += (float)f.z;
    }
    // triangles in reach: particle_polygonObject_collision_kernel<1>
    // (impl:923-1021) in FP64, the normal from the face winding, the wall
    // velocity of the body at the contact point, no particle moment (ir = 0
    // as the reference calls DHSModel); Ft persists across triangles.  The
    // reaction on each body accumulates in this particle's own slots of rxn
    // over the steps and is summed over particles in a fixed order when the
    // slots are flushed (at a re-binning and at the end of a call).
    const unsigned tc = P.ntri ? __ldg(tcount + i) : 0u;
    if (tc) {
        const float4 vh = __ldg(M.vh + i), vl = __ldg(M.vl + i);
        const float4 wl = __ldg(M.wl + i), wh = __ldg(M.wh + i);
        const double m = __ldg(mass0 + __float_as_uint(wl.w));
        const d3 ip = mk(__ldg(M.x + i), __ldg(M.y + i), __ldg(M.z + i));
        const double r = __ldg(M.r + i);
        const d3 iv = mk(df_to_d(vh.x, vl.x), df_to_d(vh.y, vl.y), df_to_d(vh.z, vl.z));
        const d3 iw = mk(df_to_d(wh.x, wl.x), df_to_d(wh.y, wl.y), df_to_d(wh.z, wl.z));
        d3 f = mk(0, 0, 0), Ft = mk(0, 0, 0), Mo = mk(0, 0, 0);
        const double sr = sqrt(r);
        unsigned cb = 0xffffffffu;
        xd::Fc cc;
        const bool listed = !(tc & kIncomplete);
        unsigned kb = 0, ke = tc;
        if (!listed) {
            const unsigned key = __ldg(keys + i);
            kb = lower_bound_u(tpk, tcap, key);
            ke = lower_bound_u(tpk, tcap, key + 1u);
        }
        for (unsigned k = kb; k < ke; ++k) {
            const unsigned t = listed ? __ldg(tlist + (size_t)k * n + i) : __ldg(tpt + k);
            const xd_polygon_info* tri = poly + t;
            const unsigned b = (unsigned)__ldg(&tri->id);
            const d3 Pv = tri_vertex(tri->P), Qv = tri_vertex(tri->Q), Rv = tri_vertex(tri->R);
            {
                // FP32 pre-test relative to the sphere: a triangle farther than r
                // (plus a margin far above the FP32 error) is one the FP64 test below
                // skips as well
                const float ax = (float)(Pv.x - ip.x), ay = (float)(Pv.y - ip.y), az = (float)(Pv.z - ip.z);
                const float bx = (float)(Qv.x - ip.x), by = (float)(Qv.y - ip.y), bz = (float)(Qv.z - ip.z);
                const float cx = (float)(Rv.x - ip.x), cy = (float)(Rv.y - ip.y), cz = (float)(Rv.z - ip.z);
                bool face;
                const float d2f = tri_dist2_f(ax, ay, az, bx, by, bz, cx, cy, cz, face);
                const float span = fabsf(ax) + fabsf(ay) + fabsf(az) + fabsf(bx) + fabsf(by) + fabsf(bz) + fabsf(cx) +
                                   fabsf(cy) + fabsf(cz);
                const float lim = (float)r + 1e-6f + 1e-5f * span;
                if (d2f > lim * lim && d2f < 3.0e38f) continue;
            }
            const d3 cpt = closest_pt_triangle(Pv, Qv, Rv, ip);
            const double cdist = r - length(ip - cpt);
            if (!(cdist > 0)) continue;
            const d3 po2cp = cpt - tri_vertex(pmi[b].origin);
            d3 unit = -cross(Qv - Pv, Rv - Pv);
            unit = unit / length(unit);
            const d3 pvel = tri_vertex(pmi[b].vel), pom = tri_vertex(pmi[b].omega);
            const d3 dv = P.rolling ? (pvel + cross(pom, po2cp)) - (iv + cross(iw, r * unit)) : (pvel - iv);
            if (b != cb) {
                // getConstant with the body's hoisted material terms (Meq = m,
                // Req = r): the same for every triangle of the body
                cc.kn = P.pb_c43Eeq[b] * sr;
                cc.vn = sqrt((4.0 * m * cc.kn) / P.pb_one_b2[b]);
                cc.ks = cc.kn * P.pb_sratio[b];
                cc.vs = cc.vn * P.pb_sratio[b];
                cc.mu = P.pb_fric[b];
                cb = b;
            }
            const xd::Fc& c = cc;
            d3 Fn = mk(0, 0, 0);
            if (HIST) {
                Fn = normal_force(c, 0, 0, 0, 0, 0, 0, 0.0, cdist, dv, unit);
                d3 d;
                int sl = -1;
                if (HIST == 1) sl = hist_slot(ht, hs, i, kHistTri | t, d);
                else hist_peek(ht, i, kHistTri | t, d);
                hist_tangential(c, 0.0, dv, unit, P.dt, Fn, d, Ft, Mo);
                if (HIST == 1) hist_store(ht, sl, i, d);
            } else {
                dhs(c, 0, 0, 0, 0, 0, 0, 0.0, cdist, dv, unit, P.dt, Ft, Fn, Mo);
            }
            const d3 fc = Fn + Ft;
            f += fc;
            const d3 rm = -cross(po2cp, fc);
            if (rxn_on) {
                double* rb = rxn + (size_t)b * 6 * n + i;
                rb[0] -= fc.x;
                rb[n] -= fc.y;
                rb[2 * (size_t)n] -= fc.z;
                rb[3 * (size_t)n] += rm.x;
                rb[4 * (size_t)n] += rm.y;
                rb[5 * (size_t)n] += rm.z;
            }
        }
        F.x += (float)f.x;
        F.y += (float)f.y;
        F.z += (float)f.z;
    }
    if (HIST == 1) hist_end_all(ht, hs, i);
    Fc[i] = F;
    Mc[i] = make_float4(A.sumM.x, A.sumM.y, A.sumM.z, 0.f);
    if (RECORD) rec_count[i] = nc;
}

// ---- the warp-cooperative pair pass ------------------------------------------
//
// In a packed bed every listed particle has several contacts, and a thread
// per particle leaves most lanes idle while the warp runs the longest list.
// Here the 32 particles of a warp are done together in rounds.  Each lane
// first scans its own particle's Verlet list (or its cells) and keeps up to
// kCoopSlots touching partners in shared memory; then the warp's partners,
// level by level (every lane's first, then every lane's second, ...), are
// spread over the lanes, one contact per lane, each forming its contact's
// force with contact_force; and each particle's lane adds its own contacts'
// terms in its list order (accumulate).  With the contacts by level, a group
// of 32 holds one or two of most particles, so the adding is spread over
// the lanes instead of running on a few of them.  The sums are
// therefore the same bits as the per-particle pass's.  A lane with more
// than kCoopSlots contacts goes on in the next round where it stopped.

constexpr unsigned kCoopSlots = 16;

struct CoopBuf {
    unsigned cand[32 * kCoopSlots];   // k-major: lane L's k-th candidate at [k * 32 + L]
    float res[10][32];                // one contact per lane: Fn, Ft, Mm, slip
};

// A cooperative pass's buffer: the candidates k-major (so that the lanes'
// writes and a level's reads fall in distinct banks), and the round's order
// of contacts: slot[p] the candidate at position p, pos[k * 32 + L] the
// position of lane L's k-th.
struct PairBuf {
    CoopBuf c;
    unsigned short slot[32 * kCoopSlots];
    unsigned short pos[32 * kCoopSlots];
};

// Orders a round's candidates (cnt of this lane's) by level: every lane's
// first in lane order, then every lane's second, ...  A group of 32
// positions then holds one or two candidates of most particles, and each
// lane's own stay in its order.  Returns the round's count.
__device__ __forceinline__ unsigned level_order(PairBuf& PB, unsigned cnt, unsigned lane)
{
    const unsigned lt = (1u << lane) - 1u;
    const unsigned maxc = __reduce_max_sync(0xffffffffu, cnt);
    unsigned total = 0;
    for (unsigned k = 0; k < maxc; ++k) {
        const unsigned b = __ballot_sync(0xffffffffu, cnt > k);
        if (cnt > k) {
            const unsigned p = total + __popc(b & lt);
            PB.slot[p] = (unsigned short)(k * 32u + lane);
            PB.pos[k * 32u + lane] = (unsigned short)p;
        }
        total += __popc(b);
    }
    __syncwarp();
    return total;
}

// A lane whose Verlet list overflowed: its cells searched from the start,
// the partners before `done` skipped, up to kCoopSlots after them kept in
// mine[0], mine[32], ...; returns whether more are left.  Out of line:
// rare, and the pass's loop stays short.
__device__ __noinline__ bool coop_cells(const MixParams& P, const ContactArgs& C, unsigned i, float4 pi,
                                        longlong2 qai, longlong2 qbi, unsigned& done, unsigned* mine,
                                        unsigned& cnt)
{
    unsigned seen = 0;
    for_each_contact<true>(P, C.M, i, pi, qai, qbi, __ldg(C.keys + i), C.pf, C.qa, C.qb, C.lb, C.counters,
                           [&](unsigned j, bool guard) {
                               if (seen >= done && cnt < kCoopSlots)
                                   mine[32u * cnt++] = j | (guard ? kGuardBit : 0u);
                               ++seen;
                           });
    done += cnt;
    return seen > done;
}

// Own data of slot i as contact_force reads it.
__device__ __forceinline__ Own load_own(const MixParams& P, const ContactArgs& C, unsigned i)
{
    Own I;
    I.i = i;
    I.r = __ldg(C.pf + i).w;
    I.qa = __ldg(C.qa + i);
    I.qb = __ldg(C.qb + i);
    I.vh = __ldg(C.M.vh + i);
    I.vl = __ldg(C.M.vl + i);
    const float4 w4 = __ldg(C.M.wh + i);
    I.w = fk(w4.x, w4.y, w4.z);
    I.im = I.vh.w;
    I.wfloor = sqrtf(P.gf[0] * P.gf[0] + P.gf[1] * P.gf[1] + P.gf[2] * P.gf[2]) / I.im;
    I.pr = __ldg(C.pr + i);
    return I;
}

// The contact pass of list entries (valid lanes: slot i) without tangential
// history, every lane of the warp taking part: pairs cooperatively, then
// each particle's planes and triangles (walls_fp32) by its own lane.
__device__ __forceinline__ void contact_entry_coop(const MixParams& P, const ContactArgs& C, bool valid, unsigned i,
                                                   PairBuf& PB)
{
    CoopBuf& B = PB.c;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned n = P.n;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    unsigned vc = 0;
    longlong2 qai = make_longlong2(0, 0), qbi = make_longlong2(0, 0);
    if (valid) {
        pi = __ldg(C.pf + i);
        vc = __ldg(C.vcount + i);
        qai = __ldg(C.qa + i);
        qbi = __ldg(C.qb + i);
    }
    const bool incomplete = (vc & kIncomplete) != 0u;
    PairAcc A;
    A.Ft = fk(0.f, 0.f, 0.f);
    A.Mm = fk(0.f, 0.f, 0.f);
    A.sumF = fk(0.f, 0.f, 0.f);
    A.sumM = fk(0.f, 0.f, 0.f);
    HistState hs;
    unsigned kpos = 0, done = 0;
    bool more = valid;
    unsigned* mine = B.cand + lane;
    while (__any_sync(0xffffffffu, more)) {
        // this lane's next partners, in its search order
        unsigned cnt = 0;
        if (more) {
            if (!incomplete) {
                const float rt0 = pi.w + P.tol;
                // four list entries at a time, their loads issued together
                // (the partner's view and fixed point are loaded whether or
                // not the prefilter passes: most entries touch in a bed)
                while (kpos < vc && cnt < kCoopSlots) {
                    unsigned jj[4];
                    float4 pp[4];
                    longlong2 aa[4], bb[4];
#pragma unroll
                    for (unsigned q = 0; q < 4u; ++q)
                        jj[q] = kpos + q < vc ? __ldg(C.vlist + (size_t)(kpos + q) * n + i) : i;
#pragma unroll
                    for (unsigned q = 0; q < 4u; ++q) {
                        pp[q] = __ldg(C.pf + jj[q]);
                        aa[q] = __ldg(C.qa + jj[q]);
                        bb[q] = __ldg(C.qb + jj[q]);
                    }
#pragma unroll
                    for (unsigned q = 0; q < 4u; ++q) {
                        if (kpos >= vc || cnt >= kCoopSlots) break;
                        ++kpos;
                        const float dx = pp[q].x - pi.x, dy = pp[q].y - pi.y, dz = pp[q].z - pi.z;
                        const float Rt = rt0 + pp[q].w;
                        if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) >= Rt * Rt) continue;
                        const int c = exact_touch_q<true>(P, C.M, i, jj[q], qai, qbi, aa[q], bb[q], C.counters);
                        if (c) mine[32u * cnt++] = jj[q] | (c == 2 ? kGuardBit : 0u);
                    }
                }
                more = kpos < vc;
            } else {
                more = coop_cells(P, C, i, pi, qai, qbi, done, mine, cnt);
            }
        }
        __syncwarp();
        const unsigned total = level_order(PB, cnt, lane);
        unsigned kacc = 0;   // this lane's partners added so far this round
        for (unsigned base = 0; base < total; base += 32u) {
            // position c: the partner in slot sc, of lane sc % 32's particle
            const unsigned c = base + lane;
            const unsigned sc = c < total ? PB.slot[c] : 0u;
            const unsigned iL = __shfl_sync(0xffffffffu, i, sc & 31u);
            if (c < total) {
                const unsigned e = B.cand[sc];
                const Own I = load_own(P, C, iL);
                PairOut o;
                contact_force<0, true>(P, C.M, I, e & ~kGuardBit, (e & kGuardBit) != 0u, C.mass0, C.pf, C.qa,
                                       C.qb, C.pr, C.counters, A, C.ht, hs, &o);
                B.res[0][lane] = o.Fn.x;
                B.res[1][lane] = o.Fn.y;
                B.res[2][lane] = o.Fn.z;
                B.res[9][lane] = o.slip ? 1.f : 0.f;
                if (o.slip) {
                    B.res[3][lane] = o.Ft.x;
                    B.res[4][lane] = o.Ft.y;
                    B.res[5][lane] = o.Ft.z;
                    B.res[6][lane] = o.Mm.x;
                    B.res[7][lane] = o.Mm.y;
                    B.res[8][lane] = o.Mm.z;
                }
            }
            __syncwarp();
            // this lane's contacts in the group, in its list order
            for (; kacc < cnt; ++kacc) {
                const unsigned p = PB.pos[kacc * 32u + lane];
                if (p >= base + 32u) break;
                const unsigned k = p - base;
                PairOut o;
                o.Fn = fk(B.res[0][k], B.res[1][k], B.res[2][k]);
                o.slip = B.res[9][k] != 0.f;
                if (o.slip) {
                    o.Ft = fk(B.res[3][k], B.res[4][k], B.res[5][k]);
                    o.Mm = fk(B.res[6][k], B.res[7][k], B.res[8][k]);
                }
                accumulate(A, o);
            }
            __syncwarp();
        }
    }
    if (!valid) return;
    // the walls are added by the wall pass (walls_entry)
    C.Fc[i] = make_float4(A.sumF.x, A.sumF.y, A.sumF.z, 0.f);
    C.Mc[i] = make_float4(A.sumM.x, A.sumM.y, A.sumM.z, 0.f);
}

// The wall pass after the cooperative pair pass, warp-cooperative as well:
// the listed particles with walls in reach (the front of the list) list
// their wall candidates (planes in reach, then their triangles) into the
// warp's buffer, the candidates are spread one per lane in level order
// (level_order, wall_eval), and
// each particle's lane adds its results in candidate order (wall_add) and
// then its wall force to its pair force -- the additions the per-particle
// pass makes after its pairs (F += walls).  A launch of its own: the wall
// code's FP64 region tests and registers stay out of the pair pass.
// The wall pass's shared memory per warp: the candidate buffer, and each
// lane's particle data read once by its own lane for all its candidates.
struct WallBuf {
    PairBuf c;
    WallOwn own[32];
};

__device__ __forceinline__ void walls_entry_coop(const MixParams& P, const ContactArgs& C, bool valid, unsigned i,
                                                 WallBuf& WB)
{
    CoopBuf& B = WB.c.c;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned n = P.n;
    unsigned wm = 0, kb = 0, ke = 0;
    bool listed = true;
    if (valid) {
        const float4 pi = __ldg(C.pf + i);
        wm = __ldg(C.wmask + i);
        for (unsigned mask = wm; mask; mask &= mask - 1u) {
            const int w = __ffs(mask) - 1;
            const float hz = (pi.x - P.pxw[w][0]) * P.pun[w][0] + (pi.y - P.pxw[w][1]) * P.pun[w][1] +
                             (pi.z - P.pxw[w][2]) * P.pun[w][2];
            if (!(fabsf(hz) < pi.w + P.tol)) wm &= ~(1u << w);
        }
        const unsigned tc = P.ntri ? __ldg(C.tcount + i) : 0u;
        listed = !(tc & kIncomplete);
        ke = tc;
        if (!listed) {
            const unsigned key = __ldg(C.keys + i);
            kb = lower_bound_u(C.tpk, C.tcap, key);
            ke = lower_bound_u(C.tpk, C.tcap, key + 1u);
        }
    }
    const bool any = wm || kb < ke;
    if (any) WB.own[lane] = load_wall_own(P, C, i);
    f3 f = fk(0.f, 0.f, 0.f), Ftri = fk(0.f, 0.f, 0.f);
    RxnAcc ra;
    ra.b = 0xffffffffu;
    unsigned* mine = B.cand + lane;
    bool more = any;
    while (__any_sync(0xffffffffu, more)) {
        unsigned cnt = 0;
        for (; more && wm && cnt < kCoopSlots; wm &= wm - 1u)
            mine[32u * cnt++] = kWallPlane | (unsigned)(__ffs(wm) - 1);
        for (; more && kb < ke && cnt < kCoopSlots; ++kb)
            mine[32u * cnt++] = listed ? __ldg(C.tlist + (size_t)kb * n + i) : __ldg(C.tpt + kb);
        more = more && (wm || kb < ke);
        __syncwarp();
        const unsigned total = level_order(WB.c, cnt, lane);
        unsigned kacc = 0;
        for (unsigned base = 0; base < total; base += 32u) {
            const unsigned c = base + lane;
            if (c < total) {
                const unsigned sc = WB.c.slot[c];
                const WallRes r = wall_eval(P, C, WB.own[sc & 31u], B.cand[sc]);
                B.res[0][lane] = r.o.Fn.x;
                B.res[1][lane] = r.o.Fn.y;
                B.res[2][lane] = r.o.Fn.z;
                B.res[3][lane] = r.o.Ft.x;
                B.res[4][lane] = r.o.Ft.y;
                B.res[5][lane] = r.o.Ft.z;
                B.res[6][lane] = r.po2cp.x;
                B.res[7][lane] = r.po2cp.y;
                B.res[8][lane] = r.po2cp.z;
                B.res[9][lane] = __uint_as_float(r.kind | (r.kind && r.o.slip ? 4u : 0u) | (r.b << 3));
            }
            __syncwarp();
            for (; kacc < cnt; ++kacc) {
                const unsigned p = WB.c.pos[kacc * 32u + lane];
                if (p >= base + 32u) break;
                const unsigned k = p - base;
                const unsigned code = __float_as_uint(B.res[9][k]);
                WallRes r;
                r.kind = code & 3u;
                r.b = code >> 3;
                r.o.slip = (code & 4u) != 0u;
                r.o.Fn = fk(B.res[0][k], B.res[1][k], B.res[2][k]);
                r.o.Ft = fk(B.res[3][k], B.res[4][k], B.res[5][k]);
                r.po2cp = fk(B.res[6][k], B.res[7][k], B.res[8][k]);
                wall_add(C, n, i, r, f, Ftri, ra);
            }
            __syncwarp();
        }
    }
    if (!valid || !any) return;
    rxn_flush(C, n, i, ra);
    float4 F = C.Fc[i];
    F.x += f.x;
    F.y += f.y;
    F.z += f.z;
    C.Fc[i] = F;
}

__global__ void __launch_bounds__(kContactMaxThreads) k_mx_walls(MixParams P, ContactArgs C)
{
    extern __shared__ WallBuf wall_buf[];
    WallBuf& B = wall_buf[threadIdx.x / 32u];
    const unsigned front = C.counters[CN_HTRI];
    const unsigned warps = gridDim.x * (blockDim.x / 32u);
    const unsigned gw = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u;
    for (unsigned t0 = gw * 32u; t0 < front; t0 += warps * 32u) {
        const unsigned t = t0 + (threadIdx.x & 31u);
        const bool valid = t < front;
        walls_entry_coop(P, C, valid, valid ? __ldg(C.hlist + t) : 0u, B);
    }
}

// COOP: the warp-cooperative pair pass (no history, no recording; dynamic
// shared memory of one PairBuf per warp).
template <bool RECORD, int HIST, bool COOP>
__global__ void __launch_bounds__(kContactMaxThreads) k_mx_contact(MixParams P, ContactArgs C)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) C.counters[CN_REBUILD] = 0;
    const unsigned total = C.counters[CN_HEAVY], front = C.counters[CN_HTRI];
    // runs of 32 consecutive list entries go to the warps of all blocks in
    // turn: every SM gets an equal share however short the list
    const unsigned warps = gridDim.x * (blockDim.x / 32u);
    const unsigned gw = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u;
    if (COOP) {
        extern __shared__ PairBuf pair_buf[];
        PairBuf& B = pair_buf[threadIdx.x / 32u];
        for (unsigned t0 = gw * 32u; t0 < total; t0 += warps * 32u) {
            const unsigned t = t0 + (threadIdx.x & 31u);
            const bool valid = t < total;
            contact_entry_coop(P, C, valid, valid ? __ldg(C.hlist + list_index(t, front, P.n)) : 0u, B);
        }
        return;
    }
    for (unsigned t = gw * 32u + (threadIdx.x & 31u); t < total; t += warps * 32u)
        contact_entry<RECORD, HIST>(P, C, __ldg(C.hlist + list_index(t, front, P.n)));
}

// Body reactions: rxn[(b * 6 + q) * n + i] summed over i in a fixed order,
// added to the bodies and the slots cleared, in one launch (a flush).  Each block sums a fixed chunk of i for
// every q (per thread a strided run, then a fixed shuffle tree and the warps
// in order) into part[q * gridDim.x + block]; the last block to finish adds
// the blocks' partials in block order.  The order depends only on n and the
// grid, so a scene's reaction is the same in every run.
constexpr unsigned kRxnBlocks = 152 * 4;   // enough warps in flight to stream the slots from HBM
constexpr unsigned kRxnThreads = 256;

static unsigned rxn_grid(unsigned n) { return std::max(1u, std::min(kRxnBlocks, (n + kRxnThreads - 1) / kRxnThreads)); }

__global__ void __launch_bounds__(kRxnThreads) k_rxn_sum(double* __restrict__ rxn, unsigned n, unsigned nbodies,
                                                         double* __restrict__ part, unsigned* __restrict__ counters,
                                                         xd_polygon_mass_info* __restrict__ pmi)
{
    __shared__ double warp_sum[6][kRxnThreads / 32];
    __shared__ bool last;
    const unsigned nq = 6 * nbodies;
    const unsigned chunk = (n + gridDim.x - 1) / gridDim.x;
    const unsigned b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    const unsigned lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    for (unsigned b = 0; b < nbodies; ++b) {
        // the six components of one body together: six independent loads per
        // particle and one barrier per body
        double v[6] = { 0.0, 0.0, 0.0, 0.0, 0.0, 0.0 };
        double* rb = rxn + (size_t)b * 6 * n;
        for (unsigned i = b0 + threadIdx.x; i < b1; i += blockDim.x)
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                v[c] += rb[(size_t)c * n + i];
                rb[(size_t)c * n + i] = 0.0;   // flushed
            }
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            for (unsigned o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
            if (lane == 0) warp_sum[c][wid] = v[c];
        }
        __syncthreads();
        if (threadIdx.x < 6) {
            double t = 0.0;
            for (unsigned w = 0; w < blockDim.x / 32u; ++w) t += warp_sum[threadIdx.x][w];
            part[(size_t)(b * 6 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
            __threadfence();   // visible before this block is counted done
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counters + CN_RXN, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the block partials of each component: a warp per component, lane l
    // summing partials l, l + 32, ... and a fixed shuffle tree (the same
    // order every time; the loads overlap instead of forming one chain)
    for (unsigned q = wid; q < nq; q += blockDim.x / 32u) {
        double t = 0.0;
        for (unsigned k = lane; k < gridDim.x; k += 32u) t += __ldcg(part + (size_t)q * gridDim.x + k);
        for (unsigned o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) {
            const unsigned b = q / 6, c = q % 6;
            if (c < 3) pmi[b].force[c] += t;
            else pmi[b].moment[c - 3] += t;
        }
    }
    if (threadIdx.x == 0) counters[CN_RXN] = 0;
}

// ---- host-order state <-> master (reference layouts) -----------------------

__global__ void __launch_bounds__(256) k_mx_load(MixParams P, Master M, const double* __restrict__ pos,
                                                 const double* __restrict__ vel,
                                                 const double* __restrict__ acc,
                                                 const double* __restrict__ omega,
                                                 const double* __restrict__ alpha,
                                                 const double* __restrict__ mass,
                                                 const double* __restrict__ inertia,
                                                 double* __restrict__ mass0, float4* __restrict__ pf,
                                                 longlong2* __restrict__ qa, longlong2* __restrict__ qb,
                                                 float4* __restrict__ pr)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const size_t i3 = 3 * (size_t)i;
    const double x = pos[4 * (size_t)i + 0], y = pos[4 * (size_t)i + 1], z = pos[4 * (size_t)i + 2];
    const double r = pos[4 * (size_t)i + 3];
    M.x[i] = x;
    M.y[i] = y;
    M.z[i] = z;
    M.r[i] = r;
    const double m = mass[i], I = inertia[i];
    mass0[i] = m;
    float h[3], l[3], wh[3], wl[3];
    for (int a = 0; a < 3; ++a) {
        const double v = vel[i3 + a], w = omega[i3 + a];
        h[a] = __double2float_rn(v);
        l[a] = __double2float_rn(v - (double)h[a]);
        wh[a] = __double2float_rn(w);
        wl[a] = __double2float_rn(w - (double)wh[a]);
    }
    M.vh[i] = make_float4(h[0], h[1], h[2], (float)(1.0 / m));
    M.vl[i] = make_float4(l[0], l[1], l[2], 0.f);
    M.wh[i] = make_float4(wh[0], wh[1], wh[2], (float)(1.0 / I));
    M.wl[i] = make_float4(wl[0], wl[1], wl[2], __uint_as_float(i));
    M.ab[i] = make_float4((float)(acc[i3 + 0] - P.g[0]), (float)(acc[i3 + 1] - P.g[1]),
                          (float)(acc[i3 + 2] - P.g[2]), (float)alpha[i3 + 0]);
    M.b2[i] = make_float2((float)alpha[i3 + 1], (float)alpha[i3 + 2]);
    write_view(P, i, x, y, z, r, pf, qa, qb, pr);
}

__global__ void __launch_bounds__(256) k_mx_store(MixParams P, Master M, const double* __restrict__ mass0,
                                                  double* __restrict__ pos, double* __restrict__ vel,
                                                  double* __restrict__ acc, double* __restrict__ omega,
                                                  double* __restrict__ alpha,
                                                  double* __restrict__ force,
                                                  double* __restrict__ moment)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const float4 vh = M.vh[i], vl = M.vl[i], wh = M.wh[i], wl = M.wl[i], ab = M.ab[i];
    const float2 b2 = M.b2[i];
    const size_t o = __float_as_uint(wl.w);
    pos[4 * o + 0] = M.x[i];
    pos[4 * o + 1] = M.y[i];
    pos[4 * o + 2] = M.z[i];
    pos[4 * o + 3] = M.r[i];
    const double m = mass0[o];
    const float vh3[3] = { vh.x, vh.y, vh.z }, vl3[3] = { vl.x, vl.y, vl.z };
    const float wh3[3] = { wh.x, wh.y, wh.z }, wl3[3] = { wl.x, wl.y, wl.z };
    const float a3[3] = { ab.x, ab.y, ab.z }, b3[3] = { ab.w, b2.x, b2.y };
    for (int a = 0; a < 3; ++a) {
        vel[3 * o + a] = df_to_d(vh3[a], vl3[a]);
        omega[3 * o + a] = df_to_d(wh3[a], wl3[a]);
        acc[3 * o + a] = P.g[a] + (double)a3[a];
        alpha[3 * o + a] = b3[a];
        force[3 * o + a] = m * P.g[a];
        moment[3 * o + a] = 0.0;
    }
}

__global__ void __launch_bounds__(256) k_mx_store_forces(MixParams P, Master M,
                                                         const float4* __restrict__ Fc,
                                                         const float4* __restrict__ Mc,
                                                         double* __restrict__ force,
                                                         double* __restrict__ moment)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const size_t o = __float_as_uint(M.wl[i].w);
    const float4 f = Fc[i], t = Mc[i];
    force[3 * o + 0] = f.x;
    force[3 * o + 1] = f.y;
    force[3 * o + 2] = f.z;
    moment[3 * o + 0] = t.x;
    moment[3 * o + 1] = t.y;
    moment[3 * o + 2] = t.z;
}

__global__ void __launch_bounds__(256) k_mx_ids(MixParams P, Master M, unsigned* __restrict__ ids)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    ids[i] = __float_as_uint(M.wl[i].w);
}

}  // namespace

__global__ void k_plane_recs(const xd_plane_info* __restrict__ planes, unsigned nplanes, PlaneRec* __restrict__ out)
{
    const unsigned w = threadIdx.x;
    if (w >= nplanes) return;
    const PlaneD pe = load_plane(planes + w);
    const d3 uu = rn::divs(pe.uw, rn::length(pe.uw));
    PlaneRec r;
    r.xw[0] = pe.xw.x; r.xw[1] = pe.xw.y; r.xw[2] = pe.xw.z;
    r.n[0] = uu.x; r.n[1] = uu.y; r.n[2] = uu.z;
    r.u1[0] = (float)pe.u1.x; r.u1[1] = (float)pe.u1.y; r.u1[2] = (float)pe.u1.z;
    r.u2[0] = (float)pe.u2.x; r.u2[1] = (float)pe.u2.y; r.u2[2] = (float)pe.u2.z;
    r.l1 = (float)pe.l1;
    r.l2 = (float)pe.l2;
    out[w] = r;
}

static int launch_plane_recs(const xd_plane_info* planes, unsigned nplanes, PlaneRec* out, cudaStream_t q)
{
    if (!nplanes) return XD_OK;
    k_plane_recs<<<1, 32, 0, q>>>(planes, nplanes, out);
    return launch_status("plane records");
}

// ------------------------------------------------------------------ host

static void plane_prefilter(MixParams& P, const xd_plane_info* planes, unsigned nplanes);

static int mixed_setup(MixedScene* s, const xd_scene_desc& d, const double* pos_host)
{
    s->n = d.np;
    s->cap = d.np;
    s->nplanes = d.nplanes;
    if (d.np >= 0x7fffffffu) return set_error(XD_ERR_CAPACITY, "mixed mode: too many particles");
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
    // triangle meshes (as placed now; a body that later moves beyond the grid
    // has its triangles clamped into the boundary cells)
    double tri_edge = 0.0;
    for (unsigned t = 0; t < d.ntri; ++t) {
        const xd_polygon_info& tr = d.poly[t];
        const double* V[3] = { tr.P, tr.Q, tr.R };
        for (int k = 0; k < 3; ++k) {
            for (int a = 0; a < 3; ++a) {
                lo[a] = fmin(lo[a], V[k][a]);
                hi[a] = fmax(hi[a], V[k][a]);
            }
            const double* W = V[(k + 1) % 3];
            const double e = sqrt((V[k][0] - W[0]) * (V[k][0] - W[0]) + (V[k][1] - W[1]) * (V[k][1] - W[1]) +
                                  (V[k][2] - W[2]) * (V[k][2] - W[2]));
            tri_edge = fmax(tri_edge, e);
        }
    }
    if (d.np == 0) {
        for (int a = 0; a < 3; ++a) { lo[a] = 0; hi[a] = 1; }
        rmax = 0.5;
    }
    if (!(rmax > 0.0)) return set_error(XD_ERR_INVALID, "mixed mode: particle radii must be > 0");
    double extent = 0.0;
    for (int a = 0; a < 3; ++a) extent = fmax(extent, hi[a] - lo[a] + 8.0 * rmax);
    if (!(extent < 16384.0))
        return set_error(XD_ERR_INVALID, "mixed mode: scene extent %g m exceeds 16384 m", extent);
    // The cell is the contact range 2 r_max plus the skin, plus 0.1 % and the
    // error of the FP32 position estimates that place particles (a few ulp of
    // the extent): two touching particles, each within half the skin of its
    // assigned cell, always have neighbouring assigned cells.
    const double skin = (double)s->skin_factor * rmax;
    s->cs = 2.0 * rmax * 1.001 + skin + extent * 0x1p-19;
    double margin = 2.0 * s->cs;
    int g[3];
    unsigned long long ncell = 1;
    for (int a = 0; a < 3; ++a) {
        lo[a] -= margin;
        hi[a] += margin;
        // origin on the 2^-20 m grid: a multiple of 2^-36 m as well
        lo[a] = std::floor(lo[a] * 1048576.0) / 1048576.0;
        g[a] = (int)ceil((hi[a] - lo[a]) / s->cs) + 2;
        ncell *= (unsigned long long)g[a];
    }
    if (ncell > 0x7ffffff0ull)
        return set_error(XD_ERR_CAPACITY, "mixed mode: grid of %llu cells is too large", ncell);
    s->gx = g[0]; s->gy = g[1]; s->gz = g[2];
    s->ncell = (unsigned)ncell;
    MixParams& P = s->P;
    memset(&P, 0, sizeof(P));
    P.gx = g[0]; P.gy = g[1]; P.gz = g[2];
    P.gxy = (unsigned)(g[0] * g[1]);
    P.n = d.np;
    const double dt = d.params.dt, half2dt = d.params.half2dt;
    for (int a = 0; a < 3; ++a) {
        P.wo[a] = lo[a];
        P.qoff[a] = kMagic - lo[a] * kQ;
        P.g[a] = d.params.gravity[a];
        P.gf[a] = (float)P.g[a];
        P.G1[a] = df_split(dt * P.g[a]);
        P.G2[a] = df_split(half2dt * P.g[a]);
    }
    P.dt = dt;
    P.csf = (float)s->cs;
    P.inv_csf = (float)(1.0 / s->cs);
    P.half_skin = (float)(0.5 * skin);
    P.rmaxf = (float)rmax;
    P.small_q = 2.0 * rmax < 0x1p-6 ? 1 : 0;
    P.inv_gx = 1.0f / (float)g[0];
    P.inv_gxy = 1.0f / (float)((double)g[0] * g[1]);
    P.dtf = (float)dt;
    P.hf = (float)(0.5 * dt);
    P.half2dtf = (float)half2dt;
    P.dt_df = df_split(dt);
    P.tol = (float)(4e-6 + extent * 0x1p-20);
    // The Verlet list holds the pairs within ri + rj + skin + tol at its build;
    // re-binning (and a new list) comes before any particle has moved half the
    // skin less the FP32 position error, so no unlisted pair can touch.
    P.vcut = (float)skin + P.tol;
    P.disp2 = (float)((0.5 * skin - P.tol) * (0.5 * skin - P.tol));
    P.wall_tol = (float)(1e-5 + extent * 0x1p-20);
    const xd_contact_property& cp = d.cp_pp;
    double Eeq = (cp.Ei * cp.Ej) / (cp.Ei * (1 - cp.prj * cp.prj) + cp.Ej * (1 - cp.pri * cp.pri));
    double beta = M_PI / log(cp.rest);
    P.c43Eeq_d = (4.0 / 3.0) * Eeq;
    P.one_b2_d = 1.0 + beta * beta;
    P.c43Eeq = (float)P.c43Eeq_d;
    P.one_b2 = (float)P.one_b2_d;
    P.c43Eeq_p = df_split(P.c43Eeq_d);
    P.one_b2_p = df_split(P.one_b2_d);
    P.sratio = (float)cp.sratio;
    P.fric = (float)cp.fric;
    P.coh_d = cp.coh;
    P.coh_eeq_d = cp.coh != 0.0 ? ((1.0 - cp.pri * cp.pri) / cp.Ei) + ((1.0 - cp.prj * cp.prj) / cp.Ej) : 0.0;
    P.coh = (float)P.coh_d;
    P.coh_eeq = (float)P.coh_eeq_d;
    P.guard_q = (long long)ceil(kGuard * kQ);
    P.nplanes = (int)d.nplanes;
    P.rolling = d.params.rollingCondition ? 1 : 0;
    P.ntri = d.ntri;
    P.nbodies = d.ntri ? d.nbodies : 0;
    P.vcap = s->vcap;
    P.tcap = s->tcap;
    // a particle within r + skin of a triangle has its centre within this of
    // the triangle's bounding box
    P.tri_reach = (float)(rmax + skin) + 2.0f * P.tol;
    for (unsigned b = 0; b < P.nbodies; ++b) {
        // getConstant's material terms (impl:214-256) of each body's contact property
        const xd_contact_property& c = d.cp_poly[b];
        const double eq = (c.Ei * c.Ej) / (c.Ei * (1 - c.prj * c.prj) + c.Ej * (1 - c.pri * c.pri));
        const double bt = M_PI / log(c.rest);
        P.pb_c43Eeq[b] = (4.0 / 3.0) * eq;
        P.pb_one_b2[b] = 1.0 + bt * bt;
        P.pb_sratio[b] = c.sratio;
        P.pb_fric[b] = c.fric;
    }
    for (unsigned w = 0; w < d.nplanes; ++w) {
        // getConstant's material terms (impl:214-256), hoisted out of the kernel
        const xd_contact_property& c = d.cp_planes[w];
        const double eq = (c.Ei * c.Ej) / (c.Ei * (1 - c.prj * c.prj) + c.Ej * (1 - c.pri * c.pri));
        const double bt = M_PI / log(c.rest);
        P.pl_c43Eeq[w] = (4.0 / 3.0) * eq;
        P.pl_one_b2[w] = 1.0 + bt * bt;
        P.pl_sratio[w] = c.sratio;
        P.pl_fric[w] = c.fric;
    }
    plane_prefilter(P, d.planes, d.nplanes);

    const size_t n = d.np;
    int st = XD_OK;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    for (int b = 0; b < 2; ++b) {
        Master& M = s->m[b];
        A(alloc(s, &M.x, n));
        A(alloc(s, &M.y, n));
        A(alloc(s, &M.z, n));
        A(alloc(s, &M.r, n));
        A(alloc(s, &M.vh, n));
        A(alloc(s, &M.vl, n));
        A(alloc(s, &M.wh, n));
        A(alloc(s, &M.wl, n));
        A(alloc(s, &M.ab, n));
        A(alloc(s, &M.b2, n));
    }
    A(alloc(s, &s->mass0, n));
    A(alloc(s, &s->pf, n));
    A(alloc(s, &s->qa, n));
    A(alloc(s, &s->qb, n));
    A(alloc(s, &s->pr, n));
    A(alloc(s, &s->Fc, n));
    A(alloc(s, &s->Mc, n));
    A(alloc(s, &s->hlist, n));
    A(alloc(s, &s->wmask, n));
    A(alloc(s, &s->vcount, n));
    A(alloc(s, &s->vlist, n * s->vcap));
    A(alloc(s, &s->pref, n));
    A(alloc(s, &s->keys, n));
    A(alloc(s, &s->vals, n));
    A(alloc(s, &s->prev_keys, n));
    A(alloc(s, &s->lb, (size_t)s->ncell + 1));
    s->gap_cap = s->ncell / kGapWarp + 2;
    A(alloc(s, &s->gaps, s->gap_cap));
    char* scr = nullptr;
    A(alloc(s, &scr, radix_sort_scratch_bytes((unsigned)n)));
    s->sort_scratch = scr;
    A(alloc(s, &s->planes, s->nplanes));
    A(alloc(s, &s->prec, s->nplanes));
    A(alloc(s, &s->cps, s->nplanes));
    A(alloc(s, &s->counters, kCounters));
    s->passes = (key_bits_for(s->ncell) + 7) / 8;
    if (st == XD_OK) A(cuda_status(cudaMemset(s->counters, 0, sizeof(unsigned) * kCounters), "mixed counters"));
    if (st == XD_OK && s->nplanes) {
        A(cuda_status(cudaMemcpy(s->planes, d.planes, sizeof(xd_plane_info) * s->nplanes, cudaMemcpyHostToDevice), "mixed planes"));
        A(launch_plane_recs(s->planes, s->nplanes, s->prec, 0));
        A(cuda_status(cudaStreamSynchronize(0), "mixed planes"));
        A(cuda_status(cudaMemcpy(s->cps, d.cp_planes, sizeof(xd_contact_property) * s->nplanes, cudaMemcpyHostToDevice), "mixed planes"));
    }
    if (st == XD_OK && d.ntri) {
        s->ntri = d.ntri;
        s->nbodies = d.nbodies;
        // (cell, triangle) pairs: a triangle's box, widened by the reach, spans
        // at most ceil((edge + 2 reach) / cs) + 1 cells per axis in any pose
        const double span = ceil((tri_edge + 2.0 * (double)P.tri_reach) / s->cs) + 1.0;
        const double cap = (double)d.ntri * span * span * span;
        if (cap > (double)(1u << 30))
            return set_error(XD_ERR_CAPACITY, "mixed mode: %u triangles of up to %g m span %g cells each; "
                             "the cell-triangle table would exceed 2^30 entries", d.ntri, tri_edge,
                             span * span * span);
        s->tpair_cap = (unsigned)cap;
        A(alloc(s, &s->poly, s->ntri));
        A(alloc(s, &s->sphere, 4 * (size_t)s->ntri));
        A(alloc(s, &s->vlist_body, 9 * (size_t)s->ntri));
        A(alloc(s, &s->pmi, s->nbodies));
        A(alloc(s, &s->tri_ref, 9 * (size_t)s->ntri));
        A(alloc(s, &s->tbound, (size_t)s->ntri));
        A(alloc(s, &s->trec, (size_t)s->ntri));
        A(alloc(s, &s->tcells, (size_t)s->ntri + 1));
        A(alloc(s, &s->tpk, s->tpair_cap));
        A(alloc(s, &s->tpt, s->tpair_cap));
        char* tscr = nullptr;
        A(alloc(s, &tscr, radix_sort_scratch_bytes(s->tpair_cap)));
        s->tsort_scratch = tscr;
        A(alloc(s, &s->tcount, n));
        A(alloc(s, &s->tlist, n * s->tcap));
        A(alloc(s, &s->rxn, (size_t)6 * s->nbodies * n));
        A(alloc(s, &s->rxn_part, (size_t)6 * s->nbodies * kRxnBlocks));
        if (st == XD_OK) {
            A(cuda_status(cudaMemcpy(s->poly, d.poly, sizeof(xd_polygon_info) * s->ntri, cudaMemcpyHostToDevice), "mixed mesh"));
            A(cuda_status(cudaMemcpy(s->sphere, d.sphere, sizeof(double) * 4 * s->ntri, cudaMemcpyHostToDevice), "mixed mesh"));
            A(cuda_status(cudaMemcpy(s->vlist_body, d.vlist, sizeof(double) * 9 * s->ntri, cudaMemcpyHostToDevice), "mixed mesh"));
            A(cuda_status(cudaMemcpy(s->pmi, d.pmi, sizeof(xd_polygon_mass_info) * s->nbodies, cudaMemcpyHostToDevice), "mixed mesh"));
            A(launch_tri_records(s->poly, s->ntri, s->trec, 0));
            A(cuda_status(cudaStreamSynchronize(0), "mixed mesh"));
        }
    }
    return st;
}

int mixed_create(const xd_scene_desc& d, MixedScene** out)
{
    *out = nullptr;
    if (d.ntri && (!d.poly || !d.sphere || !d.vlist || !d.pmi || !d.cp_poly || !d.nbodies))
        return set_error(XD_ERR_INVALID, "mixed mode: triangles given without mesh arrays");
    if (d.ntri && d.nbodies > (unsigned)kMaxBodies)
        return set_error(XD_ERR_INVALID, "mixed mode: at most %d polygon bodies", kMaxBodies);
    for (unsigned t = 0; t < d.ntri; ++t)
        if (d.poly[t].id < 0 || (unsigned)d.poly[t].id >= d.nbodies)
            return set_error(XD_ERR_INVALID, "mixed mode: triangle %u names body %d of %u", t, d.poly[t].id,
                             d.nbodies);
    if (d.nplanes > (unsigned)kMaxPlanes)
        return set_error(XD_ERR_INVALID, "mixed mode: at most %d planes", kMaxPlanes);
    if (d.nplanes && (!d.planes || !d.cp_planes))
        return set_error(XD_ERR_INVALID, "mixed mode: planes given without arrays");
    for (unsigned w = 0; w < d.nplanes; ++w)
        if (d.cp_planes[w].coh != 0.0)
            return set_error(XD_ERR_INVALID,
                             "mixed mode: plane cohesion is not supported (plane %u; the reference's plane "
                             "kernel forms it with zero radii and moduli)", w);
    MixedScene* s = new (std::nothrow) MixedScene();
    if (!s) return set_error(XD_ERR_NOMEM, "mixed scene: host allocation");
    s->desc = d;
    // XDEM_NO_GRAPHS=1: launch every kernel directly (the host reads the
    // re-binning flag each step), so that a profiler sees each kernel
    const char* ng = getenv("XDEM_NO_GRAPHS");
    s->use_graphs = !(ng && ng[0] && ng[0] != '0');
    s->host_planes.assign(d.planes, d.planes + d.nplanes);
    s->host_cps.assign(d.cp_planes, d.cp_planes + d.nplanes);
    s->desc.planes = s->host_planes.data();
    s->desc.cp_planes = s->host_cps.data();
    if (d.ntri) {
        s->host_poly.assign(d.poly, d.poly + d.ntri);
        s->host_sphere.assign(d.sphere, d.sphere + 4 * (size_t)d.ntri);
        s->host_vlist.assign(d.vlist, d.vlist + 9 * (size_t)d.ntri);
        s->host_pmi.assign(d.pmi, d.pmi + d.nbodies);
        s->host_cppoly.assign(d.cp_poly, d.cp_poly + d.nbodies);
    }
    s->desc.poly = s->host_poly.data();
    s->desc.sphere = s->host_sphere.data();
    s->desc.vlist = s->host_vlist.data();
    s->desc.pmi = s->host_pmi.data();
    s->desc.cp_poly = s->host_cppoly.data();
    *out = s;
    return XD_OK;
}

void mixed_destroy(MixedScene* s)
{
    if (!s) return;
    cudaDeviceSynchronize();
    for (int k = 0; k < 5; ++k)
        if (s->graph[k]) cudaGraphExecDestroy(s->graph[k]);
    for (void* p : s->allocs) cudaFree(p);
    delete s;
}

static int ensure_xfer(MixedScene* s)
{
    if (s->xfer) return XD_OK;
    return alloc(s, &s->xfer, (size_t)s->cap * (4 + 3 * 6 + 2));
}

static int reset_history(MixedScene* s, cudaStream_t q);

// Host <-> transfer-buffer copies of several arrays: arrays the caller keeps
// back to back in the buffer's own order go as one copy (a null host array
// is skipped and ends a run).
struct CopyPart {
    double* dev;
    double* host;
    size_t count;
};

static int copy_runs(const CopyPart* parts, int k, bool to_device, cudaStream_t q, const char* what)
{
    int st = XD_OK;
    for (int a = 0; a < k && st == XD_OK;) {
        if (!parts[a].host || !parts[a].count) {
            ++a;
            continue;
        }
        int e = a + 1;
        size_t n = parts[a].count;
        while (e < k && parts[e].host && parts[e].host == parts[a].host + n && parts[e].dev == parts[a].dev + n) {
            n += parts[e].count;
            ++e;
        }
        st = cuda_status(to_device ? cudaMemcpyAsync(parts[a].dev, parts[a].host, sizeof(double) * n,
                                                     cudaMemcpyHostToDevice, q)
                                   : cudaMemcpyAsync(parts[a].host, parts[a].dev, sizeof(double) * n,
                                                     cudaMemcpyDeviceToHost, q),
                         what);
        a = e;
    }
    return st;
}

int mixed_upload(MixedScene* s, const double* pos, const double* vel, const double* acc,
                 const double* omega, const double* alpha, const double* mass,
                 const double* inertia, cudaStream_t q, bool sync)
{
    if (!pos || !vel || !acc || !omega || !alpha || !mass || !inertia)
        return set_error(XD_ERR_INVALID, "mixed mode: upload needs pos, vel, acc, omega, alpha, mass, inertia");
    if (!s->ready) {
        int r = mixed_setup(s, s->desc, pos);
        if (r != XD_OK) return r;
        s->ready = true;
        if (s->active_req != ~0u) {   // an emitter set before the first upload
            s->n = s->active_req;
            s->P.n = s->active_req;
            s->active_req = ~0u;
        }
    }
    int st = ensure_xfer(s);
    if (st != XD_OK) return st;
    size_t n = s->cap;   // every held particle, emitted or not
    double* b = s->xfer;
    double *dpos = b, *dvel = b + 4 * n, *dacc = dvel + 3 * n, *dom = dacc + 3 * n,
           *dal = dom + 3 * n, *dm = dal + 3 * n, *dI = dm + n;
    const CopyPart parts[7] = { { dpos, const_cast<double*>(pos), 4 * n },   { dvel, const_cast<double*>(vel), 3 * n },
                                { dacc, const_cast<double*>(acc), 3 * n },   { dom, const_cast<double*>(omega), 3 * n },
                                { dal, const_cast<double*>(alpha), 3 * n },  { dm, const_cast<double*>(mass), n },
                                { dI, const_cast<double*>(inertia), n } };
    st = copy_runs(parts, 7, true, q, "mixed upload");
    if (st != XD_OK) return st;
    s->cur = 0;
    s->cells_clean = false;   // the state is in upload order again: the next step re-bins
    st = reset_history(s, q);   // an uploaded state starts with no springs
    if (st == XD_OK && s->nbodies)   // nor unflushed body reactions
        st = cuda_status(cudaMemsetAsync(s->rxn, 0, sizeof(double) * 6 * s->nbodies * (size_t)s->cap, q),
                         "mixed upload");
    if (st != XD_OK) return st;
    st = cuda_status(cudaMemsetAsync(s->counters, 0, sizeof(unsigned) * CN_DECISIONS, q), "mixed upload");
    if (st != XD_OK) return st;
    MixParams Pc = s->P;
    Pc.n = s->cap;
    k_mx_load<<<blocks(s->cap, 256), 256, 0, q>>>(Pc, s->m[0], dpos, dvel, dacc, dom, dal, dm, dI,
                                                  s->mass0, s->pf, s->qa, s->qb, s->pr);
    st = launch_status("mixed upload");
    if (st == XD_OK && sync) st = cuda_status(cudaStreamSynchronize(q), "mixed upload");
    return st;
}

int mixed_download(MixedScene* s, double* pos, double* vel, double* acc, double* omega,
                   double* alpha, double* force, double* moment, cudaStream_t q, bool sync)
{
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    int st = ensure_xfer(s);
    if (st != XD_OK) return st;
    size_t n = s->cap;
    double* b = s->xfer;
    double *dpos = b, *dvel = b + 4 * n, *dacc = dvel + 3 * n, *dom = dacc + 3 * n,
           *dal = dom + 3 * n, *df = dal + 3 * n, *dmo = df + 3 * n;
    // xfer holds 4n + 18n + 2n doubles: pos, vel, acc, omega, alpha, force, moment fit in 22n
    MixParams Pc = s->P;
    Pc.n = s->cap;
    k_mx_store<<<blocks(s->cap, 256), 256, 0, q>>>(Pc, s->m[s->cur], s->mass0, dpos, dvel, dacc, dom,
                                                   dal, df, dmo);
    st = launch_status("mixed download");
    const CopyPart parts[7] = { { dpos, pos, 4 * n }, { dvel, vel, 3 * n },  { dacc, acc, 3 * n },
                                { dom, omega, 3 * n }, { dal, alpha, 3 * n }, { df, force, 3 * n },
                                { dmo, moment, 3 * n } };
    if (st == XD_OK) st = copy_runs(parts, 7, false, q, "mixed download");
    if (st == XD_OK && sync) st = cuda_status(cudaStreamSynchronize(q), "mixed download");
    return st;
}

// Re-binning: cell keys of the current positions, stable radix sort, the
// state permuted into the new order, the cell lower bounds, then the Verlet
// lists, plane masks and heavy list.
static HistTable history_table(MixedScene* s)
{
    HistTable h;
    h.key = s->hkey;
    h.delta = s->hdelta;
    h.slots = s->hslots;
    h.n = s->cap;   // row stride: the tables hold every particle
    h.overflow = s->hoverflow;
    return h;
}

// Re-binning with history: the tables follow their particles (new slot i
// takes old slot perm[i]); the partner keys are original indices and stay.
__global__ void __launch_bounds__(256) k_hist_permute(unsigned n, unsigned stride, unsigned slots,
                                                      const unsigned* __restrict__ perm,
                                                      const unsigned* __restrict__ key, const double* __restrict__ delta,
                                                      unsigned* __restrict__ key2, double* __restrict__ delta2)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned o = __ldg(perm + i);
    for (unsigned s = 0; s < slots; ++s) {
        const size_t a = (size_t)s * stride + i, b = (size_t)s * stride + o;
        key2[a] = __ldg(key + b);
        delta2[3 * a + 0] = __ldg(delta + 3 * b + 0);
        delta2[3 * a + 1] = __ldg(delta + 3 * b + 1);
        delta2[3 * a + 2] = __ldg(delta + 3 * b + 2);
    }
}

// Rows [0, n) of every slot's table (row stride `stride`) back from key2/delta2.
__global__ void __launch_bounds__(256) k_hist_copy(unsigned n, unsigned stride, unsigned slots,
                                                   const unsigned* __restrict__ key2,
                                                   const double* __restrict__ delta2, unsigned* __restrict__ key,
                                                   double* __restrict__ delta)
{
    const size_t e = (size_t)slots * n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < e; t += (size_t)gridDim.x * blockDim.x) {
        const size_t a = (t / n) * stride + t % n;
        key[a] = key2[a];
        delta[3 * a + 0] = delta2[3 * a + 0];
        delta[3 * a + 1] = delta2[3 * a + 1];
        delta[3 * a + 2] = delta2[3 * a + 2];
    }
}

// The tables in original order (diagnostic download): row id of the output
// takes slot i, id = the particle's original index.
__global__ void __launch_bounds__(256) k_hist_gather(unsigned n, unsigned slots, Master M,
                                                     const unsigned* __restrict__ key,
                                                     const double* __restrict__ delta, unsigned* __restrict__ okey,
                                                     double* __restrict__ odelta)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned id = __float_as_uint(M.wl[i].w);
    for (unsigned s = 0; s < slots; ++s) {
        const size_t a = (size_t)s * n + i, b = (size_t)s * n + id;
        okey[b] = key[a];
        odelta[3 * b + 0] = delta[3 * a + 0];
        odelta[3 * b + 1] = delta[3 * a + 1];
        odelta[3 * b + 2] = delta[3 * a + 2];
    }
}

// The reactions accumulated in the per-particle slots since the last flush
// go to the bodies (the slots belong to particle slots, which a re-binning
// reorders).
// The tables of slots [0, n) follow the permutation (new slot -> old slot).
static int permute_history(MixedScene* s, unsigned n, const unsigned* perm, cudaStream_t q)
{
    k_hist_permute<<<blocks(n, 256), 256, 0, q>>>(n, s->cap, s->hslots, perm, s->hkey, s->hdelta, s->hkey2,
                                                  s->hdelta2);
    int st = launch_status("mixed history re-binning");
    if (st != XD_OK) return st;
    const size_t e = (size_t)s->hslots * n;
    k_hist_copy<<<(unsigned)std::min<size_t>((e + 255) / 256, 152 * 16), 256, 0, q>>>(n, s->cap, s->hslots, s->hkey2,
                                                                                     s->hdelta2, s->hkey, s->hdelta);
    return launch_status("mixed history re-binning");
}

// inv[id of slot i] = i over all held slots: the permutation back to id order.
__global__ void __launch_bounds__(256) k_mx_inverse(unsigned cap, Master M, unsigned* __restrict__ inv)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    inv[__float_as_uint(M.wl[i].w)] = i;
}

static int flush_reactions(MixedScene* s, cudaStream_t q);

// Every held particle back to slot = id (the order an upload leaves), with
// its history rows; the cells must be re-binned afterwards.
static int restore_id_order(MixedScene* s, cudaStream_t q)
{
    const unsigned cap = s->cap;
    if (!cap) return XD_OK;
    int st = flush_reactions(s, q);   // the reaction slots belong to the old order
    if (st != XD_OK) return st;
    MixParams Pc = s->P;
    Pc.n = cap;
    k_mx_inverse<<<blocks(cap, 256), 256, 0, q>>>(cap, s->m[0], s->vals);
    k_mx_permute<<<blocks(cap, 256), 256, 0, q>>>(Pc, s->m[0], s->m[1], s->vals);
    k_mx_copyback<<<blocks(cap, 256), 256, 0, q>>>(Pc, s->m[1], s->m[0], s->pf, s->qa, s->qb, s->pr);
    st = launch_status("mixed id order");
    if (st == XD_OK && s->hslots) st = permute_history(s, cap, s->vals, q);
    s->cells_clean = false;
    return st;
}

static int flush_reactions(MixedScene* s, cudaStream_t q)
{
    if (!s->nbodies || !s->n) return XD_OK;
    k_rxn_sum<<<rxn_grid(s->n), kRxnThreads, 0, q>>>(s->rxn, s->n, s->nbodies, s->rxn_part, s->counters, s->pmi);
    return launch_status("mixed body reaction");
}

// The triangles' cell table: every triangle registered in each cell its
// box widened by the reach covers, as (cell, triangle) pairs sorted by cell,
// and the vertices it was built with (the moved-vertex test's reference).
static int build_tri_table(MixedScene* s, cudaStream_t q)
{
    const unsigned T = s->ntri, cap = s->tpair_cap;
    k_tri_count<<<blocks(T + 1, 256), 256, 0, q>>>(s->P, s->poly, s->tcells, s->tri_ref, s->tbound);
    k_scan1<<<1, 1024, 0, q>>>(s->tcells, T + 1);
    k_tri_fill<<<blocks(T, 256), 256, 0, q>>>(s->P, s->poly, s->tcells, cap, s->tpk, s->tpt);
    k_tri_pad<<<blocks(cap, 256), 256, 0, q>>>(s->tcells, T, cap, s->ncell, s->tpk, s->tpt);
    int st = launch_status("mixed triangle cells");
    unsigned *tk = nullptr, *tt = nullptr;
    if (st == XD_OK)
        st = radix_sort_pairs(s->tpk, s->tpt, cap, key_bits_for(s->ncell + 1), s->tsort_scratch, q, &tk, &tt);
    if (st != XD_OK) return st;
    s->tpk_sorted = tk;
    s->tpt_sorted = tt;
    return XD_OK;
}

static int rebuild(MixedScene* s, cudaStream_t q)
{
    const unsigned n = s->n;
    int st = flush_reactions(s, q);
    if (st != XD_OK) return st;
    st = cuda_status(cudaMemsetAsync(s->counters + CN_GAPS, 0, 2 * sizeof(unsigned), q), "mixed re-binning");
    if (st == XD_OK)
        st = cuda_status(cudaMemsetAsync(s->counters + CN_HTRI, 0, 2 * sizeof(unsigned), q), "mixed re-binning");
    if (st == XD_OK)
        st = cuda_status(cudaMemsetAsync(s->counters + CN_VINC, 0, 4 * sizeof(unsigned), q), "mixed re-binning");
    if (st != XD_OK) return st;
    k_mx_keys<<<blocks(n, 256), 256, 0, q>>>(s->P, s->pf, s->keys, s->vals);
    st = launch_status("mixed keys");
    if (st != XD_OK) return st;
    unsigned *sk = nullptr, *sv = nullptr;
    st = radix_sort_pairs(s->keys, s->vals, n, key_bits_for(s->ncell), s->sort_scratch, q, &sk, &sv);
    if (st != XD_OK) return st;
    k_mx_permute<<<blocks(n, 256), 256, 0, q>>>(s->P, s->m[0], s->m[1], sv);
    k_mx_copyback<<<blocks(n, 256), 256, 0, q>>>(s->P, s->m[1], s->m[0], s->pf, s->qa, s->qb, s->pr);
    if (s->hslots) {
        st = permute_history(s, n, sv, q);
        if (st != XD_OK) return st;
    }
    k_lb_fill<<<blocks(n + 1, 256), 256, 0, q>>>(sk, n, s->ncell, s->lb, s->prev_keys, s->gaps, s->counters);
    k_lb_long<<<152 * 4, 256, 0, q>>>(s->gaps, s->counters, s->lb);
    st = launch_status("mixed re-binning");
    if (st == XD_OK && s->ntri) {
        // triangles: the (cell, triangle) table -- here for meshes that move
        // on the device; the host keeps a static mesh's table (update_mesh)
        // -- then each particle's list
        if (s->kinematic) st = build_tri_table(s, q);
        if (st != XD_OK) return st;
        k_tri_build<<<blocks(n, 256), 256, 0, q>>>(s->P, s->pf, s->prev_keys, s->tpk_sorted, s->tpt_sorted,
                                                   s->tpair_cap, s->tri_ref, s->tbound, s->tcount, s->tlist,
                                                   s->counters);
        st = launch_status("mixed triangle lists");
    }
    if (st != XD_OK) return st;
    k_mx_build<<<blocks(n, 256), 256, 0, q>>>(s->P, s->pf, s->prev_keys, s->lb, s->vcount, s->vlist, s->pref,
                                              s->wmask, s->tcount, s->rxn, s->hlist, s->Fc, s->Mc,
                                              s->counters);
    return launch_status("mixed re-binning");
}

// Moves the triangles to the bodies' current poses (after xd_scene_set_bodies)
// and raises the re-binning flag if a vertex moved half the skin since the
// last build.  Runs before a step's advance.
static int update_mesh(MixedScene* s, cudaStream_t q)
{
    if (!s->ntri) return XD_OK;
    int st = XD_OK;
    if (s->bodies_dirty) {
        st = launch_mesh_move(s->pmi, s->vlist_body, s->sphere, s->poly, s->ntri, s->tri_ref, s->P.wo,
                              s->P.disp2, s->counters + CN_REBUILD, s->trec, q);
        if (st != XD_OK) return st;
        s->bodies_dirty = false;
        if (!s->kinematic) s->tri_table_dirty = true;
    }
    // A mesh that moves only between calls keeps its cell table out of the
    // re-binning: built here when it has moved (and after an upload), with a
    // re-binning of the lists forced, so that the moved-vertex reference and
    // the lists stay those of one build.
    if (!s->kinematic && s->tri_table_dirty) {
        st = build_tri_table(s, q);
        if (st != XD_OK) return st;
        s->tri_table_dirty = false;
        s->cells_clean = false;
    }
    return XD_OK;
}

// Inside a stream capture: a conditional node that runs body(s, stream) when
// the handle is set (by k_mx_keys); the capture continues after it.
template <typename Body>
static int capture_conditional(MixedScene* s, cudaStream_t q, cudaGraphConditionalHandle h, Body body)
{
    cudaStreamCaptureStatus cst;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    int st = cuda_status(cudaStreamGetCaptureInfo(q, &cst, nullptr, &g, &deps, nullptr, &nd), "mixed capture info");
    if (st != XD_OK) return st;
    cudaGraphNodeParams np = { cudaGraphNodeTypeConditional };
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    st = cuda_status(cudaGraphAddNode(&node, g, deps, nullptr, nd, &np), "mixed conditional node");
    if (st != XD_OK) return st;
    cudaStream_t bs = nullptr;
    st = cuda_status(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking), "mixed conditional stream");
    if (st != XD_OK) return st;
    st = cuda_status(cudaStreamBeginCaptureToGraph(bs, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeThreadLocal), "mixed conditional capture");
    if (st == XD_OK) {
        int r = body(s, bs);
        cudaGraph_t body_graph = nullptr;
        st = cuda_status(cudaStreamEndCapture(bs, &body_graph), "mixed conditional capture");
        if (r != XD_OK) st = r;
    }
    cudaStreamDestroy(bs);
    if (st != XD_OK) return st;
    return cuda_status(cudaStreamUpdateCaptureDependencies(q, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
                       "mixed capture dependencies");
}

// One step: the state advanced in place with the skin test, re-binning when
// a particle has left its skin (or the cells are not set up), then the
// contact forces.  cond: the conditional handle when capturing into a graph
// (nullptr for direct launches, where the host reads the flag).
static ContactArgs contact_args(MixedScene* s, unsigned* rc, unsigned* rp, unsigned rec_cap, const HistTable& ht,
                                int rxn_on)
{
    ContactArgs C;
    C.M = s->m[0];
    C.pf = s->pf;
    C.qa = s->qa;
    C.qb = s->qb;
    C.pr = s->pr;
    C.keys = s->prev_keys;
    C.lb = s->lb;
    C.vcount = s->vcount;
    C.vlist = s->vlist;
    C.hlist = s->hlist;
    C.wmask = s->wmask;
    C.planes = s->planes;
    C.prec = s->prec;
    C.mass0 = s->mass0;
    C.poly = s->poly;
    C.trec = s->trec;
    C.pmi = s->pmi;
    C.tcount = s->tcount;
    C.tlist = s->tlist;
    C.tpk = s->tpk_sorted;
    C.tpt = s->tpt_sorted;
    C.tcap = s->tpair_cap;
    C.rxn = s->rxn;
    C.Fc = s->Fc;
    C.Mc = s->Mc;
    C.counters = s->counters;
    C.rec_count = rc;
    C.rec_pairs = rp;
    C.rec_cap = rec_cap;
    C.ht = ht;
    C.rxn_on = rxn_on;
    return C;
}

template <int MODE>
static int step_once(MixedScene* s, cudaStream_t q, const Phases& ph, bool record, unsigned rec_cap,
                     const cudaGraphConditionalHandle* cond)
{
    const unsigned n = s->n;
    const Master& M = s->m[0];
    int st = XD_OK;
    if (s->kinematic && s->ntri && MODE != 3) {
        // prescribed body motion: pose, triangles, and the re-binning flag
        // once a vertex has moved half the skin since the last build
        st = launch_body_advance(s->pmi, s->nbodies, s->P.dt, q);
        if (st == XD_OK)
            st = launch_mesh_move(s->pmi, s->vlist_body, s->sphere, s->poly, s->ntri, s->tri_ref, s->P.wo,
                                  s->P.disp2, s->counters + CN_REBUILD, s->trec, q);
        if (st != XD_OK) return st;
    }
    ph.begin(0, q);
    k_mx_advance<MODE><<<blocks(n, 256), 256, 0, q>>>(s->P, M, s->Fc, s->Mc, s->pref, s->pf, s->qa, s->qb, s->pr,
                                                      s->counters, cond ? *cond : 0, cond ? 1 : 0);
    st = launch_status("mixed advance");
    ph.end(0, q);
    if (st != XD_OK) return st;
    ph.begin(2, q);
    if (cond) {
        st = capture_conditional(s, q, *cond, rebuild);
    } else {
        bool need = !s->cells_clean;
        if (!need) {
            unsigned flag = 0;
            st = cuda_status(cudaMemcpyAsync(&flag, s->counters + CN_REBUILD, sizeof(unsigned),
                                             cudaMemcpyDeviceToHost, q), "mixed re-binning flag");
            if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "mixed re-binning flag");
            need = flag != 0;
        }
        if (st == XD_OK && need) st = rebuild(s, q);
    }
    ph.end(2, q);
    if (st != XD_OK) return st;
    s->cells_clean = true;
    ph.begin(3, q);
    // the list holds at most n particles: no more warps than that
    const unsigned ct = s->cthreads;
    const unsigned grid = std::max(1u, std::min(kContactWarpsTotal * 32u / ct, (n + ct - 1) / ct));
    // tangential springs: updated by a step, read only by the diagnostic evaluation (MODE 3)
    const HistTable ht = history_table(s);
    const int hist = s->hslots ? (MODE == 3 ? 2 : 1) : 0;
    unsigned* rc = nullptr;
    unsigned* rp = nullptr;
    if (record) {
        st = cuda_status(cudaMemsetAsync(s->rec_count, 0, sizeof(unsigned) * n, q), "mixed pair count");
        if (st != XD_OK) return st;
        rc = s->rec_count;
        rp = s->rec_pairs;
    }
    const ContactArgs C = contact_args(s, rc, rp, record ? rec_cap : 0u, ht, MODE == 3 ? 0 : 1);
#define XD_MX_CONTACT(REC, H) k_mx_contact<REC, H, false><<<grid, ct, 0, q>>>(s->P, C)
    if (record) {
        if (hist == 2) XD_MX_CONTACT(true, 2);
        else if (hist == 1) XD_MX_CONTACT(true, 1);
        else XD_MX_CONTACT(true, 0);
    } else {
        if (hist == 2) XD_MX_CONTACT(false, 2);
        else if (hist == 1) XD_MX_CONTACT(false, 1);
        else if (s->cmode == 1) {
            k_mx_contact<false, 0, true><<<grid, ct, (ct / 32u) * sizeof(PairBuf), q>>>(s->P, C);
            if (s->P.nplanes || s->P.ntri) k_mx_walls<<<grid, ct, (ct / 32u) * sizeof(WallBuf), q>>>(s->P, C);
        } else XD_MX_CONTACT(false, 0);
    }
#undef XD_MX_CONTACT
    st = launch_status("mixed contact");
    ph.end(3, q);
    return st;
}

// Step graphs of a scene: kFirstStep (the first step of a call, MODE 0) and
// graphs of 1, 2, 4 and 8 middle steps (MODE 1), each step with its own
// conditional re-binning node; a call replays the first step, then runs of
// eight, then the binary digits of what is left.
enum { kFirstStep = 0, kSteps1 = 1, kSteps2 = 2, kSteps4 = 3, kSteps8 = 4, kGraphKinds = 5 };

static unsigned graph_steps(int kind) { return kind == kFirstStep ? 1u : 1u << (kind - 1); }

constexpr unsigned kGraphMinSteps = 16;

static void destroy_graphs(MixedScene* s)
{
    ++s->version;   // batches holding this scene capture it again
    for (int k = 0; k < kGraphKinds; ++k)
        if (s->graph[k]) {
            cudaGraphExecDestroy(s->graph[k]);
            s->graph[k] = nullptr;
        }
}

static int capture_steps(MixedScene* s, int kind)
{
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "mixed graph stream");
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int st = cuda_status(e, "mixed graph capture");
    cudaGraph_t cg = nullptr;
    cudaGraphConditionalHandle h[8] = {};
    if (st == XD_OK) {
        cudaStreamCaptureStatus cst;
        st = cuda_status(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg), "mixed capture info");
    }
    const unsigned nh = graph_steps(kind);
    for (unsigned k = 0; k < nh && st == XD_OK; ++k)
        st = cuda_status(cudaGraphConditionalHandleCreate(&h[k], cg, 0, cudaGraphCondAssignDefault),
                         "mixed conditional handle");
    const bool clean = s->cells_clean;
    Phases none;
    for (unsigned k = 0; k < nh && st == XD_OK; ++k)
        st = kind == kFirstStep ? step_once<0>(s, cs, none, false, 0, &h[k]) : step_once<1>(s, cs, none, false, 0, &h[k]);
    s->cells_clean = clean;   // capture only recorded the launches
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    if (st == XD_OK) st = cuda_status(e, "mixed graph capture");
    if (st == XD_OK) st = cuda_status(cudaGraphInstantiate(&s->graph[kind], g, 0), "mixed graph instantiate");
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    return st;
}

static int launch_steps(MixedScene* s, int kind, cudaStream_t q)
{
    if (!s->graph[kind]) {
        int st = capture_steps(s, kind);
        if (st != XD_OK) return st;
    }
    return cuda_status(cudaGraphLaunch(s->graph[kind], q), "mixed graph launch");
}

int mixed_step(MixedScene* s, unsigned nsteps, cudaStream_t q, const Phases& ph)
{
    if (nsteps == 0) return XD_OK;
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    if (s->n == 0) {
        // no particle emitted yet: only the prescribed body motion; the
        // emission that follows re-bins, triangles included
        if (!s->kinematic || !s->ntri) return XD_OK;
        int st = XD_OK;
        for (unsigned t = 0; t < nsteps && st == XD_OK; ++t) {
            st = launch_body_advance(s->pmi, s->nbodies, s->P.dt, q);
            if (st == XD_OK) st = launch_update_polygon(s->pmi, s->vlist_body, s->sphere, s->poly, s->ntri, q);
        }
        if (st == XD_OK) st = launch_tri_records(s->poly, s->ntri, s->trec, q);
        s->cells_clean = false;
        return st;
    }
    int st = update_mesh(s, q);
    if (st != XD_OK) return st;
    // graphs pay for their capture over many steps: a short call on a scene
    // whose graphs an emission has just dropped (its particle count changed)
    // launches directly
    const bool graphs = s->use_graphs && ph.fn == nullptr &&
                        (!s->emitted || s->graph[kFirstStep] || nsteps >= kGraphMinSteps);
    if (graphs) {
        // Every step in a graph, re-binning decided on the device: the call
        // never waits for the GPU.  A scene without cells yet (after an
        // upload) is made to re-bin through the same flag.
        // all step graphs are captured at the first call, so that later calls
        // of any length only replay
        for (int kind = 0; kind < kGraphKinds && st == XD_OK; ++kind)
            if (!s->graph[kind]) st = capture_steps(s, kind);
        if (st == XD_OK && !s->cells_clean)
            st = cuda_status(cudaMemsetAsync(s->counters + CN_REBUILD, 1, 1, q), "mixed re-binning flag");
        if (st == XD_OK) st = launch_steps(s, kFirstStep, q);
        unsigned left = nsteps - 1;
        for (; st == XD_OK && left >= 8; left -= 8) st = launch_steps(s, kSteps8, q);
        for (int kind = kSteps4; kind >= kSteps1 && st == XD_OK; --kind)
            if (left & graph_steps(kind)) st = launch_steps(s, kind, q);
        if (st != XD_OK) return st;
        s->cells_clean = true;
    } else {
        // direct launches (phase timing): the host reads the re-binning flag
        st = step_once<0>(s, q, ph, false, 0, nullptr);
        for (unsigned t = 1; t < nsteps && st == XD_OK; ++t) st = step_once<1>(s, q, ph, false, 0, nullptr);
        if (st != XD_OK) return st;
    }
    // the last velocity update, and the call's body reactions
    ph.begin(0, q);
    k_mx_finish<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[0], s->Fc, s->Mc);
    st = launch_status("mixed finish");
    ph.end(0, q);
    if (st == XD_OK) {
        ph.begin(3, q);
        st = flush_reactions(s, q);
        ph.end(3, q);
    }
    return st;
}

unsigned long long mixed_launches(MixedScene* s, unsigned nsteps)
{
    if (!s || nsteps == 0 || s->n == 0) return 0;
    // per step: advance + contact; + the last velocity update; a step that
    // re-bins adds mixed_rebuild_launches()
    // (and the wall pass after a cooperative pair pass)
    const unsigned long long per = 2 + (s->kinematic && s->ntri ? 3 : 0) +
                                   (s->cmode == 1 && (s->P.nplanes || s->P.ntri) ? 1 : 0);
    unsigned long long total = per * nsteps + 1 + (s->nbodies ? 1 : 0);
    if (!s->cells_clean) total += mixed_rebuild_launches(s);   // the first step re-bins
    return total;
}

unsigned long long mixed_rebuild_launches(MixedScene* s)
{
    if (!s || s->n == 0) return 0;
    // keys, sort, permute, copy back, cell bounds (2), list build; with
    // triangles also their lists, and for a mesh that moves on the device
    // its cell table (count, scan, fill, pad and their sort)
    unsigned long long k = (s->n > 1 ? 5ull * s->passes : 0ull) + 6;
    if (s->ntri) k += 1 + (s->kinematic ? 4 + 5ull * ((key_bits_for(s->ncell + 1) + 7) / 8) : 0ull);
    if (s->nbodies) k += 1;   // the reactions flushed first
    return k;
}

int mixed_rebuilds(MixedScene* s, unsigned long long* out, cudaStream_t q)
{
    unsigned c = 0;
    int st = cuda_status(cudaMemcpyAsync(&c, s->counters + CN_REBUILDS, sizeof(unsigned), cudaMemcpyDeviceToHost, q),
                         "rebuilds");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "rebuilds");
    *out = c;
    return st;
}

// Contacts of the current state: keys of the current positions, re-binning
// if needed, and the gather without an update.
static int current_contacts(MixedScene* s, cudaStream_t q, bool record, unsigned rec_cap)
{
    if (!s->n) return XD_OK;   // nothing emitted yet
    Phases none;
    int st = update_mesh(s, q);
    if (st != XD_OK) return st;
    return step_once<3>(s, q, none, record, rec_cap, nullptr);
}

int mixed_eval_contacts(MixedScene* s, double* force, double* moment, cudaStream_t q)
{
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    int st = ensure_xfer(s);
    if (st == XD_OK) st = current_contacts(s, q, false, 0);
    if (st != XD_OK) return st;
    size_t n = s->cap;
    double *df = s->xfer, *dm = s->xfer + 3 * n;
    if (s->n < s->cap)   // particles not emitted yet: zero rows
        st = cuda_status(cudaMemsetAsync(df, 0, sizeof(double) * 6 * n, q), "eval");
    if (st != XD_OK) return st;
    if (s->n) {
        k_mx_store_forces<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->Fc, s->Mc, df, dm);
        st = launch_status("mixed store forces");
    }
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
    if (!s->rec_count) st = alloc(s, &s->rec_count, s->cap);
    if (st == XD_OK && s->rec_cap_alloc < cap_per_particle) {
        st = alloc(s, &s->rec_pairs, (size_t)s->cap * cap_per_particle);
        s->rec_cap_alloc = cap_per_particle;
    }
    if (st == XD_OK) st = current_contacts(s, q, true, cap_per_particle);
    if (st != XD_OK) return st;
    // counts/partners are reported in original particle ids
    size_t n = s->n;
    k_mx_ids<<<blocks(s->n, 256), 256, 0, q>>>(s->P, s->m[s->cur], s->vals);
    st = launch_status("pairs");
    std::vector<unsigned> ids(n), cnt(n), part((size_t)n * cap_per_particle);
    if (st == XD_OK) st = cuda_status(cudaMemcpyAsync(ids.data(), s->vals, 4 * n, cudaMemcpyDeviceToHost, q), "pairs");
    if (st == XD_OK) st = cuda_status(cudaMemcpyAsync(cnt.data(), s->rec_count, 4 * n, cudaMemcpyDeviceToHost, q), "pairs");
    if (st == XD_OK)
        st = cuda_status(cudaMemcpyAsync(part.data(), s->rec_pairs, 4 * n * cap_per_particle, cudaMemcpyDeviceToHost, q), "pairs");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "pairs");
    if (st != XD_OK) return st;
    for (size_t o = n; o < s->cap; ++o) counts[o] = 0;   // not emitted yet
    for (size_t i = 0; i < n; ++i) {
        unsigned o = ids[i];
        counts[o] = cnt[i];
        unsigned c = cnt[i] < cap_per_particle ? cnt[i] : cap_per_particle;
        for (unsigned k = 0; k < c; ++k) partners[(size_t)o * cap_per_particle + k] = ids[part[i * cap_per_particle + k]];
    }
    return XD_OK;
}

int mixed_set_bodies(MixedScene* s, const xd_polygon_mass_info* pmi, cudaStream_t q)
{
    if (!s->ntri) return set_error(XD_ERR_STATE, "scene_set_bodies: scene has no polygon bodies");
    if (!s->ready) {
        // before the first upload: the set-up takes the bodies from the description
        s->host_pmi.assign(pmi, pmi + s->nbodies);
        s->desc.pmi = s->host_pmi.data();
        return XD_OK;
    }
    int st = cuda_status(cudaMemcpyAsync(s->pmi, pmi, sizeof(xd_polygon_mass_info) * s->nbodies,
                                         cudaMemcpyHostToDevice, q), "scene_set_bodies");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_set_bodies");
    s->bodies_dirty = true;
    return st;
}

// FP32 prefilter copies of the planes (corner relative to the grid origin,
// unit normal) in the step parameters.
static void plane_prefilter(MixParams& P, const xd_plane_info* planes, unsigned nplanes)
{
    for (unsigned w = 0; w < nplanes; ++w) {
        const xd_plane_info& p = planes[w];
        const double un = sqrt(p.uw[0] * p.uw[0] + p.uw[1] * p.uw[1] + p.uw[2] * p.uw[2]);
        for (int a = 0; a < 3; ++a) {
            P.pxw[w][a] = (float)(p.xw[a] - P.wo[a]);
            P.pun[w][a] = (float)(p.uw[a] / un);
        }
    }
}

int mixed_set_planes(MixedScene* s, const xd_plane_info* planes, cudaStream_t q)
{
    s->host_planes.assign(planes, planes + s->nplanes);
    s->desc.planes = s->host_planes.data();
    if (!s->ready) return XD_OK;   // the set-up takes them from the description
    int st = cuda_status(cudaMemcpyAsync(s->planes, planes, sizeof(xd_plane_info) * s->nplanes,
                                         cudaMemcpyHostToDevice, q), "scene_set_planes");
    if (st == XD_OK) st = launch_plane_recs(s->planes, s->nplanes, s->prec, q);
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_set_planes");
    plane_prefilter(s->P, planes, s->nplanes);
    s->cells_clean = false;   // the planes in reach of each particle change
    destroy_graphs(s);        // the step graphs hold the prefilter copies
    return st;
}

int mixed_get_bodies(MixedScene* s, xd_polygon_mass_info* pmi, cudaStream_t q)
{
    if (!s->ntri) return set_error(XD_ERR_STATE, "scene_get_bodies: scene has no polygon bodies");
    if (!s->ready) {
        std::copy(s->host_pmi.begin(), s->host_pmi.end(), pmi);
        return XD_OK;
    }
    int st = cuda_status(cudaMemcpyAsync(pmi, s->pmi, sizeof(xd_polygon_mass_info) * s->nbodies,
                                         cudaMemcpyDeviceToHost, q), "scene_get_bodies");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_get_bodies");
    return st;
}

unsigned long long mixed_device_bytes(MixedScene* s) { return s ? s->bytes : 0; }

static int reset_history(MixedScene* s, cudaStream_t q)
{
    if (!s->hslots) return XD_OK;
    const size_t e = (size_t)s->hslots * s->desc.np;
    int st = cuda_status(cudaMemsetAsync(s->hkey, 0xff, sizeof(unsigned) * e, q), "mixed history");
    if (st == XD_OK) st = cuda_status(cudaMemsetAsync(s->hdelta, 0, sizeof(double) * 3 * e, q), "mixed history");
    if (st == XD_OK) st = cuda_status(cudaMemsetAsync(s->hoverflow, 0, sizeof(unsigned long long), q), "mixed history");
    return st;
}

int mixed_set_active(MixedScene* s, unsigned active, bool restore, cudaStream_t q)
{
    if (active > s->desc.np) return set_error(XD_ERR_INVALID, "scene emitter: active count above the particle count");
    if (!s->ready) {   // applied by the first upload
        s->active_req = active;
        return XD_OK;
    }
    int st = restore ? restore_id_order(s, q) : flush_reactions(s, q);
    if (st != XD_OK || active == s->n) return st;
    s->n = active;
    s->P.n = active;
    s->cells_clean = false;
    // the step graphs hold the particle count: replaced once the launches
    // queued from them have run
    if (s->graph[kFirstStep]) st = cuda_status(cudaStreamSynchronize(q), "scene emitter");
    destroy_graphs(s);
    s->emitted = true;
    return st;
}

unsigned mixed_active(MixedScene* s) { return s->ready ? s->n : (s->active_req != ~0u ? s->active_req : s->desc.np); }

int mixed_set_tuning(MixedScene* s, const xd_tuning* t)
{
    if (s->ready) return set_error(XD_ERR_STATE, "scene_set_tuning: set before the first upload");
    if (!(t->skin_factor >= 0.02f && t->skin_factor <= 1.0f))
        return set_error(XD_ERR_INVALID, "scene_set_tuning: skin factor %g outside [0.02, 1]", (double)t->skin_factor);
    if (t->verlet_cap < 8 || t->verlet_cap > 256)
        return set_error(XD_ERR_INVALID, "scene_set_tuning: Verlet capacity %u outside [8, 256]", t->verlet_cap);
    if (t->triangle_cap < 4 || t->triangle_cap > 128)
        return set_error(XD_ERR_INVALID, "scene_set_tuning: triangle capacity %u outside [4, 128]", t->triangle_cap);
    if (t->contact_threads != 32 && t->contact_threads != 64 && t->contact_threads != 128)
        return set_error(XD_ERR_INVALID, "scene_set_tuning: contact block of %u threads (32, 64 or 128)",
                         t->contact_threads);
    if (t->contact_mode > 1)
        return set_error(XD_ERR_INVALID, "scene_set_tuning: contact mode %u (0 or 1)", t->contact_mode);
    s->cmode = t->contact_mode;
    s->skin_factor = t->skin_factor;
    s->vcap = t->verlet_cap;
    s->tcap = t->triangle_cap;
    s->cthreads = t->contact_threads;
    return XD_OK;
}

void mixed_get_tuning(const MixedScene* s, xd_tuning* t)
{
    t->skin_factor = s->skin_factor;
    t->verlet_cap = s->vcap;
    t->triangle_cap = s->tcap;
    t->contact_threads = s->cthreads;
    t->contact_mode = s->cmode;
}

int mixed_set_kinematic(MixedScene* s, bool enable)
{
    if (enable && !s->desc.ntri) return set_error(XD_ERR_STATE, "scene_set_kinematic_bodies: no polygon bodies");
    if (enable != s->kinematic) destroy_graphs(s);   // the step graphs hold the step's launches
    if (!enable && s->kinematic) s->tri_table_dirty = true;
    s->kinematic = enable;
    return XD_OK;
}

int mixed_set_history(MixedScene* s, unsigned slots)
{
    if (slots == s->hslots) {
        int st = reset_history(s, nullptr);
        if (st == XD_OK) st = cuda_status(cudaDeviceSynchronize(), "mixed history");
        return st;
    }
    destroy_graphs(s);   // the step graphs hold the table pointers: capture them again
    s->hslots = 0;
    const unsigned n = s->desc.np;   // the particle count (set before the first upload too)
    if (slots == 0 || n == 0) return XD_OK;
    const size_t e = (size_t)slots * n;
    int st = XD_OK;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    A(alloc(s, &s->hkey, e));
    A(alloc(s, &s->hdelta, 3 * e));
    A(alloc(s, &s->hkey2, e));
    A(alloc(s, &s->hdelta2, 3 * e));
    A(alloc(s, &s->hoverflow, 1));
    if (st != XD_OK) return st;
    s->hslots = slots;
    st = reset_history(s, nullptr);
    if (st == XD_OK) st = cuda_status(cudaDeviceSynchronize(), "mixed history");
    return st;
}

int mixed_download_history(MixedScene* s, unsigned* keys, double* delta, unsigned long long* overflow,
                           cudaStream_t q)
{
    if (!s->hslots) return set_error(XD_ERR_STATE, "scene_download_history: history is off");
    if (!s->ready) return set_error(XD_ERR_STATE, "mixed mode: no state uploaded");
    const size_t e = (size_t)s->hslots * s->cap;
    unsigned* ok = nullptr;
    double* od = nullptr;
    int st = cuda_status(cudaMalloc(&ok, sizeof(unsigned) * e), "scene_download_history");
    if (st == XD_OK) st = cuda_status(cudaMalloc(&od, sizeof(double) * 3 * e), "scene_download_history");
    if (st == XD_OK) {
        k_hist_gather<<<blocks(s->cap, 256), 256, 0, q>>>(s->cap, s->hslots, s->m[0], s->hkey, s->hdelta, ok, od);
        st = launch_status("scene_download_history");
    }
    if (st == XD_OK && keys)
        st = cuda_status(cudaMemcpyAsync(keys, ok, sizeof(unsigned) * e, cudaMemcpyDeviceToHost, q), "scene_download_history");
    if (st == XD_OK && delta)
        st = cuda_status(cudaMemcpyAsync(delta, od, sizeof(double) * 3 * e, cudaMemcpyDeviceToHost, q),
                         "scene_download_history");
    if (st == XD_OK && overflow)
        st = cuda_status(cudaMemcpyAsync(overflow, s->hoverflow, sizeof(unsigned long long), cudaMemcpyDeviceToHost, q),
                         "scene_download_history");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_download_history");
    if (ok) cudaFree(ok);
    if (od) cudaFree(od);
    return st;
}

int mixed_counters(MixedScene* s, unsigned long long* out, cudaStream_t q)
{
    unsigned c[kCounters] = {};
    int st = cuda_status(cudaMemcpyAsync(c, s->counters, sizeof(c), cudaMemcpyDeviceToHost, q), "counters");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "counters");
    out[0] = c[CN_HEAVY];
    out[1] = c[CN_DECISIONS];
    out[2] = c[CN_NORMALS];
    out[3] = c[CN_SLIPS];
    return st;
}

int mixed_stats(MixedScene* s, unsigned long long* out, cudaStream_t q)
{
    unsigned c[kCounters] = {};
    int st = cuda_status(cudaMemcpyAsync(c, s->counters, sizeof(c), cudaMemcpyDeviceToHost, q), "scene_stats");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_stats");
    out[0] = c[CN_HEAVY];
    out[1] = c[CN_DECISIONS];
    out[2] = c[CN_NORMALS];
    out[3] = c[CN_SLIPS];
    out[4] = c[CN_WALLS];
    out[5] = c[CN_REBUILDS];
    out[6] = c[CN_HTRI];
    out[7] = c[CN_VINC];
    out[8] = c[CN_TINC];
    out[9] = c[CN_VSUM];
    out[10] = c[CN_TSUM];
    return st;
}

// ---- batches: many mixed scenes advanced by shared launches ----------------
//
// A step of a batch is one graph: one advance launch over every scene's
// slots, one decision kernel that reads each scene's re-binning flag, a
// conditional node per group of kBatchGroup scenes whose body holds a
// conditional re-binning per scene of the group, and one contact launch over
// every scene's listed particles.  Each scene runs the same per-slot code as
// when stepped alone (advance_one, rebuild, contact_entry, finish_one), so its
// results are the same bits; what changes is that a step costs a handful of
// graph nodes instead of three per scene (a conditional node costs a few
// microseconds of the GPU's front end whether or not its body runs).

namespace {

constexpr unsigned kBatchGroup = 32;
constexpr unsigned kBatchGraphSteps = 4;   // later steps captured per graph launch
constexpr unsigned kBatchGrab = 2;         // runs of 32 listed particles a contact warp takes at a time


// One scene of a batch as the batch kernels read it.
struct BatchScene {
    MixParams P;
    ContactArgs C;
    const float4* pref;
    float4* pf;
    longlong2* qa;
    longlong2* qb;
    float4* pr;
    unsigned adv_block0;   // first block of this scene in the advance grid
};

// per-warp copy of the scene a warp of the contact launch works on
struct WarpScene {
    MixParams P;
    ContactArgs C;
};

__device__ __forceinline__ void copy_words(void* dst, const void* src, unsigned bytes, unsigned t, unsigned nt)
{
    const unsigned* a = static_cast<const unsigned*>(src);
    unsigned* b = static_cast<unsigned*>(dst);
    for (unsigned k = t; k < bytes / 4u; k += nt) b[k] = __ldg(a + k);
}

// MODE 0: drift; MODE 1: kick then drift; MODE 2: kick only (the finish).
template <int MODE>
__global__ void __launch_bounds__(256) k_batch_advance(const BatchScene* __restrict__ D,
                                                       const unsigned* __restrict__ block_scene, unsigned nblocks)
{
    __shared__ MixParams sP;
    if (blockIdx.x >= nblocks) return;
    const unsigned sc = __ldg(block_scene + blockIdx.x);
    const BatchScene& d = D[sc];
    copy_words(&sP, &d.P, sizeof(MixParams), threadIdx.x, blockDim.x);
    __syncthreads();
    const unsigned i = (blockIdx.x - d.adv_block0) * blockDim.x + threadIdx.x;
    if (MODE == 2) {
        if (i < sP.n) finish_one(sP, d.C.M, d.C.Fc, d.C.Mc, i);
        return;
    }
    const bool out = i < sP.n && advance_one<MODE>(sP, d.C.M, d.C.Fc, d.C.Mc, d.pref, d.pf, d.qa, d.qb, d.pr, i);
    if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31u) == 0) atomicOr(d.C.counters + CN_REBUILD, 1u);
}

// Each scene's re-binning flag into flags[] (and cleared for the next step);
// the groups with a flagged scene open their conditional node.
__global__ void __launch_bounds__(256) k_batch_decide(const BatchScene* __restrict__ D, unsigned ns,
                                                      unsigned* __restrict__ flags,
                                                      const cudaGraphConditionalHandle* __restrict__ hg)
{
    __shared__ unsigned any[256];
    const unsigned ng = (ns + kBatchGroup - 1u) / kBatchGroup;
    for (unsigned g = threadIdx.x; g < 256u; g += blockDim.x) any[g] = 0;
    __syncthreads();
    for (unsigned sc = threadIdx.x; sc < ns; sc += blockDim.x) {
        unsigned* c = D[sc].C.counters;
        const unsigned f = c[CN_REBUILD] ? 1u : 0u;
        c[CN_REBUILD] = 0;
        flags[sc] = f;
        if (f) atomicOr(&any[(sc / kBatchGroup) & 255u], 1u);
    }
    __syncthreads();
    if (hg)   // inside the step graph (the direct path reads flags[] on the host)
        for (unsigned g = threadIdx.x; g < ng && g < 256u; g += blockDim.x)
            if (any[g]) cudaGraphSetConditional(hg[g], 1u);
}

// Inside a group's body: the flagged scenes of the group open their re-binning.
__global__ void k_batch_group(const unsigned* __restrict__ flags, unsigned first, unsigned count,
                              const cudaGraphConditionalHandle* __restrict__ hs)
{
    const unsigned t = threadIdx.x;
    if (t < count && flags[first + t]) cudaGraphSetConditional(hs[first + t], 1u);
}

// Runs of 32 listed particles per scene, as an exclusive prefix over scenes,
// of counter word `cw` (CN_HEAVY: every listed particle; CN_HTRI: those with
// walls in reach) into runs[0, ns]; runs[ns + 1] (the launch's next free
// run) cleared.
__device__ void batch_runs(const BatchScene* __restrict__ D, unsigned ns, unsigned cw, unsigned* __restrict__ runs,
                           unsigned* c, unsigned& carry)
{
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (unsigned base = 0; base < ns; base += 1024u) {
        const unsigned sc = base + threadIdx.x;
        const unsigned h = sc < ns ? D[sc].C.counters[cw] : 0u;
        c[threadIdx.x] = (h + 31u) / 32u;
        __syncthreads();
        // inclusive scan (Hillis-Steele)
        for (unsigned off = 1; off < 1024u; off <<= 1) {
            const unsigned v = threadIdx.x >= off ? c[threadIdx.x - off] : 0u;
            __syncthreads();
            c[threadIdx.x] += v;
            __syncthreads();
        }
        if (sc < ns) runs[sc + 1] = carry + c[threadIdx.x];
        __syncthreads();
        if (threadIdx.x == 0) carry += c[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        runs[0] = 0;
        runs[ns + 1] = 0;
    }
    __syncthreads();
}

// The runs of the contact launch (chunk_start) and of the wall launch
// (chunk_start + ns + 2).
__global__ void __launch_bounds__(1024) k_batch_chunks(const BatchScene* __restrict__ D, unsigned ns,
                                                       unsigned* __restrict__ chunk_start)
{
    __shared__ unsigned c[1024];
    __shared__ unsigned carry;
    batch_runs(D, ns, CN_HEAVY, chunk_start, c, carry);
    batch_runs(D, ns, CN_HTRI, chunk_start + ns + 2, c, carry);
}

// The contact pass of every scene: each warp takes the next kBatchGrab runs
// of all scenes' lists from a counter (chunk_start[ns + 1], cleared by
// k_batch_chunks) until none are left, so that warps that drew cheap runs
// take more; a run's result does not depend on which warp computes it.  A
// warp loads the scene of a run into its own shared-memory slot when the
// scene changes.
// Shared-memory bytes of a batch contact block's WarpScene slots (rounded to
// 16 bytes: the per-warp buffers follow).
__host__ __device__ constexpr unsigned batch_scene_bytes(unsigned nwarps)
{
    return (unsigned)((nwarps * sizeof(WarpScene) + 15u) / 16u * 16u);
}

// KIND 0: the per-particle contact pass; 1: the cooperative pair pass; 2:
// the wall pass (runs over the front of each scene's list).
template <int KIND>
__global__ void __launch_bounds__(kContactMaxThreads) k_batch_contact(const BatchScene* __restrict__ D, unsigned ns,
                                                                   unsigned* __restrict__ chunk_start)
{
    // dynamic shared memory: one WarpScene per warp of the block, then (the
    // cooperative kinds) one PairBuf or WallBuf per warp
    extern __shared__ __align__(16) unsigned char batch_smem[];
    const unsigned lane = threadIdx.x & 31u, wb = threadIdx.x / 32u, nwarps = blockDim.x / 32u;
    WarpScene& W = reinterpret_cast<WarpScene*>(batch_smem)[wb];
    unsigned char* const bufs = batch_smem + batch_scene_bytes(nwarps);
    const unsigned total = __ldg(chunk_start + ns);
    unsigned* next = chunk_start + ns + 1;
    unsigned cur = 0xffffffffu, lo = 0, heavy = 0, front = 0;
    for (;;) {
    unsigned c0 = 0;
    if (lane == 0) c0 = atomicAdd(next, kBatchGrab);
    c0 = __shfl_sync(0xffffffffu, c0, 0);
    if (c0 >= total) break;
    const unsigned c1 = min(total, c0 + kBatchGrab);
    for (unsigned ch = c0; ch < c1; ++ch) {
        if (cur == 0xffffffffu || ch >= __ldg(chunk_start + cur + 1)) {
            // the scene holding run ch: the last s with chunk_start[s] <= ch
            unsigned a = 0, b = ns;
            while (b - a > 1u) {
                const unsigned m = (a + b) / 2u;
                if (__ldg(chunk_start + m) <= ch) a = m;
                else b = m;
            }
            cur = a;
            lo = __ldg(chunk_start + cur);
            __syncwarp();
            copy_words(&W.P, &D[cur].P, sizeof(MixParams), lane, 32u);
            copy_words(&W.C, &D[cur].C, sizeof(ContactArgs), lane, 32u);
            __syncwarp();
            heavy = W.C.counters[CN_HEAVY];
            front = W.C.counters[CN_HTRI];
        }
        const unsigned t = (ch - lo) * 32u + lane;
        if (KIND == 1) {
            const bool valid = t < heavy;
            contact_entry_coop(W.P, W.C, valid, valid ? __ldg(W.C.hlist + list_index(t, front, W.P.n)) : 0u,
                               reinterpret_cast<PairBuf*>(bufs)[wb]);
        } else if (KIND == 2) {
            const bool valid = t < front;
            walls_entry_coop(W.P, W.C, valid, valid ? __ldg(W.C.hlist + t) : 0u,
                             reinterpret_cast<WallBuf*>(bufs)[wb]);
        } else if (t < heavy) {
            contact_entry<false, 0>(W.P, W.C, __ldg(W.C.hlist + list_index(t, front, W.P.n)));
        }
    }
    }
}

}  // namespace

struct MixedBatch {
    std::vector<MixedScene*> scenes;
    std::vector<unsigned> versions;
    BatchScene* d_scenes = nullptr;
    unsigned* d_block_scene = nullptr;
    unsigned nblocks = 0;
    unsigned* d_flags = nullptr;
    unsigned* d_chunks = nullptr;
    cudaGraphConditionalHandle* d_handles[3] = {};   // per graph kind and step: groups, then scenes
    cudaGraphExec_t step_graph[3] = {};              // 0: first step of a call (drift); 1: one later step;
                                                     // 2: kBatchGraphSteps later steps
    cudaGraphExec_t finish_graph = nullptr;          // last kick and the body reactions
    bool captured = false;
    unsigned cthreads = kContactThreads;             // block size of the shared contact launch
    unsigned cmode = kContactMode;                   // its pair pass (the first scene's choice)
    bool walls = false;                              // a scene has planes or triangles (a wall pass)
    // direct launches (profilers; kernel timing): CUDA events around the
    // later steps' advance and every contact launch
    bool direct = false;
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> spans;
    double ms[3] = {};                               // advance, pair pass, wall pass
    unsigned long long launches[3] = {};
};

// The batch's contact launch: every scene's listed particles.
static void launch_batch_pairs(const MixedBatch* b, unsigned ns, cudaStream_t q)
{
    const unsigned ct = b->cthreads, grid = kContactWarpsTotal * 32u / ct, w = ct / 32u;
    if (b->cmode == 1)
        k_batch_contact<1><<<grid, ct, batch_scene_bytes(w) + w * sizeof(PairBuf), q>>>(b->d_scenes, ns,
                                                                                         b->d_chunks);
    else
        k_batch_contact<0><<<grid, ct, batch_scene_bytes(w), q>>>(b->d_scenes, ns, b->d_chunks);
}

// The wall pass after a cooperative pair pass (none otherwise: the
// per-particle pass does its walls itself).
static void launch_batch_walls(const MixedBatch* b, unsigned ns, cudaStream_t q)
{
    const unsigned ct = b->cthreads, grid = kContactWarpsTotal * 32u / ct, w = ct / 32u;
    if (b->cmode == 1 && b->walls)
        k_batch_contact<2><<<grid, ct, batch_scene_bytes(w) + w * sizeof(WallBuf), q>>>(b->d_scenes, ns,
                                                                                         b->d_chunks + ns + 2);
}

static void launch_batch_contact(const MixedBatch* b, unsigned ns, cudaStream_t q)
{
    launch_batch_pairs(b, ns, q);
    launch_batch_walls(b, ns, q);
}

namespace {

void free_batch_graphs(MixedBatch* b)
{
    for (auto& g : b->step_graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    if (b->finish_graph) cudaGraphExecDestroy(b->finish_graph);
    b->finish_graph = nullptr;
    for (auto& h : b->d_handles)
        if (h) {
            cudaFree(h);
            h = nullptr;
        }
    for (void* p : { (void*)b->d_scenes, (void*)b->d_block_scene, (void*)b->d_flags, (void*)b->d_chunks })
        if (p) cudaFree(p);
    b->d_scenes = nullptr;
    b->d_block_scene = nullptr;
    b->d_flags = nullptr;
    b->d_chunks = nullptr;
    b->captured = false;
}

// A conditional (if) node in graph g after deps; its body is captured from
// what body(stream, body_graph) launches.
template <typename Body>
int add_conditional(cudaGraph_t g, const cudaGraphNode_t* deps, size_t nd, cudaGraphConditionalHandle h, Body body,
                    cudaGraphNode_t* node)
{
    cudaGraphNodeParams np = { cudaGraphNodeTypeConditional };
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    int st = cuda_status(cudaGraphAddNode(node, g, deps, nullptr, nd, &np), "batch conditional node");
    if (st != XD_OK) return st;
    cudaGraph_t bg = np.conditional.phGraph_out[0];
    cudaStream_t bs = nullptr;
    st = cuda_status(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking), "batch conditional stream");
    if (st != XD_OK) return st;
    st = cuda_status(cudaStreamBeginCaptureToGraph(bs, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                     "batch conditional capture");
    if (st == XD_OK) {
        const int r = body(bs, bg);
        cudaGraph_t out = nullptr;
        st = cuda_status(cudaStreamEndCapture(bs, &out), "batch conditional capture");
        if (r != XD_OK) st = r;
    }
    cudaStreamDestroy(bs);
    return st;
}

int current_deps(cudaStream_t q, cudaGraph_t* g, std::vector<cudaGraphNode_t>* deps)
{
    cudaStreamCaptureStatus cst;
    const cudaGraphNode_t* d = nullptr;
    size_t nd = 0;
    int st = cuda_status(cudaStreamGetCaptureInfo(q, &cst, nullptr, g, &d, nullptr, &nd), "batch capture info");
    if (st == XD_OK) deps->assign(d, d + nd);
    return st;
}

// One batch step graph: advance, decision, the groups' conditional
// re-binnings (side by side), run prefix, contact.
int capture_batch_step(MixedBatch* b, int kind)
{
    const unsigned ns = (unsigned)b->scenes.size();
    const unsigned ng = (ns + kBatchGroup - 1) / kBatchGroup;
    const unsigned nsteps = kind == 2 ? kBatchGraphSteps : 1u;
    const unsigned per = ng + ns;   // handles of one step: groups, then scenes
    std::vector<cudaGraphConditionalHandle> h((size_t)per * nsteps, 0);
    cudaStream_t cs = nullptr;
    int st = cuda_status(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "batch capture stream");
    if (st != XD_OK) return st;
    st = cuda_status(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "batch capture");
    cudaGraph_t cg = nullptr;
    std::vector<cudaGraphNode_t> deps;
    if (st == XD_OK) st = current_deps(cs, &cg, &deps);
    for (unsigned step = 0; step < nsteps && st == XD_OK; ++step) {
        cudaGraphConditionalHandle* hs = h.data() + (size_t)step * per;
        cudaGraphConditionalHandle* dh = b->d_handles[kind] + (size_t)step * per;
        for (unsigned g = 0; g < ng && st == XD_OK; ++g)
            st = cuda_status(cudaGraphConditionalHandleCreate(&hs[g], cg, 0, cudaGraphCondAssignDefault),
                             "batch conditional handle");
        if (st == XD_OK) {
            if (kind == 0)
                k_batch_advance<0><<<b->nblocks, 256, 0, cs>>>(b->d_scenes, b->d_block_scene, b->nblocks);
            else
                k_batch_advance<1><<<b->nblocks, 256, 0, cs>>>(b->d_scenes, b->d_block_scene, b->nblocks);
            k_batch_decide<<<1, 256, 0, cs>>>(b->d_scenes, ns, b->d_flags, dh);
            st = launch_status("batch advance");
        }
        if (st == XD_OK) st = current_deps(cs, &cg, &deps);
        std::vector<cudaGraphNode_t> groups(ng, nullptr);
        for (unsigned g = 0; g < ng && st == XD_OK; ++g) {
            const unsigned first = g * kBatchGroup, count = std::min(kBatchGroup, ns - first);
            auto group_body = [&](cudaStream_t bs, cudaGraph_t bg) {
                int r = XD_OK;
                for (unsigned k = 0; k < count && r == XD_OK; ++k)
                    r = cuda_status(cudaGraphConditionalHandleCreate(&hs[ng + first + k], bg, 0,
                                                                     cudaGraphCondAssignDefault),
                                    "batch conditional handle");
                if (r != XD_OK) return r;
                k_batch_group<<<1, 32, 0, bs>>>(b->d_flags, first, count, dh + ng);
                r = launch_status("batch group");
                cudaGraph_t bgc = nullptr;
                std::vector<cudaGraphNode_t> gd;
                if (r == XD_OK) r = current_deps(bs, &bgc, &gd);
                for (unsigned k = 0; k < count && r == XD_OK; ++k) {
                    MixedScene* sc = b->scenes[first + k];
                    cudaGraphNode_t node = nullptr;
                    r = add_conditional(bgc, gd.data(), gd.size(), hs[ng + first + k],
                                        [sc](cudaStream_t rs, cudaGraph_t) { return rebuild(sc, rs); }, &node);
                }
                return r;
            };
            st = add_conditional(cg, deps.data(), deps.size(), hs[g], group_body, &groups[g]);
        }
        if (st == XD_OK && ng)
            st = cuda_status(cudaStreamUpdateCaptureDependencies(cs, groups.data(), nullptr, ng,
                                                                 cudaStreamSetCaptureDependencies),
                             "batch capture dependencies");
        if (st == XD_OK) {
            k_batch_chunks<<<1, 1024, 0, cs>>>(b->d_scenes, ns, b->d_chunks);
            launch_batch_contact(b, ns, cs);
            st = launch_status("batch contact");
        }
        if (st == XD_OK) st = current_deps(cs, &cg, &deps);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (st == XD_OK) st = cuda_status(e, "batch capture");
    if (st == XD_OK) st = cuda_status(cudaGraphInstantiate(&b->step_graph[kind], graph, 0), "batch graph instantiate");
    if (graph) cudaGraphDestroy(graph);
    if (st == XD_OK)
        st = cuda_status(cudaMemcpy(b->d_handles[kind], h.data(), sizeof(cudaGraphConditionalHandle) * h.size(),
                                    cudaMemcpyHostToDevice), "batch handles");
    if (st == XD_OK) st = cuda_status(cudaGraphUpload(b->step_graph[kind], cs), "batch graph upload");
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(cs), "batch graph upload");
    cudaStreamDestroy(cs);
    return st;
}

int capture_batch_finish(MixedBatch* b)
{
    cudaStream_t cs = nullptr;
    int st = cuda_status(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "batch capture stream");
    if (st != XD_OK) return st;
    st = cuda_status(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "batch capture");
    if (st == XD_OK) {
        k_batch_advance<2><<<b->nblocks, 256, 0, cs>>>(b->d_scenes, b->d_block_scene, b->nblocks);
        st = launch_status("batch finish");
    }
    // the scenes' body reactions side by side: branches forked from the kick
    constexpr int kBranches = 16;
    cudaStream_t br[kBranches] = {};
    cudaEvent_t ev[kBranches + 1] = {};
    for (int j = 0; j < kBranches && st == XD_OK; ++j)
        st = cuda_status(cudaStreamCreateWithFlags(&br[j], cudaStreamNonBlocking), "batch capture stream");
    for (int j = 0; j <= kBranches && st == XD_OK; ++j)
        st = cuda_status(cudaEventCreateWithFlags(&ev[j], cudaEventDisableTiming), "batch capture event");
    if (st == XD_OK) st = cuda_status(cudaEventRecord(ev[kBranches], cs), "batch capture fork");
    for (int j = 0; j < kBranches && st == XD_OK; ++j)
        st = cuda_status(cudaStreamWaitEvent(br[j], ev[kBranches], 0), "batch capture fork");
    for (size_t k = 0; k < b->scenes.size() && st == XD_OK; ++k)
        st = flush_reactions(b->scenes[k], br[k % kBranches]);
    for (int j = 0; j < kBranches && st == XD_OK; ++j) {
        st = cuda_status(cudaEventRecord(ev[j], br[j]), "batch capture join");
        if (st == XD_OK) st = cuda_status(cudaStreamWaitEvent(cs, ev[j], 0), "batch capture join");
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cs, &graph);
    for (int j = 0; j < kBranches; ++j)
        if (br[j]) cudaStreamDestroy(br[j]);
    for (int j = 0; j <= kBranches; ++j)
        if (ev[j]) cudaEventDestroy(ev[j]);
    if (st == XD_OK) st = cuda_status(e, "batch capture");
    if (st == XD_OK) st = cuda_status(cudaGraphInstantiate(&b->finish_graph, graph, 0), "batch graph instantiate");
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    return st;
}

// Device descriptors of the scenes as they are now, and the step graphs.
int prepare_batch(MixedBatch* b)
{
    free_batch_graphs(b);
    const unsigned ns = (unsigned)b->scenes.size();
    std::vector<BatchScene> hs(ns);
    std::vector<unsigned> block_scene;
    for (unsigned k = 0; k < ns; ++k) {
        MixedScene* sc = b->scenes[k];
        BatchScene& d = hs[k];
        memset(&d, 0, sizeof(d));
        d.P = sc->P;
        d.C = contact_args(sc, nullptr, nullptr, 0u, history_table(sc), 1);
        d.pref = sc->pref;
        d.pf = sc->pf;
        d.qa = sc->qa;
        d.qb = sc->qb;
        d.pr = sc->pr;
        d.adv_block0 = (unsigned)block_scene.size();
        block_scene.insert(block_scene.end(), blocks(sc->n, 256), k);
    }
    b->nblocks = (unsigned)block_scene.size();
    const unsigned ng = (ns + kBatchGroup - 1) / kBatchGroup;
    int st = XD_OK;
    auto M = [&](auto** p, size_t count, const char* what) {
        if (st == XD_OK) st = cuda_status(cudaMalloc(p, sizeof(**p) * (count ? count : 1)), what);
    };
    M(&b->d_scenes, ns, "batch scenes");
    M(&b->d_block_scene, block_scene.size(), "batch blocks");
    M(&b->d_flags, ns, "batch flags");
    M(&b->d_chunks, 2 * (ns + 2), "batch runs");
    M(&b->d_handles[0], ng + ns, "batch handles");
    M(&b->d_handles[1], ng + ns, "batch handles");
    M(&b->d_handles[2], (size_t)(ng + ns) * kBatchGraphSteps, "batch handles");
    if (st == XD_OK)
        st = cuda_status(cudaMemcpy(b->d_block_scene, block_scene.data(), sizeof(unsigned) * block_scene.size(),
                                    cudaMemcpyHostToDevice), "batch blocks");
    for (int kind = 0; kind < 3 && st == XD_OK; ++kind) st = capture_batch_step(b, kind);
    if (st == XD_OK) st = capture_batch_finish(b);
    // the descriptors after the captures: capturing a re-binning fixes the
    // triangle sort's output buffers of a scene that has not re-binned yet
    for (unsigned k = 0; k < ns && st == XD_OK; ++k) {
        MixedScene* sc = b->scenes[k];
        hs[k].C.tpk = sc->tpk_sorted;
        hs[k].C.tpt = sc->tpt_sorted;
    }
    if (st == XD_OK)
        st = cuda_status(cudaMemcpy(b->d_scenes, hs.data(), sizeof(BatchScene) * ns, cudaMemcpyHostToDevice),
                         "batch scenes");
    if (st != XD_OK) {
        free_batch_graphs(b);
        return st;
    }
    b->versions.resize(ns);
    for (unsigned k = 0; k < ns; ++k) b->versions[k] = b->scenes[k]->version;
    b->captured = true;
    return XD_OK;
}

}  // namespace

int mixed_batch_create(MixedScene* const* scenes, unsigned count, MixedBatch** out)
{
    *out = nullptr;
    if (count == 0 || count > 256u * kBatchGroup)
        return set_error(XD_ERR_INVALID, "batch: 1 to %u scenes", 256u * kBatchGroup);
    for (unsigned k = 0; k < count; ++k) {
        const MixedScene* sc = scenes[k];
        if (!sc->ready) return set_error(XD_ERR_STATE, "batch: scene %u has no state uploaded", k);
        if (sc->hslots) return set_error(XD_ERR_STATE, "batch: scene %u keeps tangential history", k);
        if (sc->kinematic) return set_error(XD_ERR_STATE, "batch: scene %u has kinematic bodies", k);
        for (unsigned j = 0; j < k; ++j)
            if (scenes[j] == sc) return set_error(XD_ERR_INVALID, "batch: scene %u given twice", k);
    }
    // the cooperative kinds' shared memory at the largest block: the wall
    // pass's is above the 48 KB a launch may take without asking
    {
        const unsigned w = kContactMaxThreads / 32u;
        int st = cuda_status(cudaFuncSetAttribute(k_batch_contact<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)(batch_scene_bytes(w) + w * sizeof(PairBuf))),
                             "batch pair pass shared memory");
        if (st == XD_OK)
            st = cuda_status(cudaFuncSetAttribute(k_batch_contact<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)(batch_scene_bytes(w) + w * sizeof(WallBuf))),
                             "batch wall pass shared memory");
        if (st != XD_OK) return st;
    }
    MixedBatch* b = new (std::nothrow) MixedBatch();
    if (!b) return set_error(XD_ERR_NOMEM, "batch: host allocation");
    b->scenes.assign(scenes, scenes + count);
    b->cthreads = scenes[0]->cthreads;   // the first scene's choices (one launch serves all)
    b->cmode = scenes[0]->cmode;
    for (unsigned k = 0; k < count; ++k) b->walls = b->walls || scenes[k]->P.nplanes || scenes[k]->P.ntri;
    const char* ng = getenv("XDEM_NO_GRAPHS");
    b->direct = ng && ng[0] && ng[0] != '0';
    *out = b;
    return XD_OK;
}

void mixed_batch_destroy(MixedBatch* b)
{
    if (!b) return;
    cudaDeviceSynchronize();   // steps queued from the batch's graphs run first
    free_batch_graphs(b);
    for (cudaEvent_t e : b->ev_pool) cudaEventDestroy(e);
    delete b;
}

namespace {

cudaEvent_t batch_event(MixedBatch* b, size_t k)
{
    while (b->ev_pool.size() <= k) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        b->ev_pool.push_back(e);
    }
    return b->ev_pool[k];
}

// The batch step by direct launches: the same kernels as the step graph, the
// re-binning flags read on the host after each advance.
int batch_step_direct(MixedBatch* b, unsigned nsteps, cudaStream_t q)
{
    const unsigned ns = (unsigned)b->scenes.size();
    std::vector<unsigned> flags(ns);
    size_t nev = 0;
    int st = XD_OK;
    auto span = [&](int kind, auto launch) {
        cudaEvent_t e0 = b->timing ? batch_event(b, nev++) : nullptr;
        cudaEvent_t e1 = b->timing ? batch_event(b, nev++) : nullptr;
        if (e0) cudaEventRecord(e0, q);
        launch();
        if (e1) cudaEventRecord(e1, q);
        if (e0 && e1) b->spans.push_back({ kind, { e0, e1 } });
    };
    for (unsigned t = 0; t < nsteps && st == XD_OK; ++t) {
        if (t == 0) {
            k_batch_advance<0><<<b->nblocks, 256, 0, q>>>(b->d_scenes, b->d_block_scene, b->nblocks);
        } else {
            span(0, [&] { k_batch_advance<1><<<b->nblocks, 256, 0, q>>>(b->d_scenes, b->d_block_scene, b->nblocks); });
        }
        k_batch_decide<<<1, 256, 0, q>>>(b->d_scenes, ns, b->d_flags, nullptr);
        st = launch_status("batch advance");
        if (st == XD_OK)
            st = cuda_status(cudaMemcpyAsync(flags.data(), b->d_flags, sizeof(unsigned) * ns, cudaMemcpyDeviceToHost, q),
                             "batch flags");
        if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "batch flags");
        for (unsigned k = 0; k < ns && st == XD_OK; ++k)
            if (flags[k]) st = rebuild(b->scenes[k], q);
        if (st != XD_OK) break;
        k_batch_chunks<<<1, 1024, 0, q>>>(b->d_scenes, ns, b->d_chunks);
        span(1, [&] { launch_batch_pairs(b, ns, q); });
        if (b->cmode == 1 && b->walls) span(2, [&] { launch_batch_walls(b, ns, q); });
        st = launch_status("batch contact");
    }
    if (st == XD_OK) {
        k_batch_advance<2><<<b->nblocks, 256, 0, q>>>(b->d_scenes, b->d_block_scene, b->nblocks);
        st = launch_status("batch finish");
    }
    for (unsigned k = 0; k < ns && st == XD_OK; ++k) st = flush_reactions(b->scenes[k], q);
    if (st == XD_OK && b->timing) {
        st = cuda_status(cudaStreamSynchronize(q), "batch timing");
        for (auto& sp : b->spans) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, sp.second.first, sp.second.second) == cudaSuccess) {
                b->ms[sp.first] += ms;
                b->launches[sp.first] += 1;
            }
        }
        b->spans.clear();
    }
    return st;
}

}  // namespace

int mixed_batch_set_timing(MixedBatch* b, bool enable)
{
    b->timing = enable;
    b->ms[0] = b->ms[1] = b->ms[2] = 0.0;
    b->launches[0] = b->launches[1] = b->launches[2] = 0;
    return XD_OK;
}

void mixed_batch_kernel_times(MixedBatch* b, double ms[3], unsigned long long launches[3])
{
    for (int k = 0; k < 3; ++k) {
        ms[k] = b->ms[k];
        launches[k] = b->launches[k];
    }
}

int mixed_batch_step(MixedBatch* b, unsigned nsteps, cudaStream_t q)
{
    if (nsteps == 0) return XD_OK;
    int st = XD_OK;
    // meshes moved and cell tables built first: the batch's capture takes the tables' addresses
    for (MixedScene* sc : b->scenes) {
        if (!sc->ready) return set_error(XD_ERR_STATE, "batch: a scene has no state uploaded");
        if (!sc->kinematic) st = update_mesh(sc, q);
        if (st != XD_OK) return st;
    }
    bool stale = !b->captured;
    for (size_t k = 0; k < b->scenes.size() && !stale; ++k) stale = b->versions[k] != b->scenes[k]->version;
    if (stale) {
        for (size_t k = 0; k < b->scenes.size(); ++k) {
            const MixedScene* sc = b->scenes[k];
            if (sc->hslots || sc->kinematic)
                return set_error(XD_ERR_STATE, "batch: scene %u now keeps history or kinematic bodies", (unsigned)k);
        }
        st = cuda_status(cudaStreamSynchronize(q), "batch");   // graphs in flight finish first
        b->walls = false;
        for (const MixedScene* sc : b->scenes) b->walls = b->walls || sc->P.nplanes || sc->P.ntri;
        if (st == XD_OK) st = prepare_batch(b);
        if (st != XD_OK) return st;
    }
    for (MixedScene* sc : b->scenes) {
        if (!sc->cells_clean)
            st = cuda_status(cudaMemsetAsync(sc->counters + CN_REBUILD, 1, 1, q), "batch re-binning flag");
        if (st != XD_OK) return st;
    }
    if (b->direct || b->timing) {
        st = batch_step_direct(b, nsteps, q);
    } else {
        st = cuda_status(cudaGraphLaunch(b->step_graph[0], q), "batch graph launch");
        unsigned left = nsteps - 1;
        for (; left >= kBatchGraphSteps && st == XD_OK; left -= kBatchGraphSteps)
            st = cuda_status(cudaGraphLaunch(b->step_graph[2], q), "batch graph launch");
        for (; left > 0 && st == XD_OK; --left)
            st = cuda_status(cudaGraphLaunch(b->step_graph[1], q), "batch graph launch");
        if (st == XD_OK) st = cuda_status(cudaGraphLaunch(b->finish_graph, q), "batch graph launch");
    }
    if (st != XD_OK) return st;
    for (MixedScene* sc : b->scenes) sc->cells_clean = true;
    return XD_OK;
}

}  // namespace xd
