// The legacy DEM interface of the reference (include/cu_dem_dec.cuh,
// launchers source/cu_dem_def.cu, kernels include/cu_dem_impl.cuh) on this
// library's own parts.  See include/xdem_legacy.h for the layouts and the
// reference behaviour kept on purpose.
//
// * Grid: the shared hash kernel and stable radix sort (the legacy hash call
//   hashes the np + nsp rows of the merged array and sorts the first np), and
//   the shared cell-range kernel over the sorted keys.
// * Contacts: one warp per particle walks the particle's 27 cells in the
//   reference's order (z, y, x), 32 candidates at a time, lane l taking the
//   cell's entries l, l + 32, ...  The pair law is the shared DHS model
//   (xd_physics64.cuh, with the legacy block's global kn, vn, ks, vs and mu),
//   of which a legacy particle keeps the normal force and the shear force's
//   moment; each lane sums its own contacts and the warp adds the lanes in a
//   fixed shuffle tree (the reference sums in search order: the two orders
//   differ in the last bits only).  The shape passes keep the first contact
//   in search order, found by a ballot over the lanes.
// * The shape call's force sum is the library's deterministic reduction.
//
// Compiled with --fmad=false.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../../include/xdem_legacy.h"
#include "xd_grid.cuh"
#include "xd_internal.cuh"
#include "xd_physics64.cuh"

static_assert(sizeof(xd_legacy_parameters) == 144, "legacy device_parameters layout");
static_assert(sizeof(xd_legacy_plane_info) == 160, "legacy device_plane_info layout");
static_assert(sizeof(xd_legacy_polygon) == 144, "cu_polygon layout");
static_assert(sizeof(xd_legacy_mass_info) == 48, "cu_mass_info layout");

namespace xd {
namespace {

std::mutex g_legacy_mu;
bool g_legacy_set = false;
xd_legacy_parameters g_legacy;

// The legacy block as the shared grid parameters plus its contact law.
struct Legacy {
    Params P;
    Fc law;          // global kn, vn, ks, vs, mu of the legacy block
    double coh;      // cohesive
};

bool legacy_block(Legacy* out)
{
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    if (!g_legacy_set) return false;
    const xd_legacy_parameters& h = g_legacy;
    Legacy L{};
    L.P.rolling = true;
    L.P.np = h.np;
    L.P.nsphere = h.nsp;
    L.P.ncell = h.ncell;
    L.P.gx = h.grid_size[0];
    L.P.gy = h.grid_size[1];
    L.P.gz = h.grid_size[2];
    L.P.dt = h.dt;
    L.P.half2dt = h.half2dt;
    L.P.cs = h.cell_size;
    L.P.cohesion = h.cohesive;
    for (int a = 0; a < 3; ++a) {
        L.P.g[a] = h.gravity[a];
        L.P.wo[a] = h.world_origin[a];
    }
    L.law = Fc{ h.kn, h.vn, h.ks, h.vs, h.mu };
    L.coh = h.cohesive;
    *out = L;
    return true;
}

// rows of the legacy state: double4 (x, y, z, w)
__device__ __forceinline__ d3 row4(const double* a, size_t i) { return ldv(a + 4 * i); }
__device__ __forceinline__ void set_row4(double* a, size_t i, d3 v)
{
    double* p = a + 4 * i;
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

// warp sums in a fixed order (the same bits every run)
__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ d3 warp_sum(d3 v) { return mk(warp_sum(v.x), warp_sum(v.y), warp_sum(v.z)); }

// Calls fn(k) for the grid entries of particle ip's 27 cells in the
// reference's order, lane l of the warp taking entries l, l + 32, ... of each
// cell; stop() (warp-uniform) ends the walk after a round of 32.
template <typename Fn, typename Stop>
__device__ __forceinline__ void warp_cells(const Params& P, d3 ip, const unsigned* __restrict__ sorted,
                                           const unsigned* __restrict__ cstart, const unsigned* __restrict__ cend,
                                           Fn fn, Stop stop)
{
    const unsigned lane = threadIdx.x & 31u;
    const int3 gp = grid_pos(P, ip.x, ip.y, ip.z);
    for (int z = -1; z <= 1; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                const unsigned h = grid_hash(P, gp.x + x, gp.y + y, gp.z + z);
                const unsigned st = __ldg(cstart + h);
                if (st == 0xffffffffu) continue;
                const unsigned en = __ldg(cend + h);
                for (unsigned base = st; base < en; base += 32u) {
                    const unsigned j = base + lane;
                    fn(j < en ? __ldg(sorted + j) : 0xffffffffu);
                    if (stop()) return;
                }
            }
}

// ------------------------------------------------------------ integrator

// vv_update_position_kernel (impl:93-107): x += dt v + half2dt a
__global__ void __launch_bounds__(256) k_legacy_drift(Params P, double* __restrict__ pos,
                                                      const double* __restrict__ vel,
                                                      const double* __restrict__ acc)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.np) return;
    set_row4(pos, i, row4(pos, i) + (P.dt * row4(vel, i) + P.half2dt * row4(acc, i)));
}

// vv_update_velocity_kernel (impl:109-140): two half kicks around the new
// accelerations a = F / acc.w and alpha = M / alpha.w; the rows' w keep the
// mass and inertia (vel.w and omega.w become 0)
__global__ void __launch_bounds__(256) k_legacy_kick(Params P, double* __restrict__ vel, double* __restrict__ acc,
                                                     double* __restrict__ omega, double* __restrict__ alpha,
                                                     const double* __restrict__ force,
                                                     const double* __restrict__ moment)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.np) return;
    const size_t q = 4 * (size_t)i;
    const double m = acc[q + 3], I = alpha[q + 3];
    const double h = 0.5 * P.dt;
    const d3 a1 = (1 / m) * ldv(force + 3 * (size_t)i), b1 = (1 / I) * ldv(moment + 3 * (size_t)i);
    const d3 v = (row4(vel, i) + h * row4(acc, i)) + h * a1;
    const d3 w = (row4(omega, i) + h * row4(alpha, i)) + h * b1;
    set_row4(vel, i, v);
    set_row4(omega, i, w);
    set_row4(acc, i, a1);
    set_row4(alpha, i, b1);
    vel[q + 3] = 0.0;
    omega[q + 3] = 0.0;
}

// ------------------------------------------------------------ contacts

// One legacy pair contact of particle i (radius ir) with j: the DHS model's
// normal force into F and its shear force's moment into M (calForce,
// impl:231-252).  The unit normal is relative_pos times 1 / dist as the
// legacy operators divide (impl:68-72).
__device__ __forceinline__ void legacy_pair(const Legacy& L, double ir, double jr, d3 ip, d3 jp, d3 iv, d3 jv,
                                            d3 iw, d3 jw, d3& F, d3& M)
{
    const d3 rp = jp - ip;
    const double dist = length(rp);
    const double cd = (ir + jr) - dist;
    const d3 unit = (1 / dist) * rp;
    const d3 rv = jv + cross(jw, -jr * unit) - (iv + cross(iw, ir * unit));
    if (cd > 0) {
        d3 Ft = mk(0, 0, 0), Fn, Mp = mk(0, 0, 0);
        dhs(L.law, ir, jr, 0, 0, 0, 0, 0.0, cd, rv, unit, L.P.dt, Ft, Fn, Mp);
        F += Fn;
        M += Mp;
        return;
    }
    if (L.coh == 0) return;
    // apart within the 27 cells with cohesion (impl:211-229): the cohesive
    // pull coh / mu along the normal when the would-be normal force lies in
    // (-coh / mu, 0), and a moment from the capped shear
    const Fc& c = L.law;
    const double pull = L.coh / c.mu;
    const double fn = -c.kn * pow(-cd, 1.5) + c.vn * dot(rv, unit);
    if (fn < 0 && fn > -pull) F += pull * unit;
    const d3 e = rv - dot(rv, unit) * unit;
    const double me = length(e);
    if (me != 0.0) {
        const d3 s = (1 / me) * e;
        const double fs = fmin(c.ks * (me * L.P.dt) + c.vs * dot(rv, s), c.mu * fn);
        if (fs < fn * c.mu + L.coh) M += cross(ir * unit, (fn * c.mu + L.coh) * s);
    }
}

// calculate_p2p_kernel (impl:254-327): force += m g + the normal forces of
// the particle's contacts, moment += the shear moments; one warp a particle.
__global__ void __launch_bounds__(256) k_legacy_p2p(Legacy L, const double* __restrict__ pos,
                                                    const double* __restrict__ vel, const double* __restrict__ acc,
                                                    const double* __restrict__ omega, double* __restrict__ force,
                                                    double* __restrict__ moment, const unsigned* __restrict__ sorted,
                                                    const unsigned* __restrict__ cstart,
                                                    const unsigned* __restrict__ cend)
{
    const unsigned id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (id >= L.P.np) return;
    const unsigned np = L.P.np;
    const d3 ip = row4(pos, id), iv = row4(vel, id), iw = row4(omega, id);
    const double ir = __ldg(pos + 4 * (size_t)id + 3);
    d3 F = mk(0, 0, 0), M = mk(0, 0, 0);
    warp_cells(
        L.P, ip, sorted, cstart, cend,
        [&](unsigned k) {
            if (k == 0xffffffffu || k == id || k >= np) return;
            legacy_pair(L, ir, __ldg(pos + 4 * (size_t)k + 3), ip, row4(pos, k), iv, row4(vel, k), iw,
                        row4(omega, k), F, M);
        },
        [] { return false; });
    F = warp_sum(F);
    M = warp_sum(M);
    if ((threadIdx.x & 31u) == 0) {
        const d3 g = __ldg(acc + 4 * (size_t)id + 3) * mk(L.P.g[0], L.P.g[1], L.P.g[2]);
        double* f = force + 3 * (size_t)id;
        double* m = moment + 3 * (size_t)id;
        const d3 t = g + F;
        f[0] += t.x; f[1] += t.y; f[2] += t.z;
        m[0] += M.x; m[1] += M.y; m[2] += M.z;
    }
}

// cube_hertzian_contact_force_kernel (impl:329-378): the face contacts of
// the six planes (the shared face-region test), each adding its normal
// force and its shear force's moment.
__global__ void __launch_bounds__(128) k_legacy_cube(Legacy L, const xd_legacy_plane_info* __restrict__ planes, Fc c,
                                                     const double* __restrict__ pos, const double* __restrict__ vel,
                                                     const double* __restrict__ omega, double* __restrict__ force,
                                                     double* __restrict__ moment)
{
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= L.P.np) return;
    const double r = __ldg(pos + 4 * (size_t)id + 3);
    const d3 ip = row4(pos, id), iv = row4(vel, id), iw = row4(omega, id);
    d3 F = mk(0, 0, 0), M = mk(0, 0, 0);
    for (int w = 0; w < 6; w++) {
        const xd_legacy_plane_info& pl = planes[w];
        PlaneD pe;
        pe.l1 = pl.l1;
        pe.l2 = pl.l2;
        pe.u1 = ldv(pl.u1);
        pe.u2 = ldv(pl.u2);
        pe.uw = ldv(pl.uw);
        pe.xw = ldv(pl.xw);
        if (!plane_face_region(pe, plane_coords(pe, ip), r)) continue;
        d3 unit;
        const double cd = plane_face_depth(pe, ip, unit, r);
        d3 Ft = mk(0, 0, 0), Fn, Mp = mk(0, 0, 0);
        dhs(c, r, 0, 0, 0, 0, 0, 0.0, cd, -(iv + cross(iw, r * unit)), unit, L.P.dt, Ft, Fn, Mp);
        F += Fn;
        M += Mp;
    }
    double* f = force + 3 * (size_t)id;
    double* m = moment + 3 * (size_t)id;
    f[0] += F.x; f[1] += F.y; f[2] += F.z;
    m[0] += M.x; m[1] += M.y; m[2] += M.z;
}

struct Shape {
    const xd_legacy_mass_info* mi;
    const xd_legacy_polygon* polygons;
    const unsigned* id_set;
    const unsigned* poly_start;
    const unsigned* poly_end;
    Fc law;
};

// The first contact of vertex entry k's polygons for the pass (face: the
// closest point in a face region; edge: at a vertex or an edge), its overlap
// and unit normal (face: -N / |N|; edge: towards the closest point).
__device__ __forceinline__ bool shape_candidate(const Params& P, const Shape& S, unsigned k, d3 ip, double r,
                                                bool face, double& cd, d3& unit)
{
    const unsigned v = k - P.np;
    for (unsigned q = __ldg(S.poly_start + v); q < __ldg(S.poly_end + v); q++) {
        const xd_legacy_polygon& po = S.polygons[__ldg(S.id_set + q)];
        int region;
        const d3 cpt = closest_pt_triangle_region(ldv(po.P), ldv(po.Q), ldv(po.R), ip, region);
        const d3 sp = ip - cpt;
        const double dist = length(sp);
        const double d = r - dist;
        if (d <= 0) continue;
        if (face ? region != 2 : region == 2) continue;
        cd = d;
        if (face) {
            const d3 N = ldv(po.N);
            unit = -((1 / length(N)) * N);
        } else {
            unit = -((1 / dist) * sp);
        }
        return true;
    }
    return false;
}

// shpae_hertzian_contact_force_kernel and shape_line_or_edge_contact_force_kernel
// (impl:454-674): the face pass takes each particle's first face contact in
// search order; the edge pass, for the particles the face pass left, the
// first edge or vertex contact.  The body moves with mi.vel; the particle
// keeps the normal force and the shear force's moment.
template <bool FACE>
__global__ void __launch_bounds__(256) k_legacy_shape(Legacy L, Shape S, bool* __restrict__ line,
                                                      const double* __restrict__ pos, const double* __restrict__ vel,
                                                      const double* __restrict__ omega, double* __restrict__ force,
                                                      double* __restrict__ moment, const unsigned* __restrict__ sorted,
                                                      const unsigned* __restrict__ cstart,
                                                      const unsigned* __restrict__ cend)
{
    const unsigned id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (id >= L.P.np) return;
    const unsigned lane = threadIdx.x & 31u;
    if (FACE) {
        if (lane == 0) line[id] = false;
    } else if (line[id]) {
        return;
    }
    const d3 ip = row4(pos, id);
    const double r = __ldg(pos + 4 * (size_t)id + 3);
    bool found = false;
    warp_cells(
        L.P, ip, sorted, cstart, cend,
        [&](unsigned k) {
            double cd = 0.0;
            d3 unit = mk(0, 0, 0);
            const bool hit = k != 0xffffffffu && k != id && k >= L.P.np &&
                             shape_candidate(L.P, S, k, ip, r, FACE, cd, unit);
            const unsigned bal = __ballot_sync(0xffffffffu, hit);
            if (!bal) return;
            found = true;
            if ((int)lane != __ffs(bal) - 1) return;
            const d3 iv = row4(vel, id), iw = row4(omega, id);
            const d3 dv = ldv(S.mi->vel) - (iv + cross(iw, r * unit));
            d3 Ft = mk(0, 0, 0), Fn, Mp = mk(0, 0, 0);
            dhs(S.law, r, 0, 0, 0, 0, 0, 0.0, cd, dv, unit, L.P.dt, Ft, Fn, Mp);
            double* f = force + 3 * (size_t)id;
            double* m = moment + 3 * (size_t)id;
            f[0] += Fn.x; f[1] += Fn.y; f[2] += Fn.z;
            m[0] += Mp.x; m[1] += Mp.y; m[2] += Mp.z;
            line[id] = true;
        },
        [&] { return found; });
}

// ------------------------------------------------------------ meshes

// cu_update_polygons_position (impl:764-780): v = mpos + A l
__global__ void __launch_bounds__(256) k_legacy_place(const double* __restrict__ mpos, const double* __restrict__ A,
                                                      const double* __restrict__ local, unsigned nv,
                                                      double* __restrict__ pos)
{
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nv) return;
    const d3 l = ldv(local + 3 * (size_t)id);
    const d3 t = mk(dot(ldv(A), l), dot(ldv(A + 3), l), dot(ldv(A + 6), l));
    st3(pos, id, ldv(mpos) + t);
}

// cu_update_polygons_information (impl:798-817): vertices, edges and the
// (unnormalised) normal of each polygon from its vertex indices
__global__ void __launch_bounds__(256) k_legacy_polygons(xd_legacy_polygon* __restrict__ polygons,
                                                         const unsigned* __restrict__ indice,
                                                         const double* __restrict__ pos, unsigned ni)
{
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ni) return;
    const d3 P = ldv(pos + 3 * (size_t)indice[3 * (size_t)id]);
    const d3 Q = ldv(pos + 3 * (size_t)indice[3 * (size_t)id + 1]);
    const d3 R = ldv(pos + 3 * (size_t)indice[3 * (size_t)id + 2]);
    xd_legacy_polygon& o = polygons[id];
    st3(o.P, 0, P);
    st3(o.Q, 0, Q);
    st3(o.R, 0, R);
    st3(o.V, 0, Q - P);
    st3(o.W, 0, R - P);
    st3(o.N, 0, cross(Q - P, R - P));
}

// cu_mergedata (impl:782-796): the particles' rows, then the vertices as (x, y, z, -1)
__global__ void __launch_bounds__(256) k_legacy_merge(double* __restrict__ data, const double* __restrict__ pos,
                                                      unsigned np, const double* __restrict__ vertice,
                                                      unsigned snp)
{
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np + snp) return;
    double* d = data + 4 * (size_t)id;
    if (id < np) {
        for (int a = 0; a < 4; ++a) d[a] = pos[4 * (size_t)id + a];
    } else {
        const d3 v = ldv(vertice + 3 * (size_t)(id - np));
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
        d[3] = -1.0;
    }
}

inline cudaStream_t S_(void* s) { return static_cast<cudaStream_t>(s); }
inline unsigned nblk(unsigned n, unsigned b) { return n ? (n + b - 1) / b : 1u; }
// blocks of 256 threads, one warp per particle
inline unsigned warp_blocks(unsigned n) { return nblk(n, 8u); }

}  // namespace
}  // namespace xd

using namespace xd;

#define XL_REQUIRE(cond, ...)                                       \
    do {                                                            \
        if (!(cond)) return set_error(XD_ERR_INVALID, __VA_ARGS__); \
    } while (0)

#define XL_BLOCK(name)                                                                               \
    Legacy L;                                                                                        \
    if (!legacy_block(&L))                                                                           \
        return set_error(XD_ERR_STATE, "%s: xd_legacy_set_symbolic_parameter was not called", name)

extern "C" {

int xd_legacy_set_symbolic_parameter(const xd_legacy_parameters* h)
{
    XL_REQUIRE(h, "legacy_set_symbolic_parameter: null parameters");
    XL_REQUIRE(h->cell_size > 0.0, "legacy_set_symbolic_parameter: cell_size must be > 0");
    for (int a = 0; a < 3; ++a)
        XL_REQUIRE(h->grid_size[a] && !(h->grid_size[a] & (h->grid_size[a] - 1)),
                   "legacy_set_symbolic_parameter: grid sizes must be powers of two");
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    g_legacy = *h;
    g_legacy_set = true;
    return XD_OK;
}

int xd_legacy_vv_update_position(double* pos, const double* vel, const double* acc, unsigned np, void* s)
{
    (void)np;
    XL_BLOCK("legacy_vv_update_position");
    if (L.P.np == 0) return XD_OK;
    XL_REQUIRE(pos && vel && acc, "legacy_vv_update_position: null pointer");
    k_legacy_drift<<<nblk(L.P.np, 256), 256, 0, S_(s)>>>(L.P, pos, vel, acc);
    return launch_status("legacy_vv_update_position");
}

int xd_legacy_vv_update_velocity(double* vel, double* acc, double* omega, double* alpha, const double* force,
                                 const double* moment, unsigned np, void* s)
{
    (void)np;
    XL_BLOCK("legacy_vv_update_velocity");
    if (L.P.np == 0) return XD_OK;
    XL_REQUIRE(vel && acc && omega && alpha && force && moment, "legacy_vv_update_velocity: null pointer");
    k_legacy_kick<<<nblk(L.P.np, 256), 256, 0, S_(s)>>>(L.P, vel, acc, omega, alpha, force, moment);
    return launch_status("legacy_vv_update_velocity");
}

int xd_legacy_calculate_hash_and_index(unsigned* hash, unsigned* index, const double* pos, unsigned np, void* s)
{
    XL_BLOCK("legacy_calculate_hash_and_index");
    XL_REQUIRE(hash && index && pos, "legacy_calculate_hash_and_index: null pointer");
    int st = launch_hash(L.P, hash, index, pos, L.P.np + L.P.nsphere, 0, S_(s));
    if (st != XD_OK || np <= 1) return st;
    // the launcher sorts the first np entries (def.cu:65-67), stably by hash;
    // wrapped hashes are below gx gy gz
    void* ws = workspace(radix_sort_scratch_bytes(np), &st);
    if (!ws) return st;
    unsigned *ok = nullptr, *ov = nullptr;
    st = radix_sort_pairs(hash, index, np, key_bits_for(L.P.gx * L.P.gy * L.P.gz), ws, S_(s), &ok, &ov);
    if (st != XD_OK || ok == hash) return st;
    cudaError_t e = cudaMemcpyAsync(hash, ok, sizeof(unsigned) * (size_t)np, cudaMemcpyDeviceToDevice, S_(s));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(index, ov, sizeof(unsigned) * (size_t)np, cudaMemcpyDeviceToDevice, S_(s));
    return cuda_status(e, "legacy_calculate_hash_and_index copy-back");
}

int xd_legacy_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart, unsigned* cend,
                                          unsigned* sorted_index, unsigned np, unsigned nc, void* s)
{
    (void)np;
    XL_BLOCK("legacy_reorder_and_find_cell_start");
    XL_REQUIRE(hash && index && cstart && cend && sorted_index, "legacy_reorder_and_find_cell_start: null pointer");
    // cstart only is reset (def.cu:71-90); the shared cell-range kernel then
    // marks the runs of the sorted keys (a key >= nc is skipped)
    int st = cuda_status(cudaMemsetAsync(cstart, 0xff, sizeof(unsigned) * (size_t)nc, S_(s)),
                         "legacy_reorder_and_find_cell_start");
    if (st != XD_OK) return st;
    void* ws = workspace(256, &st);
    if (!ws) return st;
    return launch_cell_bounds_sorted(hash, index, cstart, cend, sorted_index, L.P.np + L.P.nsphere, nc,
                                     static_cast<unsigned*>(ws), S_(s));
}

int xd_legacy_calculate_p2p(const double* pos, const double* vel, const double* acc, const double* omega,
                            const double* alpha, double* force, double* moment, const unsigned* sorted_index,
                            const unsigned* cstart, const unsigned* cend, unsigned np, unsigned cRun, void* s)
{
    (void)alpha;
    (void)np;
    (void)cRun;
    XL_BLOCK("legacy_calculate_p2p");
    if (L.P.np == 0) return XD_OK;
    XL_REQUIRE(pos && vel && acc && omega && force && moment && sorted_index && cstart && cend,
               "legacy_calculate_p2p: null pointer");
    k_legacy_p2p<<<warp_blocks(L.P.np), 256, 0, S_(s)>>>(L, pos, vel, acc, omega, force, moment, sorted_index,
                                                         cstart, cend);
    return launch_status("legacy_calculate_p2p");
}

int xd_legacy_cube_hertzian_contact_force(const xd_legacy_plane_info* planes, double kn, double vn, double ks,
                                          double vs, double mu, bool* isLineContact, const double* pos,
                                          const double* vel, const double* omega, double* force, double* moment,
                                          unsigned np, void* s)
{
    (void)isLineContact;
    (void)np;
    XL_BLOCK("legacy_cube_hertzian_contact_force");
    if (L.P.np == 0) return XD_OK;
    XL_REQUIRE(planes && pos && vel && omega && force && moment, "legacy_cube_hertzian_contact_force: null pointer");
    k_legacy_cube<<<nblk(L.P.np, 128), 128, 0, S_(s)>>>(L, planes, Fc{ kn, vn, ks, vs, mu }, pos, vel, omega, force,
                                                         moment);
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
    XL_BLOCK("legacy_shape_hertzian_contact_force");
    XL_REQUIRE(minfo && polygons && id_set && poly_start && poly_end && isLineContact && pos && vel && omega &&
                   force && moment && sorted_id && cell_start && cell_end,
               "legacy_shape_hertzian_contact_force: null pointer");
    int st = cuda_status(cudaMemsetAsync(force, 0, sizeof(double) * 3 * (size_t)np, S_(s)), "legacy shape");
    if (st == XD_OK) st = cuda_status(cudaMemsetAsync(moment, 0, sizeof(double) * 3 * (size_t)np, S_(s)), "legacy shape");
    if (st != XD_OK) return st;
    const Shape S{ minfo, polygons, id_set, poly_start, poly_end, Fc{ kn, vn, ks, vs, mu } };
    if (L.P.np) {
        k_legacy_shape<true><<<warp_blocks(L.P.np), 256, 0, S_(s)>>>(L, S, isLineContact, pos, vel, omega, force,
                                                                    moment, sorted_id, cell_start, cell_end);
        k_legacy_shape<false><<<warp_blocks(L.P.np), 256, 0, S_(s)>>>(L, S, isLineContact, pos, vel, omega, force,
                                                                     moment, sorted_id, cell_start, cell_end);
        st = launch_status("legacy_shape_hertzian_contact_force");
        if (st != XD_OK) return st;
    }
    if (np == 0) return XD_OK;
    void* ws = workspace(reduction_scratch_bytes(np), &st);
    if (!ws) return st;
    return reduction_d3(force, np, out, ws, S_(s));
}

int xd_legacy_update_polygons_position(const double* mpos, const double* A, const double* local_vertice,
                                       unsigned nvertex, double* pos, void* s)
{
    if (nvertex == 0) return XD_OK;
    XL_REQUIRE(mpos && A && local_vertice && pos, "legacy_update_polygons_position: null pointer");
    k_legacy_place<<<nblk(nvertex, 256), 256, 0, S_(s)>>>(mpos, A, local_vertice, nvertex, pos);
    return launch_status("legacy_update_polygons_position");
}

int xd_legacy_update_polygons_information(xd_legacy_polygon* polygons, const unsigned* indice, const double* pos,
                                          unsigned ni, void* s)
{
    if (ni == 0) return XD_OK;
    XL_REQUIRE(polygons && indice && pos, "legacy_update_polygons_information: null pointer");
    k_legacy_polygons<<<nblk(ni, 256), 256, 0, S_(s)>>>(polygons, indice, pos, ni);
    return launch_status("legacy_update_polygons_information");
}

int xd_legacy_mergedata(double* data, const double* pos, unsigned np, const double* vertice, unsigned snp,
                        void* s)
{
    if (np + snp == 0) return XD_OK;
    XL_REQUIRE(data && (pos || !np) && (vertice || !snp), "legacy_mergedata: null pointer");
    k_legacy_merge<<<nblk(np + snp, 256), 256, 0, S_(s)>>>(data, pos, np, vertice, snp);
    return launch_status("legacy_mergedata");
}

}  // extern "C"
