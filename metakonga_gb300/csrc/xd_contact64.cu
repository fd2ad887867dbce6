// FP64 contact forces with the reference's semantics (the "plain" form):
// particle-particle (calculate_p2p_kernel<1>, mphysics_cuda_impl.cuh:403-485),
// particle-plane (plane_contact_force_kernel<1>, impl:572-621), particle-
// triangle (particle_polygonObject_collision_kernel<1>, impl:923-1021), the
// mesh update (impl:1911-1956), reductionD3 (def.cu:223-242) and a pair-list
// diagnostic.
//
// Compiled with --fmad=false.  Differences from the reference's arithmetic,
// all inside the stated FP64 tolerance:
//   * pow(cdist, 1.5) is evaluated as cdist * sqrt(cdist) (both within a few
//     ulp of the exact value; the FP64 pow is far more expensive on GB300);
//   * the pair-independent parts of getConstant (Eeq, beta = pi / ln e,
//     1 + beta^2, (4/3) Eeq) are computed once per thread from the contact
//     property instead of once per pair -- same expressions, same bits.
// Reference behaviour that is kept on purpose:
//   * Ft and M live across the pairs of one particle and are only assigned
//     when |e| != 0 (impl:390-400), so a pair with zero tangential slip adds
//     the previous pair's Ft and M again;
//   * planes and triangles are evaluated with ir = 0 in DHSModel, so they
//     apply no moment to the particle (impl:613-615, 1000-1002);
//   * corner contacts of a plane use u = (x - corner)/|x - corner|
//     (impl:506-529) and the third edge test can never pass (impl:549).
#include <cuda_runtime.h>

#include "xd_grid.cuh"
#include "xd_internal.cuh"
#include "xd_physics64.cuh"

namespace xd {

// ------------------------------------------------------- particle-particle

template <bool HIST>
__global__ void __launch_bounds__(128) k_p2p(Params P, const double* __restrict__ pos,
                                             const double* __restrict__ vel,
                                             const double* __restrict__ omega,
                                             double* __restrict__ force, double* __restrict__ moment,
                                             const double* __restrict__ mass,
                                             const unsigned* __restrict__ sorted,
                                             const unsigned* __restrict__ cstart,
                                             const unsigned* __restrict__ cend,
                                             const xd_contact_property* __restrict__ cp, unsigned np,
                                             HistTable ht)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    HistState hs;
    if (HIST) hist_begin(ht, id, hs);
    const PairConst pc = load_pair_const(cp);
    d4 ip = ld4(pos, id);
    d3 ipos = xyz(ip);
    d3 ivel = ld3(vel, id);
    d3 iomega = ld3(omega, id);
    int3 gp = grid_pos(P, ip.x, ip.y, ip.z);
    double ir = ip.w;
    double im = __ldg(mass + id);
    d3 Ft = mk(0, 0, 0), Fn = mk(0, 0, 0), M = mk(0, 0, 0);
    d3 sumF = mk(0, 0, 0), sumM = mk(0, 0, 0);
    for (int z = -1; z <= 1; z++) {
        for (int y = -1; y <= 1; y++) {
            for (int x = -1; x <= 1; x++) {
                unsigned h = grid_hash(P, gp.x + x, gp.y + y, gp.z + z);
                unsigned st = __ldg(cstart + h);
                if (st == 0xffffffffu) continue;
                unsigned en = __ldg(cend + h);
                for (unsigned j = st; j < en; j++) {
                    unsigned k = __ldg(sorted + j);
                    if (id == k || k >= np) continue;
                    d4 jp = ld4(pos, k);
                    double jr = jp.w;
                    d3 rp = mk(jp.x - ipos.x, jp.y - ipos.y, jp.z - ipos.z);
                    double dist = length(rp);
                    double cdist = (ir + jr) - dist;
                    if (cdist > 0) {
                        d3 jvel = ld3(vel, k);
                        d3 jomega = ld3(omega, k);
                        double jm = __ldg(mass + k);
                        d3 unit = rp / dist;
                        d3 rv = P.rolling ? (jvel + cross(jomega, -jr * unit)) - (ivel + cross(iomega, ir * unit))
                                          : (jvel - ivel);
                        Fc c = get_constant(pc, ir, jr, im, jm);
                        if (HIST) {
                            Fn = normal_force(c, ir, jr, pc.Ei, pc.Ej, pc.pri, pc.prj, pc.coh, cdist, rv, unit);
                            d3 d;
                            int sl = hist_slot(ht, hs, id, k, d);
                            hist_tangential(c, ir, rv, unit, P.dt, Fn, d, Ft, M);
                            hist_store(ht, sl, id, d);
                        } else {
                            dhs(c, ir, jr, pc.Ei, pc.Ej, pc.pri, pc.prj, pc.coh, cdist, rv, unit, P.dt,
                                Ft, Fn, M);
                        }
                        sumF += Fn + Ft;
                        sumM += M;
                    }
                }
            }
        }
    }
    if (HIST) hist_end(ht, hs, id, 0u);
    double* f = force + 3 * (size_t)id;
    double* m = moment + 3 * (size_t)id;
    f[0] += sumF.x; f[1] += sumF.y; f[2] += sumF.z;
    m[0] += sumM.x; m[1] += sumM.y; m[2] += sumM.z;
}

// ------------------------------------------------------------------ planes

// Planes applied in order; each adds Fn + Ft to the running force exactly
// like one plane_contact_force_kernel launch per plane.  cp_stride = 0
// shares one property (cube), 1 gives one per plane.
template <bool HIST>
__global__ void __launch_bounds__(128) k_planes(Params P, const xd_plane_info* __restrict__ planes,
                                                const xd_contact_property* __restrict__ cps,
                                                unsigned cp_stride, unsigned nplanes,
                                                const double* __restrict__ pos,
                                                const double* __restrict__ vel,
                                                const double* __restrict__ omega,
                                                double* __restrict__ force,
                                                double* __restrict__ moment,
                                                const double* __restrict__ mass, unsigned np,
                                                HistTable ht)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    HistState hs;
    if (HIST) hist_begin(ht, id, hs);
    double m = __ldg(mass + id);
    d4 ip = ld4(pos, id);
    d3 ipos3 = xyz(ip);
    double r = ip.w;
    d3 ivel = ld3(vel, id);
    d3 iomega = ld3(omega, id);
    d3 f = ld3rw(force, id);
    d3 mo = ld3rw(moment, id);
    for (unsigned w = 0; w < nplanes; ++w) {
        PlaneD pe = load_plane(planes + w);
        d3 Fn = mk(0, 0, 0), Ft = mk(0, 0, 0), M = mk(0, 0, 0);
        d3 dp = ipos3 - pe.xw;
        d3 unit = mk(0, 0, 0);
        d3 wp = mk(dot(dp, pe.u1), dot(dp, pe.u2), dot(dp, pe.uw));
        double cdist = plane_detection(pe, ipos3, wp, unit, r);
        if (cdist > 0) {
            const xd_contact_property* cp = cps + (size_t)w * cp_stride;
            PairConst pc = load_pair_const(cp);
            d3 dv = P.rolling ? -(ivel + cross(iomega, r * unit)) : -ivel;
            Fc c = get_constant(pc, r, 0.0, m, 0.0);
            if (HIST) {
                Fn = normal_force(c, 0, 0, 0, 0, 0, 0, pc.coh, cdist, dv, unit);
                d3 d;
                int sl = hist_slot(ht, hs, id, kHistPlane | w, d);
                hist_tangential(c, 0.0, dv, unit, P.dt, Fn, d, Ft, M);
                hist_store(ht, sl, id, d);
            } else {
                dhs(c, 0, 0, 0, 0, 0, 0, pc.coh, cdist, dv, unit, P.dt, Ft, Fn, M);
            }
        }
        f += Fn + Ft;
        mo += M;
    }
    if (HIST) hist_end(ht, hs, id, 1u);
    st3(force, id, f);
    st3(moment, id, mo);
}

// ---------------------------------------------------------------- cylinder

// particle_cylinder_contact_detection (impl:652-719): the contact depth (the
// reference returns it as float), the unit normal u towards the cylinder and
// the contact point cp.  Rows A1..A3 of the Euler-parameter matrix
// (makeTFM_1..3, impl:624-637); toLocal multiplies by the transpose.
__device__ __forceinline__ double cylinder_detection(const xd_cylinder_info& cy, d3 p, double r, d3& u, d3& cp)
{
    const d3 pbase = mk(cy.pbase[0], cy.pbase[1], cy.pbase[2]);
    const d3 ptop = mk(cy.ptop[0], cy.ptop[1], cy.ptop[2]);
    const d3 ab = ptop - pbase;
    const double t = dot(p - pbase, ab) / dot(ab, ab);
    d3 c = pbase + t * ab;
    double dist = length(p - c);
    if (t >= 0 && t <= 1) {
        u = (c - p) / dist;
        cp = c - cy.rbase * u;
        return (double)(float)(cy.rtop + r - dist);
    }
    if (dist < cy.rbase) {
        const d3 o2c = mk(cy.origin[0], cy.origin[1], cy.origin[2]) - c;
        const double lo = length(o2c);
        u = o2c / lo;
        cp = c - cy.rbase * u;
        return (double)(float)(cy.len * 0.5 + r - lo);
    }
    const double ex = cy.ep[0], ey = cy.ep[1], ez = cy.ep[2], ew = cy.ep[3];
    const d3 A1 = mk(2.0 * (ex * ex + ey * ey - 0.5), 2.0 * (ey * ez - ex * ew), 2.0 * (ey * ew + ex * ez));
    const d3 A2 = mk(2.0 * (ey * ez + ex * ew), 2.0 * (ex * ex + ez * ez - 0.5), 2.0 * (ez * ew - ex * ey));
    const d3 A3 = mk(2.0 * (ey * ew - ex * ez), 2.0 * (ez * ew + ex * ey), 2.0 * (ex * ex + ew * ew - 0.5));
    d3 v = p - ptop;
    d3 at = mk(A1.x * v.x + A2.x * v.y + A3.x * v.z, A1.y * v.x + A2.y * v.y + A3.y * v.z,
               A1.z * v.x + A2.z * v.y + A3.z * v.z);
    cp = ptop;
    if (fabs(at.y) > cy.len) {
        v = p - pbase;
        at = mk(A1.x * v.x + A2.x * v.y + A3.x * v.z, A1.y * v.x + A2.y * v.y + A3.y * v.z,
                A1.z * v.x + A2.z * v.y + A3.z * v.z);
        cp = pbase;
    }
    const double ang = atan(at.x / at.z);
    if ((ang < 0 && at.z < 0) || (ang > 0 && at.x < 0 && at.z < 0)) c.x = cy.rbase * sin(-ang);
    else c.x = cy.rbase * sin(ang);
    c.z = cy.rbase * cos(ang);
    if ((at.z < 0 && c.z > 0) || (at.z > 0 && c.z < 0)) c.z = -c.z;
    c.y = 0.;
    cp = cp + mk(dot(A1, c), dot(A2, c), dot(A3, c));
    const d3 dis = cp - p;
    dist = length(dis);
    u = dis / dist;
    if (dist < r) return (double)(float)(r - dist);
    return -1.0;
}

// cylinder_hertzian_contact_force_kernel<1> (impl:721-760), one thread per
// particle.
__global__ void __launch_bounds__(256) k_cylinder(Params P, const xd_cylinder_info* __restrict__ cyl,
                                                  const xd_contact_property* __restrict__ cps,
                                                  const double* __restrict__ pos, const double* __restrict__ vel,
                                                  const double* __restrict__ omega, double* __restrict__ force,
                                                  double* __restrict__ moment, const double* __restrict__ mass,
                                                  unsigned np, const double* __restrict__ mpos,
                                                  double* __restrict__ mf, double* __restrict__ mm)
{
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    const xd_cylinder_info cy = *cyl;
    const double m = __ldg(mass + id);
    const d4 ip = ld4(pos, id);
    const d3 ivel = ld3(vel, id), iomega = ld3(omega, id);
    d3 unit = mk(0, 0, 0), cpt = mk(0, 0, 0);
    const double cdist = cylinder_detection(cy, xyz(ip), ip.w, unit, cpt);
    const d3 si = cpt - mk(__ldg(mpos), __ldg(mpos + 1), __ldg(mpos + 2));
    const d3 cy2cp = cpt - mk(cy.origin[0], cy.origin[1], cy.origin[2]);
    d3 Ft = mk(0, 0, 0), Fn = mk(0, 0, 0), M = mk(0, 0, 0);
    if (cdist > 0) {
        const d3 dv = mk(cy.vel[0], cy.vel[1], cy.vel[2]) + cross(mk(cy.omega[0], cy.omega[1], cy.omega[2]), cy2cp) -
                      (ivel + cross(iomega, ip.w * unit));
        const PairConst pc = load_pair_const(cps);
        const Fc c = get_constant(pc, ip.w, 0.0, m, 0.0);
        dhs(c, 0, 0, 0, 0, 0, 0, 0.0, cdist, dv, unit, P.dt, Ft, Fn, M);
    }
    st3(force, id, ld3rw(force, id) + (Fn + Ft));
    st3(moment, id, ld3rw(moment, id) + M);
    st3(mf, id, -Fn);
    st3(mm, id, cross(si, -Fn));
}

int launch_cylinder(const Params& P, const xd_cylinder_info* cyl, const xd_contact_property* cp,
                    const double* pos, const double* vel, const double* omega, double* force,
                    double* moment, const double* mass, unsigned np, const double* mpos, double* mf,
                    double* mm, cudaStream_t s)
{
    if (np == 0) return XD_OK;
    k_cylinder<<<div_up(np, 256), 256, 0, s>>>(P, cyl, cp, pos, vel, omega, force, moment, mass, np, mpos, mf, mm);
    return launch_status("cylinder contact");
}

// ---------------------------------------------------------------- polygons

__device__ __forceinline__ d3 ldp(const double* a) { return mk(__ldg(a), __ldg(a + 1), __ldg(a + 2)); }

// Reaction on the polygon bodies: NB > 0 keeps per-thread sums for NB
// bodies and reduces them per block in a fixed order (block partials are
// summed by k_polygon_reaction_final); NB == 0 adds with atomics (used when
// the caller does not say how many bodies there are).
template <int NB, bool HIST>
__global__ void __launch_bounds__(128) k_polygon(Params P, const xd_polygon_info* __restrict__ dpi,
                                                 xd_polygon_mass_info* __restrict__ dpmi,
                                                 const double* __restrict__ pos,
                                                 const double* __restrict__ vel,
                                                 const double* __restrict__ omega,
                                                 double* __restrict__ force,
                                                 double* __restrict__ moment,
                                                 const double* __restrict__ mass,
                                                 const unsigned* __restrict__ sorted,
                                                 const unsigned* __restrict__ cstart,
                                                 const unsigned* __restrict__ cend,
                                                 const xd_contact_property* __restrict__ cp,
                                                 double* __restrict__ partials, HistTable ht)
{
    constexpr int NBR = NB > 0 ? NB : 1;
    double react[NBR][6];
#pragma unroll
    for (int b = 0; b < NBR; ++b)
#pragma unroll
        for (int q = 0; q < 6; ++q) react[b][q] = 0.0;

    const unsigned cnp = P.np;
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < cnp) {
        double im = __ldg(mass + id);
        d4 ip = ld4(pos, id);
        d3 ipos = xyz(ip);
        d3 ivel = ld3(vel, id);
        d3 iomega = ld3(omega, id);
        int3 gp = grid_pos(P, ip.x, ip.y, ip.z);
        double ir = ip.w;
        d3 M = mk(0, 0, 0), Fn = mk(0, 0, 0), Ft = mk(0, 0, 0);
        d3 sum_force = mk(0, 0, 0), sum_moment = mk(0, 0, 0);
        HistState hs;
        if (HIST) hist_begin(ht, id, hs);
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    unsigned h = grid_hash(P, gp.x + x, gp.y + y, gp.z + z);
                    unsigned st = __ldg(cstart + h);
                    if (st == 0xffffffffu) continue;
                    unsigned en = __ldg(cend + h);
                    for (unsigned j = st; j < en; j++) {
                        unsigned k = __ldg(sorted + j);
                        if (k < cnp) continue;
                        k -= cnp;
                        const xd_polygon_info* tri = dpi + k;
                        unsigned pidx = (unsigned)__ldg(&tri->id);
                        const xd_polygon_mass_info* pmi = dpmi + pidx;
                        d3 Pv = ldp(tri->P), Qv = ldp(tri->Q), Rv = ldp(tri->R);
                        d3 cpt = closest_pt_triangle(Pv, Qv, Rv, ipos);
                        d3 po2cp = cpt - ldv(pmi->origin);
                        d3 distVec = ipos - cpt;
                        double dist = length(distVec);
                        double cdist = ir - dist;
                        Fn = mk(0, 0, 0);
                        if (cdist > 0) {
                            d3 qp = Qv - Pv, rp = Rv - Pv;
                            d3 unit = -cross(qp, rp);
                            unit = unit / length(unit);
                            d3 pvel = ldv(pmi->vel), pom = ldv(pmi->omega);
                            d3 dv = P.rolling ? (pvel + cross(pom, po2cp)) - (ivel + cross(iomega, ir * unit))
                                              : (pvel - ivel);
                            PairConst pc = load_pair_const(cp + pidx);
                            Fc c = get_constant(pc, ir, 0, im, 0);
                            if (HIST) {
                                Fn = normal_force(c, 0, 0, 0, 0, 0, 0, 0, cdist, dv, unit);
                                d3 d;
                                int sl = hist_slot(ht, hs, id, kHistTri | k, d);
                                hist_tangential(c, 0.0, dv, unit, P.dt, Fn, d, Ft, M);
                                hist_store(ht, sl, id, d);
                            } else {
                                dhs(c, 0, 0, 0, 0, 0, 0, 0, cdist, dv, unit, P.dt, Ft, Fn, M);
                            }
                            sum_force += Fn + Ft;
                            sum_moment += M;
                            d3 rf = -(Fn + Ft);
                            d3 rm = -cross(po2cp, Fn + Ft);
                            if (NB == 0) {
                                atomicAdd(dpmi[pidx].force + 0, rf.x);
                                atomicAdd(dpmi[pidx].force + 1, rf.y);
                                atomicAdd(dpmi[pidx].force + 2, rf.z);
                                atomicAdd(dpmi[pidx].moment + 0, rm.x);
                                atomicAdd(dpmi[pidx].moment + 1, rm.y);
                                atomicAdd(dpmi[pidx].moment + 2, rm.z);
                            } else if (pidx >= (unsigned)NBR) {
                                // body id beyond the declared count: no slot, add directly
                                atomicAdd(dpmi[pidx].force + 0, rf.x);
                                atomicAdd(dpmi[pidx].force + 1, rf.y);
                                atomicAdd(dpmi[pidx].force + 2, rf.z);
                                atomicAdd(dpmi[pidx].moment + 0, rm.x);
                                atomicAdd(dpmi[pidx].moment + 1, rm.y);
                                atomicAdd(dpmi[pidx].moment + 2, rm.z);
                            } else {
#pragma unroll
                                for (int b = 0; b < NBR; ++b)
                                    if ((unsigned)b == pidx) {
                                        react[b][0] += rf.x; react[b][1] += rf.y; react[b][2] += rf.z;
                                        react[b][3] += rm.x; react[b][4] += rm.y; react[b][5] += rm.z;
                                    }
                            }
                        }
                    }
                }
        if (HIST) hist_end(ht, hs, id, 2u);
        double* f = force + 3 * (size_t)id;
        double* m = moment + 3 * (size_t)id;
        f[0] += sum_force.x; f[1] += sum_force.y; f[2] += sum_force.z;
        m[0] += sum_moment.x; m[1] += sum_moment.y; m[2] += sum_moment.z;
    }
    if (NB > 0) {
        // fixed-order block tree reduction of the per-thread reactions
        __shared__ double red[128];
        for (int b = 0; b < NBR; ++b)
            for (int q = 0; q < 6; ++q) {
                red[threadIdx.x] = react[b][q];
                __syncthreads();
                for (int o = 64; o > 0; o >>= 1) {
                    if (threadIdx.x < (unsigned)o) red[threadIdx.x] += red[threadIdx.x + o];
                    __syncthreads();
                }
                if (threadIdx.x == 0) partials[((size_t)blockIdx.x * NBR + b) * 6 + q] = red[0];
                __syncthreads();
            }
    }
}

// Sums the block partials of each body in block order and adds the total to
// dpmi[b].force / .moment.
__global__ void k_polygon_reaction_final(const double* __restrict__ partials, unsigned nblocks,
                                         unsigned nbodies, unsigned nbr,
                                         xd_polygon_mass_info* __restrict__ dpmi)
{
    unsigned t = threadIdx.x;   // one thread per (body, component)
    if (t >= nbodies * 6) return;
    unsigned b = t / 6, q = t % 6;
    double s = 0.0;
    for (unsigned blk = 0; blk < nblocks; ++blk) s += partials[((size_t)blk * nbr + b) * 6 + q];
    if (q < 3) dpmi[b].force[q] += s;
    else dpmi[b].moment[q - 3] += s;
}

// ----------------------------------------------------------- mesh update

// toGlobal(double3&, double4&) (impl:1898-1909)

// updatePolygonObjectData_kernel (impl:1911-1956); t = 0 where the
// reference leaves it uninitialised (all three determinants <= 1e-13).
__global__ void __launch_bounds__(256) k_update_polygon(const xd_polygon_mass_info* __restrict__ dpmi,
                                                        const double* __restrict__ vlist,
                                                        double* __restrict__ sphere,
                                                        xd_polygon_info* __restrict__ dpi,
                                                        unsigned ntri)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ntri) return;
    d3 Pv, Qv, Rv;
    update_polygon_one(dpmi, vlist, sphere, dpi, id, Pv, Qv, Rv);
}

// ----------------------------------------------------------- reductionD3

constexpr int kRedThreads = 256;
constexpr int kRedBlocksMax = 1024;

__global__ void __launch_bounds__(kRedThreads) k_reduce_d3_partial(const double* __restrict__ in,
                                                                   unsigned n,
                                                                   double* __restrict__ partial)
{
    __shared__ double red[3][kRedThreads];
    double s[3] = { 0.0, 0.0, 0.0 };
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        s[0] += in[3 * i];
        s[1] += in[3 * i + 1];
        s[2] += in[3 * i + 2];
    }
    for (int q = 0; q < 3; ++q) red[q][threadIdx.x] = s[q];
    __syncthreads();
    for (int o = kRedThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < (unsigned)o)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) partial[3 * blockIdx.x + q] = red[q][0];
}

__global__ void k_reduce_d3_final(const double* __restrict__ partial, unsigned nb, double* __restrict__ out)
{
    if (threadIdx.x >= 3) return;
    double s = 0.0;
    for (unsigned b = 0; b < nb; ++b) s += partial[3 * b + threadIdx.x];
    out[threadIdx.x] = s;
}

// ------------------------------------------------------------- pair list

__device__ __forceinline__ unsigned pair_scan(const Params& P, const double* pos,
                                              const unsigned* sorted, const unsigned* cstart,
                                              const unsigned* cend, unsigned np, unsigned id,
                                              unsigned* out, unsigned cap_left)
{
    d4 ip = ld4(pos, id);
    int3 gp = grid_pos(P, ip.x, ip.y, ip.z);
    unsigned cnt = 0;
    for (int z = -1; z <= 1; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                unsigned h = grid_hash(P, gp.x + x, gp.y + y, gp.z + z);
                unsigned st = __ldg(cstart + h);
                if (st == 0xffffffffu) continue;
                unsigned en = __ldg(cend + h);
                for (unsigned j = st; j < en; j++) {
                    unsigned k = __ldg(sorted + j);
                    if (id == k || k >= np) continue;
                    d4 jp = ld4(pos, k);
                    d3 rp = mk(jp.x - ip.x, jp.y - ip.y, jp.z - ip.z);
                    double cdist = (ip.w + jp.w) - length(rp);
                    if (cdist > 0) {
                        if (out && cnt < cap_left) {
                            out[2 * cnt] = id;
                            out[2 * cnt + 1] = k;
                        }
                        cnt++;
                    }
                }
            }
    return cnt;
}

__global__ void k_pair_count(Params P, const double* __restrict__ pos, const unsigned* __restrict__ sorted,
                             const unsigned* __restrict__ cstart, const unsigned* __restrict__ cend,
                             unsigned np, unsigned* __restrict__ counts)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    counts[id] = pair_scan(P, pos, sorted, cstart, cend, np, id, nullptr, 0);
}

__global__ void k_pair_fill(Params P, const double* __restrict__ pos, const unsigned* __restrict__ sorted,
                            const unsigned* __restrict__ cstart, const unsigned* __restrict__ cend,
                            unsigned np, const unsigned long long* __restrict__ offsets,
                            unsigned* __restrict__ pairs, unsigned long long cap)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    unsigned long long o = offsets[id];
    if (o >= cap) return;
    unsigned long long left = cap - o;
    pair_scan(P, pos, sorted, cstart, cend, np, id, pairs + 2 * o,
              left > 0xffffffffull ? 0xffffffffu : (unsigned)left);
}

__global__ void k_pair_offsets(const unsigned* __restrict__ counts, unsigned np,
                               unsigned long long* __restrict__ offsets)
{
    // single thread: exclusive prefix in 64-bit (diagnostic path)
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long run = 0;
    for (unsigned i = 0; i < np; ++i) {
        offsets[i] = run;
        run += counts[i];
    }
    offsets[np] = run;
}

// ------------------------------------------------------------- launchers

int launch_p2p(const Params& P, const double* pos, const double* vel, const double* omega,
               double* force, double* moment, const double* mass, const unsigned* sorted,
               const unsigned* cstart, const unsigned* cend, const xd_contact_property* cp,
               unsigned np, cudaStream_t s, const HistTable* ht)
{
    if (np == 0) return XD_OK;
    if (ht)
        k_p2p<true><<<div_up(np, 128), 128, 0, s>>>(P, pos, vel, omega, force, moment, mass, sorted, cstart,
                                                    cend, cp, np, *ht);
    else
        k_p2p<false><<<div_up(np, 128), 128, 0, s>>>(P, pos, vel, omega, force, moment, mass, sorted, cstart,
                                                     cend, cp, np, HistTable{});
    return launch_status("calculate_p2p");
}

int launch_planes(const Params& P, const xd_plane_info* planes, const xd_contact_property* cps,
                  unsigned cp_stride, unsigned nplanes, const double* pos, const double* vel,
                  const double* omega, double* force, double* moment, const double* mass,
                  unsigned np, cudaStream_t s, const HistTable* ht)
{
    if (np == 0 || nplanes == 0) return XD_OK;
    if (ht)
        k_planes<true><<<div_up(np, 128), 128, 0, s>>>(P, planes, cps, cp_stride, nplanes, pos, vel, omega,
                                                       force, moment, mass, np, *ht);
    else
        k_planes<false><<<div_up(np, 128), 128, 0, s>>>(P, planes, cps, cp_stride, nplanes, pos, vel, omega,
                                                        force, moment, mass, np, HistTable{});
    return launch_status("plane_contact_force");
}

static unsigned nbr_for(unsigned nbodies)
{
    if (nbodies == 0 || nbodies > 8) return 0;
    if (nbodies == 1) return 1;
    if (nbodies == 2) return 2;
    if (nbodies <= 4) return 4;
    return 8;
}

size_t polygon_scratch_bytes(unsigned np, unsigned nbodies)
{
    unsigned nbr = nbr_for(nbodies);
    if (nbr == 0) return 0;
    return sizeof(double) * 6 * (size_t)nbr * div_up(np ? np : 1u, 128);
}

int launch_polygon(const Params& P, const xd_polygon_info* dpi, xd_polygon_mass_info* dpmi,
                   const double* pos, const double* vel, const double* omega, double* force,
                   double* moment, const double* mass, const unsigned* sidx,
                   const unsigned* cstart, const unsigned* cend, const xd_contact_property* cp,
                   unsigned nbodies, void* scratch, cudaStream_t s, const HistTable* ht)
{
    unsigned np = P.np;
    if (np == 0) return XD_OK;
    unsigned nb = div_up(np, 128);
    unsigned nbr = nbr_for(nbodies);
    double* part = static_cast<double*>(scratch);
#define XD_POLY(NBV)                                                                              \
    do {                                                                                          \
        if (ht)                                                                                   \
            k_polygon<NBV, true><<<nb, 128, 0, s>>>(P, dpi, dpmi, pos, vel, omega, force, moment, \
                                                    mass, sidx, cstart, cend, cp, part, *ht);     \
        else                                                                                      \
            k_polygon<NBV, false><<<nb, 128, 0, s>>>(P, dpi, dpmi, pos, vel, omega, force, moment, \
                                                     mass, sidx, cstart, cend, cp, part, HistTable{}); \
    } while (0)
    switch (nbr) {
    case 0: XD_POLY(0); break;
    case 1: XD_POLY(1); break;
    case 2: XD_POLY(2); break;
    case 4: XD_POLY(4); break;
    default: XD_POLY(8); break;
    }
#undef XD_POLY
    int st = launch_status("particle_polygon_collision");
    if (st != XD_OK || nbr == 0) return st;
    k_polygon_reaction_final<<<1, 64, 0, s>>>(part, nb, nbodies, nbr, dpmi);
    return launch_status("particle_polygon_collision (reaction)");
}

// One step of prescribed body motion (an extension; the reference moves its
// bodies through the multibody solver on the host): origin += dt vel, the
// Euler parameters p <- q (x) p with q the rotation of angle |omega| dt about
// omega, normalised.  One thread per body.
__global__ void k_body_advance(xd_polygon_mass_info* __restrict__ pmi, unsigned nbodies, double dt)
{
    const unsigned b = threadIdx.x;
    if (b >= nbodies) return;
    xd_polygon_mass_info* m = pmi + b;
    for (int a = 0; a < 3; ++a) m->origin[a] = m->origin[a] + dt * m->vel[a];
    const double wx = m->omega[0], wy = m->omega[1], wz = m->omega[2];
    const double w = sqrt(wx * wx + wy * wy + wz * wz);
    if (w > 0.0) {
        const double h = 0.5 * w * dt;
        const double c = cos(h), sn = sin(h) / w;
        const double a0 = c, a1 = sn * wx, a2 = sn * wy, a3 = sn * wz;
        const double p0 = m->ep[0], p1 = m->ep[1], p2 = m->ep[2], p3 = m->ep[3];
        const double r0 = a0 * p0 - (a1 * p1 + a2 * p2 + a3 * p3);
        const double r1 = a0 * p1 + p0 * a1 + (a2 * p3 - a3 * p2);
        const double r2 = a0 * p2 + p0 * a2 + (a3 * p1 - a1 * p3);
        const double r3 = a0 * p3 + p0 * a3 + (a1 * p2 - a2 * p1);
        const double nr = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + r3 * r3);
        m->ep[0] = r0 / nr;
        m->ep[1] = r1 / nr;
        m->ep[2] = r2 / nr;
        m->ep[3] = r3 / nr;
    }
}

int launch_body_advance(xd_polygon_mass_info* pmi, unsigned nbodies, double dt, cudaStream_t s)
{
    if (nbodies == 0) return XD_OK;
    k_body_advance<<<1, 32, 0, s>>>(pmi, nbodies, dt);
    return launch_status("kinematic bodies");
}

// The mesh update and, for the mixed form, whether a vertex has moved from
// its position at the last list build (ref: FP32, relative to the grid origin
// wo) by disp2 or more: *flag is raised then.  rec (the mixed form's
// triangle records) is rewritten from the new vertices.
__global__ void __launch_bounds__(64) k_mesh_move(const xd_polygon_mass_info* __restrict__ dpmi,
                                                  const double* __restrict__ vlist, double* __restrict__ sphere,
                                                  xd_polygon_info* __restrict__ dpi, unsigned ntri,
                                                  const float* __restrict__ ref, double wo0, double wo1, double wo2,
                                                  float disp2, unsigned* __restrict__ flag, TriRec* __restrict__ rec)
{
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    bool out = false;
    if (id < ntri) {
        d3 V[3];
        update_polygon_one(dpmi, vlist, sphere, dpi, id, V[0], V[1], V[2]);
        if (rec) write_tri_rec(rec + id, V[0], V[1], V[2], (unsigned)dpi[id].id);
        const double wo[3] = { wo0, wo1, wo2 };
        for (int k = 0; k < 3; ++k) {
            const double c[3] = { V[k].x, V[k].y, V[k].z };
            float d2 = 0.f;
            for (int a = 0; a < 3; ++a) {
                const float d = (float)(c[a] - wo[a]) - ref[9 * (size_t)id + 3 * k + a];
                d2 += d * d;
            }
            out |= !(d2 < disp2);
        }
    }
    if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31u) == 0) atomicOr(flag, 1u);
}

int launch_mesh_move(const xd_polygon_mass_info* dpmi, const double* vlist, double* sphere, xd_polygon_info* dpi,
                     unsigned ntri, const float* ref, const double wo[3], float disp2, unsigned* flag,
                     TriRec* rec, cudaStream_t s)
{
    if (ntri == 0) return XD_OK;
    k_mesh_move<<<div_up(ntri, 64), 64, 0, s>>>(dpmi, vlist, sphere, dpi, ntri, ref, wo[0], wo[1], wo[2], disp2,
                                               flag, rec);
    return launch_status("mesh move");
}

// The mixed form's triangle records of the mesh as it stands.
__global__ void __launch_bounds__(64) k_tri_records(const xd_polygon_info* __restrict__ dpi, unsigned ntri,
                                                    TriRec* __restrict__ rec)
{
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ntri) return;
    const xd_polygon_info* t = dpi + id;
    write_tri_rec(rec + id, ldp3(t->P), ldp3(t->Q), ldp3(t->R), (unsigned)__ldg(&t->id));
}

int launch_tri_records(const xd_polygon_info* dpi, unsigned ntri, TriRec* rec, cudaStream_t s)
{
    if (ntri == 0) return XD_OK;
    k_tri_records<<<div_up(ntri, 64), 64, 0, s>>>(dpi, ntri, rec);
    return launch_status("triangle records");
}

int launch_update_polygon(const xd_polygon_mass_info* dpmi, const double* vlist, double* sphere,
                          xd_polygon_info* dpi, unsigned ntri, cudaStream_t s)
{
    if (ntri == 0) return XD_OK;
    // FP64-heavy and short: small blocks spread the triangles over every SM
    k_update_polygon<<<div_up(ntri, 64), 64, 0, s>>>(dpmi, vlist, sphere, dpi, ntri);
    return launch_status("update_polygon_object_data");
}

size_t reduction_scratch_bytes(unsigned n)
{
    (void)n;
    return sizeof(double) * 3 * (kRedBlocksMax + 1);
}

int reduction_d3(const double* in, unsigned n, double out[3], void* scratch, cudaStream_t s)
{
    double* part = static_cast<double*>(scratch);
    unsigned nb = div_up(n ? n : 1u, kRedThreads);
    if (nb > (unsigned)kRedBlocksMax) nb = kRedBlocksMax;
    k_reduce_d3_partial<<<nb, kRedThreads, 0, s>>>(in, n, part);
    k_reduce_d3_final<<<1, 32, 0, s>>>(part, nb, part + 3 * kRedBlocksMax);
    int st = launch_status("reductionD3");
    if (st != XD_OK) return st;
    cudaError_t e = cudaMemcpyAsync(out, part + 3 * kRedBlocksMax, 3 * sizeof(double),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_status(e, "reductionD3 read-back");
}

size_t pair_list_scratch_bytes(unsigned np) { return sizeof(unsigned long long) * ((size_t)np + 1); }

int pair_list(const Params& P, const double* pos, const unsigned* sorted, const unsigned* cstart,
              const unsigned* cend, unsigned np, unsigned* counts, unsigned* pairs,
              unsigned long long cap, unsigned long long* total, void* scratch, cudaStream_t s)
{
    *total = 0;
    if (np == 0) return XD_OK;
    unsigned long long* off = static_cast<unsigned long long*>(scratch);
    k_pair_count<<<div_up(np, 128), 128, 0, s>>>(P, pos, sorted, cstart, cend, np, counts);
    k_pair_offsets<<<1, 1, 0, s>>>(counts, np, off);
    k_pair_fill<<<div_up(np, 128), 128, 0, s>>>(P, pos, sorted, cstart, cend, np, off, pairs, cap);
    int st = launch_status("pair_list");
    if (st != XD_OK) return st;
    cudaError_t e = cudaMemcpyAsync(total, off + np, sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    st = cuda_status(e, "pair_list read-back");
    if (st != XD_OK) return st;
    if (*total > cap) return set_error(XD_ERR_CAPACITY, "pair_list: %llu pairs > cap %llu", *total, cap);
    return XD_OK;
}

}  // namespace xd
