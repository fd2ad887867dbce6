// FP64 contact physics shared by the plain (reference-arithmetic) kernels
// and the FP64 wall pass of the mixed form: getConstant (TCM = 1),
// cohesionForce, DHSModel, the finite-plane region test and the
// closest point on a triangle, each restating the cited reference lines.
#pragma once

#include "xd_internal.cuh"

namespace xd {

struct Fc {
    double kn, vn, ks, vs, mu;
};

struct PairConst {
    double c43Eeq, one_b2, sratio, fric, coh, Ei, Ej, pri, prj;
};

__device__ __forceinline__ PairConst load_pair_const(const xd_contact_property* cp)
{
    PairConst c;
    double Ei = __ldg(&cp->Ei), Ej = __ldg(&cp->Ej), pri = __ldg(&cp->pri), prj = __ldg(&cp->prj);
    double Eeq = (Ei * Ej) / (Ei * (1 - prj * prj) + Ej * (1 - pri * pri));
    double beta = (M_PI / log(__ldg(&cp->rest)));
    c.c43Eeq = (4.0 / 3.0) * Eeq;
    c.one_b2 = 1.0 + beta * beta;
    c.sratio = __ldg(&cp->sratio);
    c.fric = __ldg(&cp->fric);
    c.coh = __ldg(&cp->coh);
    c.Ei = Ei;
    c.Ej = Ej;
    c.pri = pri;
    c.prj = prj;
    return c;
}

// getConstant, TCM = 1 (impl:214-256)
__device__ __forceinline__ Fc get_constant(const PairConst& pc, double ir, double jr, double im,
                                           double jm)
{
    Fc c;
    double Meq = jm != 0.0 ? (im * jm) / (im + jm) : im;
    double Req = jr != 0.0 ? (ir * jr) / (ir + jr) : ir;
    c.kn = pc.c43Eeq * sqrt(Req);
    c.vn = sqrt((4.0 * Meq * c.kn) / pc.one_b2);
    c.ks = c.kn * pc.sratio;
    c.vs = c.vn * pc.sratio;
    c.mu = pc.fric;
    return c;
}

// cohesionForce (impl:259-279)
__device__ __forceinline__ double cohesion_force(double ri, double rj, double Ei, double Ej,
                                                 double pri, double prj, double coh, double Fn)
{
    double cf = 0.0;
    if (coh != 0.0) {
        double req = (ri * rj / (ri + rj));
        double Eeq = ((1.0 - pri * pri) / Ei) + ((1.0 - prj * prj) / Ej);
        double rcp = (3.0 * req * (-Fn)) / (4.0 * (1.0 / Eeq));
        double rc = pow(rcp, 1.0 / 3.0);
        double Ac = M_PI * rc * rc;
        cf = coh * Ac;
    }
    return cf;
}

// DHSModel (impl:379-401); Ft and M are in/out (kept across pairs).
__device__ __forceinline__ void dhs(const Fc& c, double ir, double jr, double Ei, double Ej,
                                    double pri, double prj, double coh, double cdist, d3 dv,
                                    d3 unit, double dt, d3& Ft, d3& Fn, d3& M)
{
    double fsn = -c.kn * (cdist * sqrt(cdist));
    double fdn = c.vn * dot(dv, unit);
    double fca = cohesion_force(ir, jr, Ei, Ej, pri, prj, coh, fsn);
    Fn = (fsn + fca + fdn) * unit;
    d3 e = dv - dot(dv, unit) * unit;
    double mag_e = length(e);
    if (mag_e != 0.0) {
        d3 sh = e / mag_e;
        double ds = mag_e * dt;
        Ft = fmin(c.ks * ds + c.vs * (dot(dv, sh)), c.mu * length(Fn)) * sh;
        M = cross(ir * unit, Ft);
    }
}

// ---------------------------------------------- tangential-spring history
//
// An extension with no counterpart in the reference (DHSModel keeps no state
// between steps).  A particle holds up to `slots` contacts, keyed by partner:
// particle j -> its original index, plane w -> kHistPlane | w, triangle t ->
// kHistTri | t; key[s * n + i], delta[(s * n + i) * 3 + a].  Per contact and
// step, vt the tangential relative velocity:
//   d <- d - (d.u)u rescaled to |d|; d <- d + vt dt; Ft = ks d + vs vt;
//   if |Ft| > mu |Fn|: Ft <- mu |Fn| Ft / |Ft|, d <- (Ft - vs vt) / ks;
//   M = (ir u) x Ft.
// A new contact starts from d = 0 (its first step is the reference's DHS
// force); a contact that ends frees its entry; a contact that finds no free
// entry is counted in *overflow and computed without history.
constexpr unsigned kHistEmpty = 0xffffffffu;
constexpr unsigned kHistPlane = 0x80000000u;
constexpr unsigned kHistTri = 0xC0000000u;
constexpr unsigned kHistMaxSlots = 32;

struct HistTable {
    unsigned* key;
    double* delta;
    unsigned slots;
    unsigned n;
    unsigned long long* overflow;
};

__device__ __forceinline__ unsigned hist_class(unsigned k) { return k < kHistPlane ? 0u : (k < kHistTri ? 1u : 2u); }

struct HistState {
    unsigned freem, matched;
};

__device__ __forceinline__ void hist_begin(const HistTable& h, unsigned i, HistState& st)
{
    st.freem = 0;
    st.matched = 0;
    for (unsigned s = 0; s < h.slots; ++s)
        if (h.key[(size_t)s * h.n + i] == kHistEmpty) st.freem |= 1u << s;
}

// the entry of `key` (its spring in d), else the lowest free entry (d = 0), else -1
__device__ __forceinline__ int hist_slot(const HistTable& h, HistState& st, unsigned i, unsigned key, d3& d)
{
    d = mk(0, 0, 0);
    for (unsigned s = 0; s < h.slots; ++s) {
        const size_t e = (size_t)s * h.n + i;
        if (h.key[e] == key) {
            const double* p = h.delta + e * 3;
            d = mk(p[0], p[1], p[2]);
            st.matched |= 1u << s;
            return (int)s;
        }
    }
    if (st.freem) {
        const unsigned s = __ffs(st.freem) - 1;
        st.freem &= ~(1u << s);
        st.matched |= 1u << s;
        h.key[(size_t)s * h.n + i] = key;
        return (int)s;
    }
    atomicAdd(h.overflow, 1ull);
    return -1;
}

__device__ __forceinline__ void hist_store(const HistTable& h, int s, unsigned i, d3 d)
{
    if (s < 0) return;
    double* p = h.delta + ((size_t)s * h.n + i) * 3;
    p[0] = d.x;
    p[1] = d.y;
    p[2] = d.z;
}

// entries of class cls whose contact did not recur are freed
__device__ __forceinline__ void hist_end(const HistTable& h, const HistState& st, unsigned i, unsigned cls)
{
    for (unsigned s = 0; s < h.slots; ++s) {
        if (st.matched & (1u << s)) continue;
        const size_t e = (size_t)s * h.n + i;
        const unsigned k = h.key[e];
        if (k == kHistEmpty || hist_class(k) != cls) continue;
        h.key[e] = kHistEmpty;
        double* p = h.delta + e * 3;
        p[0] = p[1] = p[2] = 0.0;
    }
}

// every entry whose contact did not recur this step is freed (one pass over
// all contact kinds)
__device__ __forceinline__ void hist_end_all(const HistTable& h, const HistState& st, unsigned i)
{
    for (unsigned s = 0; s < h.slots; ++s) {
        if (st.matched & (1u << s)) continue;
        const size_t e = (size_t)s * h.n + i;
        if (h.key[e] == kHistEmpty) continue;
        h.key[e] = kHistEmpty;
        double* p = h.delta + e * 3;
        p[0] = p[1] = p[2] = 0.0;
    }
}

// read-only lookup (diagnostic evaluation): the spring of `key`, or 0
__device__ __forceinline__ void hist_peek(const HistTable& h, unsigned i, unsigned key, d3& d)
{
    d = mk(0, 0, 0);
    for (unsigned s = 0; s < h.slots; ++s) {
        const size_t e = (size_t)s * h.n + i;
        if (h.key[e] == key) {
            const double* p = h.delta + e * 3;
            d = mk(p[0], p[1], p[2]);
            return;
        }
    }
}

// DHSModel's normal force (impl:385-388)
__device__ __forceinline__ d3 normal_force(const Fc& c, double ir, double jr, double Ei, double Ej, double pri,
                                           double prj, double coh, double cdist, d3 dv, d3 unit)
{
    double fsn = -c.kn * (cdist * sqrt(cdist));
    double fdn = c.vn * dot(dv, unit);
    double fca = cohesion_force(ir, jr, Ei, Ej, pri, prj, coh, fsn);
    return (fsn + fca + fdn) * unit;
}

// the tangential spring with history (see above); d in/out
__device__ __forceinline__ void hist_tangential(const Fc& c, double ir, d3 dv, d3 unit, double dt, d3 Fn, d3& d,
                                                d3& Ft, d3& M)
{
    d3 vt = dv - dot(dv, unit) * unit;
    double m0 = length(d);
    d3 dp = d - dot(d, unit) * unit;
    double mp = length(dp);
    d3 dn = mp > 0.0 ? (m0 / mp) * dp : mk(0, 0, 0);
    dn = dn + dt * vt;
    d3 ft = c.ks * dn + c.vs * vt;
    double fmax = c.mu * length(Fn);
    double mf = length(ft);
    if (mf > fmax) {
        ft = (fmax / mf) * ft;
        dn = (ft - c.vs * vt) / c.ks;
    }
    d = dn;
    Ft = ft;
    M = cross(ir * unit, ft);
}

struct PlaneD {
    double l1, l2;
    d3 u1, u2, uw, xw, w2, w3, w4;
};

__device__ __forceinline__ PlaneD load_plane(const xd_plane_info* p)
{
    PlaneD q;
    q.l1 = __ldg(&p->l1);
    q.l2 = __ldg(&p->l2);
    q.u1 = mk(__ldg(p->u1), __ldg(p->u1 + 1), __ldg(p->u1 + 2));
    q.u2 = mk(__ldg(p->u2), __ldg(p->u2 + 1), __ldg(p->u2 + 2));
    q.uw = mk(__ldg(p->uw), __ldg(p->uw + 1), __ldg(p->uw + 2));
    q.xw = mk(__ldg(p->xw), __ldg(p->xw + 1), __ldg(p->xw + 2));
    q.w2 = mk(__ldg(p->w2), __ldg(p->w2 + 1), __ldg(p->w2 + 2));
    q.w3 = mk(__ldg(p->w3), __ldg(p->w3 + 1), __ldg(p->w3 + 2));
    q.w4 = mk(__ldg(p->w4), __ldg(p->w4 + 1), __ldg(p->w4 + 2));
    return q;
}

__device__ __forceinline__ int sgn(double L) { return L < 0 ? -1 : 1; }

// Vector arithmetic with every operation rounded on its own (no multiply-add
// contraction whatever the translation unit's flags), left to right as the
// reference's operators: the region tests below give the same bits in the
// FP64 form (built with --fmad=false) and in the mixed form's FP64 fallbacks.
namespace rn {
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ d3 add(d3 a, d3 b) { return mk(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)); }
__device__ __forceinline__ d3 sub(d3 a, d3 b) { return mk(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)); }
__device__ __forceinline__ d3 scale(double s, d3 a) { return mk(mul(s, a.x), mul(s, a.y), mul(s, a.z)); }
__device__ __forceinline__ d3 divs(d3 a, double s) { return mk(div(a.x, s), div(a.y, s), div(a.z, s)); }
__device__ __forceinline__ double dot(d3 a, d3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ double length(d3 a) { return __dsqrt_rn(rn::dot(a, a)); }
__device__ __forceinline__ d3 cross(d3 a, d3 b)
{
    return mk(sub(mul(a.y, b.z), mul(a.z, b.y)), sub(mul(a.z, b.x), mul(a.x, b.z)), sub(mul(a.x, b.y), mul(a.y, b.x)));
}
}  // namespace rn

// The face region of a finite plane (impl:506-513): the overlap r - |dp . u|
// with u = uw / |uw| turned against the side of xp (-sgn(dp . uw)).
__device__ __forceinline__ double plane_face_depth(const PlaneD& pe, d3 xp, d3& u, double r)
{
    const d3 dp = rn::sub(xp, pe.xw);
    const d3 uu = rn::divs(pe.uw, rn::length(pe.uw));
    const int pp = -sgn(rn::dot(dp, pe.uw));
    u = rn::scale((double)pp, uu);
    return rn::sub(r, fabs(rn::dot(dp, u)));
}

// whether wp (plane-frame coordinates) lies in the face region
__device__ __forceinline__ bool plane_face_region(const PlaneD& pe, d3 wp, double r)
{
    return fabs(wp.z) < r && (wp.x > 0 && wp.x < pe.l1) && (wp.y > 0 && wp.y < pe.l2);
}

// particle_plane_contact_detection (impl:487-570); pow(x, 2.0) is x * x
// (IEEE: the correctly rounded square).
__device__ __forceinline__ double plane_detection(const PlaneD& pe, d3 xp, d3 wp, d3& u, double r)
{
    const double a_l1 = rn::mul(rn::sub(wp.x, pe.l1), rn::sub(wp.x, pe.l1));
    const double b_l2 = rn::mul(rn::sub(wp.y, pe.l2), rn::sub(wp.y, pe.l2));
    const double sqa = rn::mul(wp.x, wp.x);
    const double sqb = rn::mul(wp.y, wp.y);
    const double sqc = rn::mul(wp.z, wp.z);
    const double sqr = rn::mul(r, r);
    if (plane_face_region(pe, wp, r)) return plane_face_depth(pe, xp, u, r);
    if (wp.x < 0 && wp.y < 0 && rn::add(rn::add(sqa, sqb), sqc) < sqr) {
        const d3 X = rn::sub(xp, pe.xw); const double h = rn::length(X); u = rn::divs(X, h); return rn::sub(r, h);
    } else if (wp.x > pe.l1 && wp.y < 0 && rn::add(rn::add(a_l1, sqb), sqc) < sqr) {
        const d3 X = rn::sub(xp, pe.w2); const double h = rn::length(X); u = rn::divs(X, h); return rn::sub(r, h);
    } else if (wp.x > pe.l1 && wp.y > pe.l2 && rn::add(rn::add(a_l1, b_l2), sqc) < sqr) {
        const d3 X = rn::sub(xp, pe.w3); const double h = rn::length(X); u = rn::divs(X, h); return rn::sub(r, h);
    } else if (wp.x < 0 && wp.y > pe.l2 && rn::add(rn::add(sqa, b_l2), sqc) < sqr) {
        const d3 X = rn::sub(xp, pe.w4); const double h = rn::length(X); u = rn::divs(X, h); return rn::sub(r, h);
    }
    d3 X, wj;
    if ((wp.x > 0 && wp.x < pe.l1) && wp.y < 0 && rn::add(sqb, sqc) < sqr) {
        X = rn::sub(xp, pe.xw); wj = rn::sub(pe.w2, pe.xw);
    } else if ((wp.x > 0 && wp.x < pe.l1) && wp.y > pe.l2 && rn::add(b_l2, sqc) < sqr) {
        X = rn::sub(xp, pe.w4); wj = rn::sub(pe.w3, pe.w4);
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x < 0 && rn::add(sqr, sqc) < sqr) {
        X = rn::sub(xp, pe.xw); wj = rn::sub(pe.w4, pe.xw);
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x > pe.l1 && rn::add(a_l1, sqc) < sqr) {
        X = rn::sub(xp, pe.w2); wj = rn::sub(pe.w3, pe.w2);
    } else {
        return -1.0;
    }
    const d3 us = rn::divs(wj, rn::length(wj));
    const d3 hs = rn::sub(X, rn::scale(rn::dot(X, us), us));
    const double h = rn::length(hs);
    u = rn::divs(mk(-hs.x, -hs.y, -hs.z), h);
    return rn::sub(r, h);
}

// The reference's plane-frame coordinates wp = (dp.u1, dp.u2, dp.uw) of
// dp = xp - xw (plane_contact_force_kernel, impl:596-600), rounded per operation.
__device__ __forceinline__ d3 plane_coords(const PlaneD& pe, d3 xp)
{
    const d3 dp = rn::sub(xp, pe.xw);
    return mk(rn::dot(dp, pe.u1), rn::dot(dp, pe.u2), rn::dot(dp, pe.uw));
}

// closestPtPointTriangle (impl:837-899), Ericson's region test; region: 0 a
// vertex, 1 an edge, 2 the face (the legacy shape kernels branch on it,
// cu_dem_impl.cuh:380-441).
__device__ __forceinline__ d3 closest_pt_triangle_region(d3 a, d3 b, d3 c, d3 p, int& region)
{
    const d3 ab = rn::sub(b, a), ac = rn::sub(c, a), ap = rn::sub(p, a);
    const double d1 = rn::dot(ab, ap), d2 = rn::dot(ac, ap);
    region = 0;
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    const d3 bp = rn::sub(p, b);
    const double d3_ = rn::dot(ab, bp), d4 = rn::dot(ac, bp);
    if (d3_ >= 0.0 && d4 <= d3_) return b;
    const double vc = rn::sub(rn::mul(d1, d4), rn::mul(d3_, d2));
    region = 1;
    if (vc <= 0.0 && d1 >= 0.0 && d3_ <= 0.0) {
        const double v = rn::div(d1, rn::sub(d1, d3_));
        return rn::add(a, rn::scale(v, ab));
    }
    const d3 cp = rn::sub(p, c);
    const double d5 = rn::dot(ab, cp), d6 = rn::dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) {
        region = 0;
        return c;
    }
    const double vb = rn::sub(rn::mul(d5, d2), rn::mul(d1, d6));
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        const double w = rn::div(d2, rn::sub(d2, d6));
        return rn::add(a, rn::scale(w, ac));
    }
    const double va = rn::sub(rn::mul(d3_, d6), rn::mul(d5, d4));
    if (va <= 0.0 && rn::sub(d4, d3_) >= 0.0 && rn::sub(d5, d6) >= 0.0) {
        const double w = rn::div(rn::sub(d4, d3_), rn::add(rn::sub(d4, d3_), rn::sub(d5, d6)));
        return rn::add(b, rn::scale(w, rn::sub(c, b)));
    }
    region = 2;
    const double denom = rn::div(1.0, rn::add(rn::add(va, vb), vc));
    const double v = rn::mul(vb, denom);
    const double w = rn::mul(vc, denom);
    return rn::add(rn::add(a, rn::scale(v, ab)), rn::scale(w, ac));
}

__device__ __forceinline__ d3 closest_pt_triangle(d3 a, d3 b, d3 c, d3 p)
{
    int region;
    return closest_pt_triangle_region(a, b, c, p, region);
}

// The face normal particle_polygonObject_collision_kernel<1> pushes along
// (impl:985-987): -(Q - P) x (R - P), normalised.
__device__ __forceinline__ d3 triangle_normal(d3 P, d3 Q, d3 R)
{
    const d3 c = rn::cross(rn::sub(Q, P), rn::sub(R, P));
    const d3 u = mk(-c.x, -c.y, -c.z);
    return rn::divs(u, rn::length(u));
}

// Per-triangle record of the mixed form's contact pass, written whenever a
// mesh is placed: vertex P and the face normal in FP64 (the plane distance
// of a face contact is n . (x - P)), the edges Q - P and R - P in FP32 (the
// region test relative to the sphere), and the polygon body.
struct __align__(16) TriRec {
    double p[3];
    double n[3];
    float q[3], r[3];
    unsigned body;
    unsigned pad;
};

__device__ __forceinline__ void write_tri_rec(TriRec* __restrict__ out, d3 P, d3 Q, d3 R, unsigned body)
{
    const d3 n = triangle_normal(P, Q, R);
    TriRec t;
    t.p[0] = P.x; t.p[1] = P.y; t.p[2] = P.z;
    t.n[0] = n.x; t.n[1] = n.y; t.n[2] = n.z;
    t.q[0] = (float)rn::sub(Q.x, P.x); t.q[1] = (float)rn::sub(Q.y, P.y); t.q[2] = (float)rn::sub(Q.z, P.z);
    t.r[0] = (float)rn::sub(R.x, P.x); t.r[1] = (float)rn::sub(R.y, P.y); t.r[2] = (float)rn::sub(R.z, P.z);
    t.body = body;
    t.pad = 0;
    *out = t;
}

// ---------------------------------------------- mesh update
//
__device__ __forceinline__ d3 ldp3(const double* a) { return mk(__ldg(a), __ldg(a + 1), __ldg(a + 2)); }

// Body frame to world frame by the Euler parameters (e0 = ex scalar).
__device__ __forceinline__ d3 to_global(d3 v, double ex, double ey, double ez, double ew)
{
    d3 r0 = mk(2.0 * (ex * ex + ey * ey - 0.5), 2.0 * (ey * ez - ex * ew), 2.0 * (ey * ew + ex * ez));
    d3 r1 = mk(2.0 * (ey * ez + ex * ew), 2.0 * (ex * ex + ez * ez - 0.5), 2.0 * (ez * ew - ex * ey));
    d3 r2 = mk(2.0 * (ey * ew - ex * ez), 2.0 * (ez * ew + ex * ey), 2.0 * (ex * ex + ew * ew - 0.5));
    return mk(r0.x * v.x + r0.y * v.y + r0.z * v.z, r1.x * v.x + r1.y * v.y + r1.z * v.z,
              r2.x * v.x + r2.y * v.y + r2.z * v.z);
}

// updatePolygonObjectData_kernel (impl:1911-1956) for triangle id: the world
// vertices from the body's pose, the circumcentre, and the triangle record;
// the new vertices are returned as well.
__device__ __forceinline__ void update_polygon_one(const xd_polygon_mass_info* __restrict__ dpmi,
                                                   const double* __restrict__ vlist, double* __restrict__ sphere,
                                                   xd_polygon_info* __restrict__ dpi, unsigned id, d3& Pv, d3& Qv,
                                                   d3& Rv)
{
    size_t s = (size_t)id * 9;
    int mid = dpi[id].id;
    d3 o = ldp3(dpmi[mid].origin);
    const double* ep = dpmi[mid].ep;
    double ex = __ldg(ep), ey = __ldg(ep + 1), ez = __ldg(ep + 2), ew = __ldg(ep + 3);
    Pv = o + to_global(ldp3(vlist + s + 0), ex, ey, ez, ew);
    Qv = o + to_global(ldp3(vlist + s + 3), ex, ey, ez, ew);
    Rv = o + to_global(ldp3(vlist + s + 6), ex, ey, ez, ew);
    d3 V = Qv - Pv, W = Rv - Pv;
    d3 N = cross(V, W);
    N = N / length(N);
    d3 M1 = 0.5 * (Qv + Pv);
    d3 M2 = 0.5 * (Rv + Pv);
    d3 D1 = cross(N, V), D2 = cross(N, W);
    double t = 0.0;
    if (fabs(D1.x * D2.y - D1.y * D2.x) > 1E-13)
        t = (D2.x * (M1.y - M2.y)) / (D1.x * D2.y - D1.y * D2.x) - (D2.y * (M1.x - M2.x)) / (D1.x * D2.y - D1.y * D2.x);
    else if (fabs(D1.x * D2.z - D1.z * D2.x) > 1E-13)
        t = (D2.x * (M1.z - M2.z)) / (D1.x * D2.z - D1.z * D2.x) - (D2.z * (M1.x - M2.x)) / (D1.x * D2.z - D1.z * D2.x);
    else if (fabs(D1.y * D2.z - D1.z * D2.y) > 1E-13)
        t = (D2.y * (M1.z - M2.z)) / (D1.y * D2.z - D1.z * D2.y) - (D2.z * (M1.y - M2.y)) / (D1.y * D2.z - D1.z * D2.y);
    d3 ctri = M1 + t * D1;
    double* sp = sphere + 4 * (size_t)id;
    sp[0] = ctri.x;
    sp[1] = ctri.y;
    sp[2] = ctri.z;
    st3(dpi[id].P, 0, Pv);
    st3(dpi[id].Q, 0, Qv);
    st3(dpi[id].R, 0, Rv);
}

}  // namespace xd
