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

// particle_plane_contact_detection (impl:487-570); pow(x, 2.0) is x * x
// (IEEE: the correctly rounded square).
__device__ __forceinline__ double plane_detection(const PlaneD& pe, d3 xp, d3 wp, d3& u, double r)
{
    double a_l1 = (wp.x - pe.l1) * (wp.x - pe.l1);
    double b_l2 = (wp.y - pe.l2) * (wp.y - pe.l2);
    double sqa = wp.x * wp.x;
    double sqb = wp.y * wp.y;
    double sqc = wp.z * wp.z;
    double sqr = r * r;
    if (fabs(wp.z) < r && (wp.x > 0 && wp.x < pe.l1) && (wp.y > 0 && wp.y < pe.l2)) {
        d3 dp = xp - pe.xw;
        d3 uu = pe.uw / length(pe.uw);
        int pp = -sgn(dot(dp, pe.uw));
        u = (double)pp * uu;
        return r - fabs(dot(dp, u));
    }
    if (wp.x < 0 && wp.y < 0 && (sqa + sqb + sqc) < sqr) {
        d3 X = xp - pe.xw; double h = length(X); u = X / h; return r - h;
    } else if (wp.x > pe.l1 && wp.y < 0 && (a_l1 + sqb + sqc) < sqr) {
        d3 X = xp - pe.w2; double h = length(X); u = X / h; return r - h;
    } else if (wp.x > pe.l1 && wp.y > pe.l2 && (a_l1 + b_l2 + sqc) < sqr) {
        d3 X = xp - pe.w3; double h = length(X); u = X / h; return r - h;
    } else if (wp.x < 0 && wp.y > pe.l2 && (sqa + b_l2 + sqc) < sqr) {
        d3 X = xp - pe.w4; double h = length(X); u = X / h; return r - h;
    }
    d3 X, wj;
    if ((wp.x > 0 && wp.x < pe.l1) && wp.y < 0 && (sqb + sqc) < sqr) {
        X = xp - pe.xw; wj = pe.w2 - pe.xw;
    } else if ((wp.x > 0 && wp.x < pe.l1) && wp.y > pe.l2 && (b_l2 + sqc) < sqr) {
        X = xp - pe.w4; wj = pe.w3 - pe.w4;
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x < 0 && (sqr + sqc) < sqr) {
        X = xp - pe.xw; wj = pe.w4 - pe.xw;
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x > pe.l1 && (a_l1 + sqc) < sqr) {
        X = xp - pe.w2; wj = pe.w3 - pe.w2;
    } else {
        return -1.0;
    }
    d3 us = wj / length(wj);
    d3 hs = X - (dot(X, us)) * us;
    double h = length(hs);
    u = (-hs) / h;
    return r - h;
}

// closestPtPointTriangle (impl:837-899)
__device__ __forceinline__ d3 closest_pt_triangle(d3 a, d3 b, d3 c, d3 p)
{
    d3 ab = b - a, ac = c - a, ap = p - a;
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    d3 bp = p - b;
    double d3_ = dot(ab, bp), d4 = dot(ac, bp);
    if (d3_ >= 0.0 && d4 <= d3_) return b;
    double vc = d1 * d4 - d3_ * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3_ <= 0.0) {
        double v = d1 / (d1 - d3_);
        return a + v * ab;
    }
    d3 cp = p - c;
    double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) return c;
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        return a + w * ac;
    }
    double va = d3_ * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3_) >= 0.0 && (d5 - d6) >= 0.0) {
        double w = (d4 - d3_) / ((d4 - d3_) + (d5 - d6));
        return b + w * (c - b);
    }
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom;
    double w = vc * denom;
    return (a + v * ab) + w * ac;
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
