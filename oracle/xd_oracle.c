/*
 * xd_oracle.c: CPU restatement of the xdynamics DEM contact step (checker only).
 *
 * TEST INFRASTRUCTURE ONLY -- see xd_oracle.h.  Every function cites the
 * reference lines it restates.  "impl:" means include/mphysics_cuda_impl.cuh,
 * "def.cu:" means source/mphysics_cuda_def.cu of the xdynamics reference.
 *
 * Evaluation order follows the reference expression by expression (vector
 * operators are component-wise, left to right).  Build with -ffp-contract=off
 * so that no multiply-add is fused: the oracle's arithmetic is plain IEEE
 * double, identical on x86-64 and aarch64.
 */
#include "xd_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct { double x, y, z; } v3;

static inline v3 mk(double x, double y, double z) { v3 r = { x, y, z }; return r; }
static inline v3 ld3(const double* a) { return mk(a[0], a[1], a[2]); }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline v3 scl(double s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
static inline v3 dvd(v3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double len(v3 a) { return sqrt(dot(a, a)); }
static inline v3 cross(v3 a, v3 b)
{
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* operator+=(double3&, double3) (impl:43-48) */
static inline void acc3(double* a, v3 b) { a[0] += b.x; a[1] += b.y; a[2] += b.z; }
static inline void st3(double* a, v3 b) { a[0] = b.x; a[1] = b.y; a[2] = b.z; }

/* CUDA's device min(double, double) is fmin. */
static inline double dmin(double a, double b) { return fmin(a, b); }

/* __umul24 (PTX mul24.lo.u32): low 32 bits of the product of the low 24 bits. */
static inline unsigned umul24(unsigned a, unsigned b) { return (a & 0xffffffu) * (b & 0xffffffu); }

unsigned xdo_sizeof_params(void) { return (unsigned)sizeof(xdo_params); }
unsigned xdo_sizeof_plane(void) { return (unsigned)sizeof(xdo_plane); }
unsigned xdo_sizeof_polygon(void) { return (unsigned)sizeof(xdo_polygon); }
unsigned xdo_sizeof_polygon_mass(void) { return (unsigned)sizeof(xdo_polygon_mass); }
unsigned xdo_sizeof_contact_property(void) { return (unsigned)sizeof(xdo_contact_property); }

static double plane_detection(const xdo_plane* pe, v3 xp, v3 wp, v3* u, double r);

/* ------------------------------------------------------------------ grid */

/* calcGridPos (impl:74-83): floor((p - wo) / cs), double -> int. */
void xdo_grid_pos(const xdo_params* prm, const double p[3], int out[3])
{
    out[0] = (int)floor((p[0] - prm->world_origin[0]) / prm->cell_size);
    out[1] = (int)floor((p[1] - prm->world_origin[1]) / prm->cell_size);
    out[2] = (int)floor((p[2] - prm->world_origin[2]) / prm->cell_size);
}

/* calcGridHash (impl:65-72): wrap each coordinate with & (g - 1), then
 * z*gy*gx + y*gx + x with 24-bit multiplies. */
unsigned xdo_grid_hash(const xdo_params* prm, const int c[3])
{
    unsigned x = (unsigned)c[0] & (prm->grid[0] - 1u);
    unsigned y = (unsigned)c[1] & (prm->grid[1] - 1u);
    unsigned z = (unsigned)c[2] & (prm->grid[2] - 1u);
    return umul24(umul24(z, prm->grid[1]), prm->grid[0]) + umul24(y, prm->grid[0]) + x;
}

/* calculateHashAndIndex_kernel (impl:137-151), launcher def.cu:58-66. */
void xdo_calculate_hash_and_index(const xdo_params* prm, unsigned* hash, unsigned* index,
                                  const double* pos, unsigned np)
{
    for (unsigned id = 0; id < np; ++id) {
        int c[3];
        xdo_grid_pos(prm, pos + 4 * (size_t)id, c);
        hash[id] = xdo_grid_hash(prm, c);
        index[id] = id;
    }
}

/* calculateHashAndIndexForPolygonSphere_kernel (impl:153-164), def.cu:68-77:
 * triangle circumspheres go at offset sid with index sid + id. */
void xdo_calculate_hash_and_index_polysphere(const xdo_params* prm, unsigned* hash,
                                             unsigned* index, unsigned sid, unsigned nsphere,
                                             const double* sphere)
{
    for (unsigned id = 0; id < nsphere; ++id) {
        int c[3];
        xdo_grid_pos(prm, sphere + 4 * (size_t)id, c);
        hash[sid + id] = xdo_grid_hash(prm, c);
        index[sid + id] = sid + id;
    }
}

/* Stable LSD counting sort of (key, value) by key, 16 bits per pass.  This
 * restates thrust::sort_by_key on 32-bit keys (def.cu:92-94), whose radix
 * sort keeps equal keys in input order. */
static void stable_sort_by_key(unsigned* key, unsigned* val, unsigned n)
{
    if (n < 2) return;
    unsigned* k2 = (unsigned*)malloc(sizeof(unsigned) * n);
    unsigned* v2 = (unsigned*)malloc(sizeof(unsigned) * n);
    size_t* cnt = (size_t*)malloc(sizeof(size_t) * 65536);
    unsigned *ks = key, *vs = val, *kd = k2, *vd = v2;
    for (int shift = 0; shift < 32; shift += 16) {
        memset(cnt, 0, sizeof(size_t) * 65536);
        for (unsigned i = 0; i < n; ++i) cnt[(ks[i] >> shift) & 0xffffu]++;
        size_t run = 0;
        for (unsigned d = 0; d < 65536; ++d) { size_t c = cnt[d]; cnt[d] = run; run += c; }
        for (unsigned i = 0; i < n; ++i) {
            size_t o = cnt[(ks[i] >> shift) & 0xffffu]++;
            kd[o] = ks[i];
            vd[o] = vs[i];
        }
        unsigned* t;
        t = ks; ks = kd; kd = t;
        t = vs; vs = vd; vd = t;
    }
    /* two passes: the result is back in key/val */
    free(k2);
    free(v2);
    free(cnt);
}

/* cu_reorderDataAndFindCellStart (def.cu:80-108): sort, cstart = ~0 and
 * cend = 0 over all ncell cells, then reorderDataAndFindCellStart_kernel
 * (impl:166-212): a run of equal hashes [b, e) gives cstart[h] = b,
 * cend[h] = e, and sorted_index = index after the sort. */
void xdo_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart,
                                     unsigned* cend, unsigned* sorted_index, unsigned n,
                                     unsigned ncell)
{
    stable_sort_by_key(hash, index, n);
    memset(cstart, 0xff, sizeof(unsigned) * (size_t)ncell);
    memset(cend, 0, sizeof(unsigned) * (size_t)ncell);
    for (unsigned id = 0; id < n; ++id) {
        unsigned h = hash[id];
        if (id == 0 || h != hash[id - 1]) {
            cstart[h] = id;
            if (id > 0) cend[hash[id - 1]] = id;
        }
        if (id == n - 1) cend[h] = id + 1;
        sorted_index[id] = index[id];
    }
}

/* ------------------------------------------------------------ integrator */

/* vv_update_position_kernel (impl:85-96): _p = dt*v + half2dt*a; pos.xyz += _p. */
void xdo_vv_update_position(const xdo_params* prm, double* pos, const double* vel,
                            const double* acc, unsigned np)
{
    for (unsigned id = 0; id < np; ++id) {
        v3 p = add(scl(prm->dt, ld3(vel + 3 * (size_t)id)), scl(prm->half2dt, ld3(acc + 3 * (size_t)id)));
        double* q = pos + 4 * (size_t)id;
        q[0] += p.x;
        q[1] += p.y;
        q[2] += p.z;
    }
}

/* vv_update_velocity_kernel (impl:98-134): a' = (1/m)F, alpha' = (1/I)M,
 * v += (0.5 dt)(a + a'), w += (0.5 dt)(alpha + alpha'), then F = m g, M = 0. */
void xdo_vv_update_velocity(const xdo_params* prm, double* vel, double* acc, double* omega,
                            double* alpha, double* force, double* moment, const double* mass,
                            const double* inertia, unsigned np)
{
    v3 g = ld3(prm->gravity);
    for (unsigned id = 0; id < np; ++id) {
        size_t o = 3 * (size_t)id;
        double m = mass[id];
        v3 v = ld3(vel + o);
        v3 av = ld3(omega + o);
        v3 a = scl(1.0 / m, ld3(force + o));
        v3 in = scl(1.0 / inertia[id], ld3(moment + o));
        double h = 0.5 * prm->dt;
        v = add(v, scl(h, add(ld3(acc + o), a)));
        av = add(av, scl(h, add(ld3(alpha + o), in)));
        st3(force + o, scl(m, g));
        st3(moment + o, mk(0.0, 0.0, 0.0));
        st3(vel + o, v);
        st3(omega + o, av);
        st3(acc + o, a);
        st3(alpha + o, in);
    }
}

/* --------------------------------------------------------- contact model */

typedef struct { double kn, vn, ks, vs, mu, ms; } fconst;

/* getConstant, TCM = 1 (impl:214-256). */
static fconst get_constant(double ir, double jr, double im, double jm,
                           const xdo_contact_property* cp)
{
    fconst c;
    double Meq = jm != 0.0 ? (im * jm) / (im + jm) : im;
    double Req = jr != 0.0 ? (ir * jr) / (ir + jr) : ir;
    double Eeq = (cp->Ei * cp->Ej) / (cp->Ei * (1 - cp->prj * cp->prj) + cp->Ej * (1 - cp->pri * cp->pri));
    double beta = (M_PI / log(cp->rest));
    c.kn = (4.0 / 3.0) * Eeq * sqrt(Req);
    c.vn = sqrt((4.0 * Meq * c.kn) / (1.0 + beta * beta));
    c.ks = c.kn * cp->sratio;
    c.vs = c.vn * cp->sratio;
    c.mu = cp->fric;
    c.ms = cp->rfric;
    return c;
}

/* cohesionForce (impl:259-279). */
static double cohesion_force(double ri, double rj, double Ei, double Ej, double pri, double prj,
                             double coh, double Fn)
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

/* DHSModel (impl:379-401).  Ft and M are in/out: the reference keeps them
 * in the calling kernel across pairs and only assigns them when |e| != 0. */
static void dhs_model(const fconst* c, double ir, double jr, double Ei, double Ej, double pri,
                      double prj, double coh, double cdist, v3 dv, v3 unit, double dt,
                      v3* Ft, v3* Fn, v3* M)
{
    double fsn = -c->kn * pow(cdist, 1.5);
    double fdn = c->vn * dot(dv, unit);
    double fca = cohesion_force(ir, jr, Ei, Ej, pri, prj, coh, fsn);
    *Fn = scl(fsn + fca + fdn, unit);
    v3 e = sub(dv, scl(dot(dv, unit), unit));
    double mag_e = len(e);
    if (mag_e != 0.0) {
        v3 sh = dvd(e, mag_e);
        double ds = mag_e * dt;
        *Ft = scl(dmin(c->ks * ds + c->vs * (dot(dv, sh)), c->mu * len(*Fn)), sh);
        *M = cross(scl(ir, unit), *Ft);
    }
}

/* calculate_p2p_kernel<1> (impl:403-485), launcher def.cu:110-136. */
void xdo_calculate_p2p(const xdo_params* prm, const double* pos, const double* vel,
                       const double* omega, double* force, double* moment, const double* mass,
                       const unsigned* sorted_index, const unsigned* cstart,
                       const unsigned* cend, const xdo_contact_property* cp, unsigned np)
{
    for (unsigned id = 0; id < np; ++id) {
        const double* ip4 = pos + 4 * (size_t)id;
        v3 ipos = ld3(ip4);
        v3 ivel = ld3(vel + 3 * (size_t)id);
        v3 iomega = ld3(omega + 3 * (size_t)id);
        int gp[3];
        xdo_grid_pos(prm, ip4, gp);
        double ir = ip4[3];
        double im = mass[id];
        v3 Ft = mk(0, 0, 0), Fn = mk(0, 0, 0), M = mk(0, 0, 0);
        v3 sumF = mk(0, 0, 0), sumM = mk(0, 0, 0);
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    int nb[3] = { gp[0] + x, gp[1] + y, gp[2] + z };
                    unsigned h = xdo_grid_hash(prm, nb);
                    unsigned st = cstart[h];
                    if (st == 0xffffffffu) continue;
                    unsigned en = cend[h];
                    for (unsigned j = st; j < en; j++) {
                        unsigned k = sorted_index[j];
                        if (id == k || k >= np) continue;
                        const double* jp4 = pos + 4 * (size_t)k;
                        v3 jvel = ld3(vel + 3 * (size_t)k);
                        v3 jomega = ld3(omega + 3 * (size_t)k);
                        double jr = jp4[3];
                        double jm = mass[k];
                        v3 rp = mk(jp4[0] - ipos.x, jp4[1] - ipos.y, jp4[2] - ipos.z);
                        double dist = len(rp);
                        double cdist = (ir + jr) - dist;
                        if (cdist > 0) {
                            v3 unit = dvd(rp, dist);
                            v3 rv = prm->rolling
                                ? sub(add(jvel, cross(jomega, scl(-jr, unit))),
                                      add(ivel, cross(iomega, scl(ir, unit))))
                                : sub(jvel, ivel);
                            fconst c = get_constant(ir, jr, im, jm, cp);
                            dhs_model(&c, ir, jr, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh,
                                      cdist, rv, unit, prm->dt, &Ft, &Fn, &M);
                            sumF = add(sumF, add(Fn, Ft));
                            sumM = add(sumM, M);
                        }
                    }
                }
        acc3(force + 3 * (size_t)id, sumF);
        acc3(moment + 3 * (size_t)id, sumM);
    }
}

void xdo_contact_magnitudes(const xdo_params* prm, const double* pos, const double* vel,
                            const double* omega, const double* mass, const unsigned* sorted_index,
                            const unsigned* cstart, const unsigned* cend,
                            const xdo_contact_property* cp, unsigned np, const xdo_plane* planes,
                            const xdo_contact_property* cp_planes, unsigned nplanes, double* mag)
{
    for (unsigned id = 0; id < np; ++id) {
        const double* ip4 = pos + 4 * (size_t)id;
        v3 ipos = ld3(ip4), ivel = ld3(vel + 3 * (size_t)id), iomega = ld3(omega + 3 * (size_t)id);
        int gp[3];
        xdo_grid_pos(prm, ip4, gp);
        double ir = ip4[3], im = mass[id];
        v3 Ft = mk(0, 0, 0), Fn = mk(0, 0, 0), M = mk(0, 0, 0);
        double sum = 0.0;
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    int nb[3] = { gp[0] + x, gp[1] + y, gp[2] + z };
                    unsigned h = xdo_grid_hash(prm, nb);
                    unsigned st = cstart[h];
                    if (st == 0xffffffffu) continue;
                    for (unsigned j = st; j < cend[h]; j++) {
                        unsigned k = sorted_index[j];
                        if (id == k || k >= np) continue;
                        const double* jp4 = pos + 4 * (size_t)k;
                        v3 rp = mk(jp4[0] - ipos.x, jp4[1] - ipos.y, jp4[2] - ipos.z);
                        double dist = len(rp), jr = jp4[3];
                        double cdist = (ir + jr) - dist;
                        if (cdist > 0) {
                            v3 unit = dvd(rp, dist);
                            v3 jvel = ld3(vel + 3 * (size_t)k), jomega = ld3(omega + 3 * (size_t)k);
                            v3 rv = prm->rolling
                                ? sub(add(jvel, cross(jomega, scl(-jr, unit))), add(ivel, cross(iomega, scl(ir, unit))))
                                : sub(jvel, ivel);
                            fconst c = get_constant(ir, jr, im, mass[k], cp);
                            dhs_model(&c, ir, jr, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh, cdist, rv,
                                      unit, prm->dt, &Ft, &Fn, &M);
                            sum += len(add(Fn, Ft));
                        }
                    }
                }
        for (unsigned w = 0; w < nplanes; ++w) {
            const xdo_plane* pl = planes + w;
            v3 dp = sub(ipos, ld3(pl->xw));
            v3 wp = mk(dot(dp, ld3(pl->u1)), dot(dp, ld3(pl->u2)), dot(dp, ld3(pl->uw)));
            v3 u = mk(0, 0, 0), pFn = mk(0, 0, 0), pFt = mk(0, 0, 0), pM = mk(0, 0, 0);
            double cdist = plane_detection(pl, ipos, wp, &u, ir);
            if (cdist > 0) {
                v3 dv = prm->rolling ? neg(add(ivel, cross(iomega, scl(ir, u)))) : neg(ivel);
                fconst c = get_constant(ir, 0.0, im, 0.0, cp_planes + w);
                dhs_model(&c, 0, 0, 0, 0, 0, 0, cp_planes[w].coh, cdist, dv, u, prm->dt, &pFt, &pFn, &pM);
                sum += len(add(pFn, pFt));
            }
        }
        mag[id] += sum;
    }
}

unsigned long long xdo_pair_list(const xdo_params* prm, const double* pos,
                                 const unsigned* sorted_index, const unsigned* cstart,
                                 const unsigned* cend, unsigned np, unsigned* pairs,
                                 unsigned long long cap)
{
    unsigned long long n = 0;
    for (unsigned id = 0; id < np; ++id) {
        const double* ip4 = pos + 4 * (size_t)id;
        int gp[3];
        xdo_grid_pos(prm, ip4, gp);
        double ir = ip4[3];
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    int nb[3] = { gp[0] + x, gp[1] + y, gp[2] + z };
                    unsigned h = xdo_grid_hash(prm, nb);
                    unsigned st = cstart[h];
                    if (st == 0xffffffffu) continue;
                    unsigned en = cend[h];
                    for (unsigned j = st; j < en; j++) {
                        unsigned k = sorted_index[j];
                        if (id == k || k >= np) continue;
                        const double* jp4 = pos + 4 * (size_t)k;
                        v3 rp = mk(jp4[0] - ip4[0], jp4[1] - ip4[1], jp4[2] - ip4[2]);
                        double cdist = (ir + jp4[3]) - len(rp);
                        if (cdist > 0) {
                            if (n < cap) { pairs[2 * n] = id; pairs[2 * n + 1] = k; }
                            n++;
                        }
                    }
                }
    }
    return n;
}

static inline int sgn(double L) { return L < 0 ? -1 : 1; }

/* particle_plane_contact_detection (impl:487-570): face, 4 corners, 4 edges.
 * The third edge test (impl:549) can never be true (wp.x > 0 && wp.x < 0); it
 * is kept as written. */
static double plane_detection(const xdo_plane* pe, v3 xp, v3 wp, v3* u, double r)
{
    double a_l1 = pow(wp.x - pe->l1, 2.0);
    double b_l2 = pow(wp.y - pe->l2, 2.0);
    double sqa = wp.x * wp.x;
    double sqb = wp.y * wp.y;
    double sqc = wp.z * wp.z;
    double sqr = r * r;
    v3 xw = ld3(pe->xw), w2 = ld3(pe->w2), w3 = ld3(pe->w3), w4 = ld3(pe->w4);

    if (fabs(wp.z) < r && (wp.x > 0 && wp.x < pe->l1) && (wp.y > 0 && wp.y < pe->l2)) {
        v3 dp = sub(xp, xw);
        v3 uw = ld3(pe->uw);
        v3 uu = dvd(uw, len(uw));
        int pp = -sgn(dot(dp, uw));
        *u = scl((double)pp, uu);
        return r - fabs(dot(dp, *u));
    }
    if (wp.x < 0 && wp.y < 0 && (sqa + sqb + sqc) < sqr) {
        v3 X = sub(xp, xw); double h = len(X); *u = dvd(X, h); return r - h;
    } else if (wp.x > pe->l1 && wp.y < 0 && (a_l1 + sqb + sqc) < sqr) {
        v3 X = sub(xp, w2); double h = len(X); *u = dvd(X, h); return r - h;
    } else if (wp.x > pe->l1 && wp.y > pe->l2 && (a_l1 + b_l2 + sqc) < sqr) {
        v3 X = sub(xp, w3); double h = len(X); *u = dvd(X, h); return r - h;
    } else if (wp.x < 0 && wp.y > pe->l2 && (sqa + b_l2 + sqc) < sqr) {
        v3 X = sub(xp, w4); double h = len(X); *u = dvd(X, h); return r - h;
    }
    v3 X, wj, us, hs;
    double h;
    if ((wp.x > 0 && wp.x < pe->l1) && wp.y < 0 && (sqb + sqc) < sqr) {
        X = sub(xp, xw); wj = sub(w2, xw);
    } else if ((wp.x > 0 && wp.x < pe->l1) && wp.y > pe->l2 && (b_l2 + sqc) < sqr) {
        X = sub(xp, w4); wj = sub(w3, w4);
    } else if ((wp.x > 0 && wp.y < pe->l2) && wp.x < 0 && (sqr + sqc) < sqr) {
        X = sub(xp, xw); wj = sub(w4, xw);
    } else if ((wp.x > 0 && wp.y < pe->l2) && wp.x > pe->l1 && (a_l1 + sqc) < sqr) {
        X = sub(xp, w2); wj = sub(w3, w2);
    } else {
        return -1.0;
    }
    us = dvd(wj, len(wj));
    hs = sub(X, scl(dot(X, us), us));
    h = len(hs);
    *u = dvd(neg(hs), h);
    return r - h;
}

/* plane_contact_force_kernel<1> (impl:572-621), launcher def.cu:138-156.
 * DHSModel is called with ir = 0, so the plane adds no moment; with
 * rolling on, dv = -(v + w x (r u)). */
void xdo_plane_contact_force(const xdo_params* prm, const xdo_plane* plane, const double* pos,
                             const double* vel, const double* omega, double* force,
                             double* moment, const double* mass, unsigned np,
                             const xdo_contact_property* cp)
{
    v3 u1 = ld3(plane->u1), u2 = ld3(plane->u2), uw = ld3(plane->uw), xw = ld3(plane->xw);
    for (unsigned id = 0; id < np; ++id) {
        double m = mass[id];
        const double* p4 = pos + 4 * (size_t)id;
        v3 ipos3 = ld3(p4);
        double r = p4[3];
        v3 ivel = ld3(vel + 3 * (size_t)id);
        v3 iomega = ld3(omega + 3 * (size_t)id);
        v3 Fn = mk(0, 0, 0), Ft = mk(0, 0, 0), M = mk(0, 0, 0);
        v3 dp = sub(ipos3, xw);
        v3 unit = mk(0, 0, 0);
        v3 wp = mk(dot(dp, u1), dot(dp, u2), dot(dp, uw));
        double cdist = plane_detection(plane, ipos3, wp, &unit, r);
        if (cdist > 0) {
            v3 dv = prm->rolling ? neg(add(ivel, cross(iomega, scl(r, unit)))) : neg(ivel);
            fconst c = get_constant(r, 0.0, m, 0.0, cp);
            dhs_model(&c, 0, 0, 0, 0, 0, 0, cp->coh, cdist, dv, unit, prm->dt, &Ft, &Fn, &M);
        }
        acc3(force + 3 * (size_t)id, add(Fn, Ft));
        acc3(moment + 3 * (size_t)id, M);
    }
}

/* particle_cylinder_contact_detection (impl:652-719).  The reference returns
 * the depth as float; the rows A1..A3 are makeTFM_1..3 (impl:624-637), toLocal
 * multiplies by their transpose, toGlobal by the rows. */
static double cylinder_detection(const xdo_cylinder* cy, v3 p, double r, v3* u, v3* cp)
{
    v3 pbase = ld3(cy->pbase), ptop = ld3(cy->ptop);
    v3 ab = sub(ptop, pbase);
    double t = dot(sub(p, pbase), ab) / dot(ab, ab);
    v3 c = add(pbase, scl(t, ab));
    double dist = len(sub(p, c));
    if (t >= 0 && t <= 1) {
        *u = dvd(sub(c, p), dist);
        *cp = sub(c, scl(cy->rbase, *u));
        return (double)(float)(cy->rtop + r - dist);
    }
    if (dist < cy->rbase) {
        v3 o2c = sub(ld3(cy->origin), c);
        double lo = len(o2c);
        *u = dvd(o2c, lo);
        *cp = sub(c, scl(cy->rbase, *u));
        return (double)(float)(cy->len * 0.5 + r - lo);
    }
    double ex = cy->ep[0], ey = cy->ep[1], ez = cy->ep[2], ew = cy->ep[3];
    v3 A1 = mk(2.0 * (ex * ex + ey * ey - 0.5), 2.0 * (ey * ez - ex * ew), 2.0 * (ey * ew + ex * ez));
    v3 A2 = mk(2.0 * (ey * ez + ex * ew), 2.0 * (ex * ex + ez * ez - 0.5), 2.0 * (ez * ew - ex * ey));
    v3 A3 = mk(2.0 * (ey * ew - ex * ez), 2.0 * (ez * ew + ex * ey), 2.0 * (ex * ex + ew * ew - 0.5));
    v3 v = sub(p, ptop);
    v3 at = mk(A1.x * v.x + A2.x * v.y + A3.x * v.z, A1.y * v.x + A2.y * v.y + A3.y * v.z,
               A1.z * v.x + A2.z * v.y + A3.z * v.z);
    *cp = ptop;
    if (fabs(at.y) > cy->len) {
        v = sub(p, pbase);
        at = mk(A1.x * v.x + A2.x * v.y + A3.x * v.z, A1.y * v.x + A2.y * v.y + A3.y * v.z,
                A1.z * v.x + A2.z * v.y + A3.z * v.z);
        *cp = pbase;
    }
    double ang = atan(at.x / at.z);
    if (ang < 0 && at.z < 0) c.x = cy->rbase * sin(-ang);
    else if (ang > 0 && at.x < 0 && at.z < 0) c.x = cy->rbase * sin(-ang);
    else c.x = cy->rbase * sin(ang);
    c.z = cy->rbase * cos(ang);
    if (at.z < 0 && c.z > 0) c.z = -c.z;
    else if (at.z > 0 && c.z < 0) c.z = -c.z;
    c.y = 0.;
    *cp = add(*cp, mk(dot(A1, c), dot(A2, c), dot(A3, c)));
    v3 dis = sub(*cp, p);
    dist = len(dis);
    *u = dvd(dis, dist);
    if (dist < r) return (double)(float)(r - dist);
    return -1.0;
}

/* cylinder_hertzian_contact_force_kernel<1> (impl:721-760) for every particle;
 * mf/mm: each particle's reaction on the cylinder (slot 0 included). */
void xdo_cylinder_contact_force(const xdo_params* prm, const xdo_cylinder* cy, const double* pos,
                                const double* vel, const double* omega, double* force, double* moment,
                                const double* mass, unsigned np, const xdo_contact_property* cp,
                                const double mpos[3], double* mf, double* mm)
{
    for (unsigned id = 0; id < np; ++id) {
        const double* p4 = pos + 4 * (size_t)id;
        double r = p4[3];
        v3 ivel = ld3(vel + 3 * (size_t)id), iomega = ld3(omega + 3 * (size_t)id);
        v3 unit = mk(0, 0, 0), cpt = mk(0, 0, 0);
        double cdist = cylinder_detection(cy, ld3(p4), r, &unit, &cpt);
        v3 si = sub(cpt, ld3(mpos));
        v3 cy2cp = sub(cpt, ld3(cy->origin));
        v3 Ft = mk(0, 0, 0), Fn = mk(0, 0, 0), M = mk(0, 0, 0);
        if (cdist > 0) {
            v3 dv = sub(add(ld3(cy->vel), cross(ld3(cy->omega), cy2cp)), add(ivel, cross(iomega, scl(r, unit))));
            fconst c = get_constant(r, 0.0, mass[id], 0.0, cp);
            dhs_model(&c, 0, 0, 0, 0, 0, 0, 0.0, cdist, dv, unit, prm->dt, &Ft, &Fn, &M);
        }
        acc3(force + 3 * (size_t)id, add(Fn, Ft));
        acc3(moment + 3 * (size_t)id, M);
        st3(mf + 3 * (size_t)id, neg(Fn));
        st3(mm + 3 * (size_t)id, cross(si, neg(Fn)));
    }
}

/* cu_cube_contact_force (def.cu:158-179): six plane launches in order. */
void xdo_cube_contact_force(const xdo_params* prm, const xdo_plane* planes6, const double* pos,
                            const double* vel, const double* omega, double* force,
                            double* moment, const double* mass, unsigned np,
                            const xdo_contact_property* cp)
{
    for (int i = 0; i < 6; ++i)
        xdo_plane_contact_force(prm, planes6 + i, pos, vel, omega, force, moment, mass, np, cp);
}

/* closestPtPointTriangle (impl:837-899), Ericson's Voronoi-region test. */
static v3 closest_pt_triangle(v3 a, v3 b, v3 c, v3 p)
{
    v3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    v3 bp = sub(p, b);
    double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) return b;
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        return add(a, scl(v, ab));
    }
    v3 cp = sub(p, c);
    double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) return c;
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        return add(a, scl(w, ac));
    }
    double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return add(b, scl(w, sub(c, b)));
    }
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom;
    double w = vc * denom;
    return add(add(a, scl(v, ab)), scl(w, ac));
}

/* particle_polygonObject_collision_kernel<1> (impl:923-1021), launcher
 * def.cu:203-221.  Grid entries k >= np are triangles (index k - np).  The
 * reaction on the polygon body is accumulated in particle order here; the
 * reference's unsynchronised += on dpmi (impl:1010-1011) has no defined
 * order.  The particle gets no moment (DHSModel with ir = 0). */
void xdo_particle_polygon_collision(const xdo_params* prm, const xdo_polygon* dpi,
                                    const double* sphere, xdo_polygon_mass* dpmi,
                                    const double* pos, const double* vel, const double* omega,
                                    double* force, double* moment, const double* mass,
                                    const unsigned* sorted_index, const unsigned* cstart,
                                    const unsigned* cend, const xdo_contact_property* cp,
                                    unsigned np)
{
    (void)sphere;
    (void)np;
    unsigned cnp = prm->np;
    for (unsigned id = 0; id < cnp; ++id) {
        const double* p4 = pos + 4 * (size_t)id;
        double im = mass[id];
        v3 ipos = ld3(p4);
        v3 ivel = ld3(vel + 3 * (size_t)id);
        v3 iomega = ld3(omega + 3 * (size_t)id);
        int gp[3];
        xdo_grid_pos(prm, p4, gp);
        double ir = p4[3];
        v3 M = mk(0, 0, 0), Fn = mk(0, 0, 0), Ft = mk(0, 0, 0);
        v3 sum_force = mk(0, 0, 0), sum_moment = mk(0, 0, 0);
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    int nb[3] = { gp[0] + x, gp[1] + y, gp[2] + z };
                    unsigned h = xdo_grid_hash(prm, nb);
                    unsigned st = cstart[h];
                    if (st == 0xffffffffu) continue;
                    unsigned en = cend[h];
                    for (unsigned j = st; j < en; j++) {
                        unsigned k = sorted_index[j];
                        if (k < cnp) continue;
                        k -= cnp;
                        const xdo_polygon* tri = dpi + k;
                        unsigned pidx = (unsigned)tri->id;
                        const xdo_contact_property* cmp = cp + pidx;
                        xdo_polygon_mass* pmi = dpmi + pidx;
                        v3 P = ld3(tri->P), Q = ld3(tri->Q), R = ld3(tri->R);
                        v3 cpt = closest_pt_triangle(P, Q, R, ipos);
                        v3 po2cp = sub(cpt, ld3(pmi->origin));
                        v3 distVec = sub(ipos, cpt);
                        double dist = len(distVec);
                        double cdist = ir - dist;
                        Fn = mk(0, 0, 0);
                        if (cdist > 0) {
                            v3 qp = sub(Q, P), rp = sub(R, P);
                            v3 unit = neg(cross(qp, rp));
                            unit = dvd(unit, len(unit));
                            v3 pvel = ld3(pmi->vel), pom = ld3(pmi->omega);
                            v3 dv = prm->rolling
                                ? sub(add(pvel, cross(pom, po2cp)), add(ivel, cross(iomega, scl(ir, unit))))
                                : sub(pvel, ivel);
                            fconst c = get_constant(ir, 0, im, 0, cmp);
                            dhs_model(&c, 0, 0, 0, 0, 0, 0, 0, cdist, dv, unit, prm->dt, &Ft, &Fn, &M);
                            sum_force = add(sum_force, add(Fn, Ft));
                            sum_moment = add(sum_moment, M);
                            acc3(pmi->force, neg(add(Fn, Ft)));
                            acc3(pmi->moment, neg(cross(po2cp, add(Fn, Ft))));
                        }
                    }
                }
        acc3(force + 3 * (size_t)id, sum_force);
        acc3(moment + 3 * (size_t)id, sum_moment);
    }
}

/* toGlobal(double3&, double4&) (impl:1898-1909): rotation by Euler parameters. */
static v3 to_global(v3 v, const double ep[4])
{
    double ex = ep[0], ey = ep[1], ez = ep[2], ew = ep[3];
    v3 r0 = mk(2.0 * (ex * ex + ey * ey - 0.5), 2.0 * (ey * ez - ex * ew), 2.0 * (ey * ew + ex * ez));
    v3 r1 = mk(2.0 * (ey * ez + ex * ew), 2.0 * (ex * ex + ez * ez - 0.5), 2.0 * (ez * ew - ex * ey));
    v3 r2 = mk(2.0 * (ey * ew - ex * ez), 2.0 * (ez * ew + ex * ey), 2.0 * (ex * ex + ew * ew - 0.5));
    return mk(r0.x * v.x + r0.y * v.y + r0.z * v.z,
              r1.x * v.x + r1.y * v.y + r1.z * v.z,
              r2.x * v.x + r2.y * v.y + r2.z * v.z);
}

/* updatePolygonObjectData_kernel (impl:1911-1956), def.cu:469-475: move the
 * local vertices by the body's origin and Euler parameters, recompute the
 * circumcentre.  When all three 2x2 determinants are below 1e-13 the
 * reference leaves t uninitialised; the restatement uses t = 0 there. */
void xdo_update_polygon_object_data(const xdo_polygon_mass* dpmi, const double* vlist,
                                    double* sphere, xdo_polygon* dpi, unsigned ntri)
{
    for (unsigned id = 0; id < ntri; ++id) {
        size_t s = (size_t)id * 9;
        int mid = dpi[id].id;
        v3 o = ld3(dpmi[mid].origin);
        const double* ep = dpmi[mid].ep;
        v3 P = add(o, to_global(ld3(vlist + s + 0), ep));
        v3 Q = add(o, to_global(ld3(vlist + s + 3), ep));
        v3 R = add(o, to_global(ld3(vlist + s + 6), ep));
        v3 V = sub(Q, P), W = sub(R, P);
        v3 N = cross(V, W);
        N = dvd(N, len(N));
        v3 M1 = scl(0.5, add(Q, P));
        v3 M2 = scl(0.5, add(R, P));
        v3 D1 = cross(N, V), D2 = cross(N, W);
        double t = 0.0;
        if (fabs(D1.x * D2.y - D1.y * D2.x) > 1E-13)
            t = (D2.x * (M1.y - M2.y)) / (D1.x * D2.y - D1.y * D2.x) - (D2.y * (M1.x - M2.x)) / (D1.x * D2.y - D1.y * D2.x);
        else if (fabs(D1.x * D2.z - D1.z * D2.x) > 1E-13)
            t = (D2.x * (M1.z - M2.z)) / (D1.x * D2.z - D1.z * D2.x) - (D2.z * (M1.x - M2.x)) / (D1.x * D2.z - D1.z * D2.x);
        else if (fabs(D1.y * D2.z - D1.z * D2.y) > 1E-13)
            t = (D2.y * (M1.z - M2.z)) / (D1.y * D2.z - D1.z * D2.y) - (D2.z * (M1.y - M2.y)) / (D1.y * D2.z - D1.z * D2.y);
        v3 ctri = add(M1, scl(t, D1));
        double* sp = sphere + 4 * (size_t)id;
        sp[0] = ctri.x; sp[1] = ctri.y; sp[2] = ctri.z;
        st3(dpi[id].P, P);
        st3(dpi[id].Q, Q);
        st3(dpi[id].R, R);
    }
}

/* ------------------------------------------------ tangential history */

typedef struct {
    unsigned keys[XDO_HIST_MAX];
    unsigned freem, matched;
} hstate;

static unsigned hist_class(unsigned k) { return k < XDO_HIST_PLANE ? 0u : (k < XDO_HIST_TRI ? 1u : 2u); }

static void hist_begin(const xdo_history* h, unsigned i, hstate* st)
{
    st->freem = 0;
    st->matched = 0;
    for (unsigned s = 0; s < h->slots; ++s) {
        st->keys[s] = h->key[(size_t)s * h->np + i];
        if (st->keys[s] == XDO_HIST_EMPTY) st->freem |= 1u << s;
    }
}

/* The entry of `key` (its old d in d[]), else a free entry (d = 0); -1 when
 * none is free (the contact then has no history this step). */
static int hist_slot(xdo_history* h, hstate* st, unsigned i, unsigned key, double d[3])
{
    d[0] = d[1] = d[2] = 0.0;
    for (unsigned s = 0; s < h->slots; ++s)
        if (st->keys[s] == key) {
            const double* p = h->delta + ((size_t)s * h->np + i) * 3;
            d[0] = p[0]; d[1] = p[1]; d[2] = p[2];
            st->matched |= 1u << s;
            return (int)s;
        }
    if (st->freem) {
        unsigned s = 0;
        while (!(st->freem & (1u << s))) ++s;
        st->freem &= ~(1u << s);
        h->key[(size_t)s * h->np + i] = key;
        return (int)s;
    }
    h->overflow++;
    return -1;
}

static void hist_store(xdo_history* h, int s, unsigned i, const double d[3])
{
    if (s < 0) return;
    double* p = h->delta + ((size_t)s * h->np + i) * 3;
    p[0] = d[0]; p[1] = d[1]; p[2] = d[2];
}

/* entries of class cls whose contact did not recur this step are freed */
static void hist_end(xdo_history* h, const hstate* st, unsigned i, unsigned cls)
{
    for (unsigned s = 0; s < h->slots; ++s) {
        unsigned k = st->keys[s];
        if (k == XDO_HIST_EMPTY || hist_class(k) != cls || (st->matched & (1u << s))) continue;
        h->key[(size_t)s * h->np + i] = XDO_HIST_EMPTY;
        double* p = h->delta + ((size_t)s * h->np + i) * 3;
        p[0] = p[1] = p[2] = 0.0;
    }
}

/* DHSModel's normal force (impl:385-388). */
static v3 normal_force(const fconst* c, double ir, double jr, double Ei, double Ej, double pri,
                       double prj, double coh, double cdist, v3 dv, v3 unit)
{
    double fsn = -c->kn * pow(cdist, 1.5);
    double fdn = c->vn * dot(dv, unit);
    double fca = cohesion_force(ir, jr, Ei, Ej, pri, prj, coh, fsn);
    return scl(fsn + fca + fdn, unit);
}

/* The tangential spring with history (see xd_oracle.h). */
static void hist_tangential(const fconst* c, double ir, v3 dv, v3 unit, double dt, v3 Fn,
                            double d[3], v3* Ft, v3* M)
{
    v3 vt = sub(dv, scl(dot(dv, unit), unit));
    v3 d0 = mk(d[0], d[1], d[2]);
    double m0 = len(d0);
    v3 dp = sub(d0, scl(dot(d0, unit), unit));
    double mp = len(dp);
    v3 dn = mp > 0.0 ? scl(m0 / mp, dp) : mk(0, 0, 0);
    dn = add(dn, scl(dt, vt));
    v3 ft = add(scl(c->ks, dn), scl(c->vs, vt));
    double fmax = c->mu * len(Fn);
    double mf = len(ft);
    if (mf > fmax) {
        ft = scl(fmax / mf, ft);
        dn = dvd(sub(ft, scl(c->vs, vt)), c->ks);
    }
    d[0] = dn.x; d[1] = dn.y; d[2] = dn.z;
    *Ft = ft;
    *M = cross(scl(ir, unit), ft);
}

void xdo_hist_p2p(const xdo_params* prm, const double* pos, const double* vel,
                  const double* omega, double* force, double* moment, const double* mass,
                  const unsigned* sorted_index, const unsigned* cstart, const unsigned* cend,
                  const xdo_contact_property* cp, unsigned np, xdo_history* h)
{
    for (unsigned id = 0; id < np; ++id) {
        const double* ip4 = pos + 4 * (size_t)id;
        v3 ipos = ld3(ip4);
        v3 ivel = ld3(vel + 3 * (size_t)id);
        v3 iomega = ld3(omega + 3 * (size_t)id);
        int gp[3];
        xdo_grid_pos(prm, ip4, gp);
        double ir = ip4[3];
        double im = mass[id];
        hstate st;
        hist_begin(h, id, &st);
        v3 sumF = mk(0, 0, 0), sumM = mk(0, 0, 0);
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    int nb[3] = { gp[0] + x, gp[1] + y, gp[2] + z };
                    unsigned hh = xdo_grid_hash(prm, nb);
                    unsigned s0 = cstart[hh];
                    if (s0 == 0xffffffffu) continue;
                    unsigned en = cend[hh];
                    for (unsigned j = s0; j < en; j++) {
                        unsigned k = sorted_index[j];
                        if (id == k || k >= np) continue;
                        const double* jp4 = pos + 4 * (size_t)k;
                        double jr = jp4[3];
                        v3 rp = mk(jp4[0] - ipos.x, jp4[1] - ipos.y, jp4[2] - ipos.z);
                        double dist = len(rp);
                        double cdist = (ir + jr) - dist;
                        if (cdist > 0) {
                            v3 jvel = ld3(vel + 3 * (size_t)k);
                            v3 jomega = ld3(omega + 3 * (size_t)k);
                            v3 unit = dvd(rp, dist);
                            v3 rv = prm->rolling
                                ? sub(add(jvel, cross(jomega, scl(-jr, unit))),
                                      add(ivel, cross(iomega, scl(ir, unit))))
                                : sub(jvel, ivel);
                            fconst c = get_constant(ir, jr, im, mass[k], cp);
                            v3 Fn = normal_force(&c, ir, jr, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh,
                                                 cdist, rv, unit);
                            double d[3];
                            int sl = hist_slot(h, &st, id, k, d);
                            v3 Ft, M;
                            hist_tangential(&c, ir, rv, unit, prm->dt, Fn, d, &Ft, &M);
                            hist_store(h, sl, id, d);
                            sumF = add(sumF, add(Fn, Ft));
                            sumM = add(sumM, M);
                        }
                    }
                }
        hist_end(h, &st, id, 0u);
        acc3(force + 3 * (size_t)id, sumF);
        acc3(moment + 3 * (size_t)id, sumM);
    }
}

void xdo_hist_planes(const xdo_params* prm, const xdo_plane* planes,
                     const xdo_contact_property* cps, unsigned nplanes, const double* pos,
                     const double* vel, const double* omega, double* force, double* moment,
                     const double* mass, unsigned np, xdo_history* h)
{
    for (unsigned id = 0; id < np; ++id) {
        double m = mass[id];
        const double* p4 = pos + 4 * (size_t)id;
        v3 ipos3 = ld3(p4);
        double r = p4[3];
        v3 ivel = ld3(vel + 3 * (size_t)id);
        v3 iomega = ld3(omega + 3 * (size_t)id);
        hstate st;
        hist_begin(h, id, &st);
        for (unsigned w = 0; w < nplanes; ++w) {
            const xdo_plane* pl = planes + w;
            v3 Fn = mk(0, 0, 0), Ft = mk(0, 0, 0), M = mk(0, 0, 0);
            v3 dp = sub(ipos3, ld3(pl->xw));
            v3 unit = mk(0, 0, 0);
            v3 wp = mk(dot(dp, ld3(pl->u1)), dot(dp, ld3(pl->u2)), dot(dp, ld3(pl->uw)));
            double cdist = plane_detection(pl, ipos3, wp, &unit, r);
            if (cdist > 0) {
                v3 dv = prm->rolling ? neg(add(ivel, cross(iomega, scl(r, unit)))) : neg(ivel);
                fconst c = get_constant(r, 0.0, m, 0.0, cps + w);
                Fn = normal_force(&c, 0, 0, 0, 0, 0, 0, cps[w].coh, cdist, dv, unit);
                double d[3];
                int sl = hist_slot(h, &st, id, XDO_HIST_PLANE | w, d);
                hist_tangential(&c, 0.0, dv, unit, prm->dt, Fn, d, &Ft, &M);
                hist_store(h, sl, id, d);
            }
            acc3(force + 3 * (size_t)id, add(Fn, Ft));
            acc3(moment + 3 * (size_t)id, M);
        }
        hist_end(h, &st, id, 1u);
    }
}

void xdo_hist_polygon(const xdo_params* prm, const xdo_polygon* dpi, xdo_polygon_mass* dpmi,
                      const double* pos, const double* vel, const double* omega, double* force,
                      double* moment, const double* mass, const unsigned* sorted_index,
                      const unsigned* cstart, const unsigned* cend, const xdo_contact_property* cp,
                      xdo_history* h)
{
    unsigned cnp = prm->np;
    for (unsigned id = 0; id < cnp; ++id) {
        const double* p4 = pos + 4 * (size_t)id;
        double im = mass[id];
        v3 ipos = ld3(p4);
        v3 ivel = ld3(vel + 3 * (size_t)id);
        v3 iomega = ld3(omega + 3 * (size_t)id);
        int gp[3];
        xdo_grid_pos(prm, p4, gp);
        double ir = p4[3];
        hstate st;
        hist_begin(h, id, &st);
        v3 sum_force = mk(0, 0, 0), sum_moment = mk(0, 0, 0);
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    int nb[3] = { gp[0] + x, gp[1] + y, gp[2] + z };
                    unsigned hh = xdo_grid_hash(prm, nb);
                    unsigned s0 = cstart[hh];
                    if (s0 == 0xffffffffu) continue;
                    unsigned en = cend[hh];
                    for (unsigned j = s0; j < en; j++) {
                        unsigned k = sorted_index[j];
                        if (k < cnp) continue;
                        k -= cnp;
                        const xdo_polygon* tri = dpi + k;
                        unsigned pidx = (unsigned)tri->id;
                        xdo_polygon_mass* pmi = dpmi + pidx;
                        v3 P = ld3(tri->P), Q = ld3(tri->Q), R = ld3(tri->R);
                        v3 cpt = closest_pt_triangle(P, Q, R, ipos);
                        v3 po2cp = sub(cpt, ld3(pmi->origin));
                        double cdist = ir - len(sub(ipos, cpt));
                        if (cdist > 0) {
                            v3 unit = neg(cross(sub(Q, P), sub(R, P)));
                            unit = dvd(unit, len(unit));
                            v3 pvel = ld3(pmi->vel), pom = ld3(pmi->omega);
                            v3 dv = prm->rolling
                                ? sub(add(pvel, cross(pom, po2cp)), add(ivel, cross(iomega, scl(ir, unit))))
                                : sub(pvel, ivel);
                            fconst c = get_constant(ir, 0, im, 0, cp + pidx);
                            v3 Fn = normal_force(&c, 0, 0, 0, 0, 0, 0, 0, cdist, dv, unit);
                            double d[3];
                            int sl = hist_slot(h, &st, id, XDO_HIST_TRI | k, d);
                            v3 Ft, M;
                            hist_tangential(&c, 0.0, dv, unit, prm->dt, Fn, d, &Ft, &M);
                            hist_store(h, sl, id, d);
                            sum_force = add(sum_force, add(Fn, Ft));
                            sum_moment = add(sum_moment, M);
                            acc3(pmi->force, neg(add(Fn, Ft)));
                            acc3(pmi->moment, neg(cross(po2cp, add(Fn, Ft))));
                        }
                    }
                }
        hist_end(h, &st, id, 2u);
        acc3(force + 3 * (size_t)id, sum_force);
        acc3(moment + 3 * (size_t)id, sum_moment);
    }
}

/* ------------------------------------------------------ kinematic bodies */

void xdo_advance_bodies(xdo_polygon_mass* pmi, unsigned nbodies, double dt)
{
    for (unsigned b = 0; b < nbodies; ++b) {
        xdo_polygon_mass* m = pmi + b;
        for (int a = 0; a < 3; ++a) m->origin[a] = m->origin[a] + dt * m->vel[a];
        double wx = m->omega[0], wy = m->omega[1], wz = m->omega[2];
        double w = sqrt(wx * wx + wy * wy + wz * wz);
        if (w > 0.0) {
            double h = 0.5 * w * dt;
            double c = cos(h), sn = sin(h) / w;
            double a0 = c, a1 = sn * wx, a2 = sn * wy, a3 = sn * wz;
            double p0 = m->ep[0], p1 = m->ep[1], p2 = m->ep[2], p3 = m->ep[3];
            double r0 = a0 * p0 - (a1 * p1 + a2 * p2 + a3 * p3);
            double r1 = a0 * p1 + p0 * a1 + (a2 * p3 - a3 * p2);
            double r2 = a0 * p2 + p0 * a2 + (a3 * p1 - a1 * p3);
            double r3 = a0 * p3 + p0 * a3 + (a1 * p2 - a2 * p1);
            double nr = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + r3 * r3);
            m->ep[0] = r0 / nr;
            m->ep[1] = r1 / nr;
            m->ep[2] = r2 / nr;
            m->ep[3] = r3 / nr;
        }
    }
}

/* ------------------------------------------------------------ whole step */

/* dem_simulation::oneStepAnalysis (dem_simulation.cpp:447-469) with
 * contactManager::deviceCollision (contactManager.cpp:156-185):
 * VV position, grid, particle-particle, planes in name order, polygons,
 * VV velocity (which also resets F = m g, M = 0). */
unsigned xdo_emitter_before_step(xdo_emitter* e, unsigned np)
{
    e->step += 1;
    if (e->period && (e->step - 1) % e->period == 0 && e->active < np) {
        unsigned add = 1;
        if (e->groups) add = e->next < e->ngroups ? e->groups[e->next++] : 0;
        e->active = add > np - e->active ? np : e->active + add;
    }
    return e->active;
}

void xdo_step(xdo_scene* s)
{
    /* with an emitter the step runs over the active particles, the parameter
     * block's np included (the polygon pass reads it) */
    xdo_params local = s->prm;
    xdo_params* prm = &local;
    unsigned np = s->emit ? xdo_emitter_before_step(s->emit, s->np) : s->np;
    local.np = s->emit ? np : s->prm.np;
    unsigned n = np + s->ntri;
    if (s->kinematic && s->ntri) {
        xdo_advance_bodies(s->pmi, s->nbodies, prm->dt);
        xdo_update_polygon_object_data(s->pmi, s->vlist, s->sphere, s->poly, s->ntri);
    }
    xdo_vv_update_position(prm, s->pos, s->vel, s->acc, np);
    xdo_calculate_hash_and_index(prm, s->hash, s->index, s->pos, np);
    if (s->ntri)
        xdo_calculate_hash_and_index_polysphere(prm, s->hash, s->index, np, s->ntri, s->sphere);
    xdo_reorder_and_find_cell_start(s->hash, s->index, s->cstart, s->cend, s->sorted, n, prm->ncell);
    if (s->hist) {
        if (s->cp_pp)
            xdo_hist_p2p(prm, s->pos, s->vel, s->omega, s->force, s->moment, s->mass, s->sorted,
                         s->cstart, s->cend, s->cp_pp, np, s->hist);
        if (s->nplanes)
            xdo_hist_planes(prm, s->planes, s->cp_planes, s->nplanes, s->pos, s->vel, s->omega,
                            s->force, s->moment, s->mass, np, s->hist);
        if (s->ntri)
            xdo_hist_polygon(prm, s->poly, s->pmi, s->pos, s->vel, s->omega, s->force, s->moment,
                             s->mass, s->sorted, s->cstart, s->cend, s->cp_poly, s->hist);
    } else {
        if (s->cp_pp)
            xdo_calculate_p2p(prm, s->pos, s->vel, s->omega, s->force, s->moment, s->mass,
                              s->sorted, s->cstart, s->cend, s->cp_pp, np);
        for (unsigned i = 0; i < s->nplanes; ++i)
            xdo_plane_contact_force(prm, s->planes + i, s->pos, s->vel, s->omega, s->force,
                                    s->moment, s->mass, np, s->cp_planes + i);
        if (s->ntri)
            xdo_particle_polygon_collision(prm, s->poly, s->sphere, s->pmi, s->pos, s->vel,
                                           s->omega, s->force, s->moment, s->mass, s->sorted,
                                           s->cstart, s->cend, s->cp_poly, np);
    }
    xdo_vv_update_velocity(prm, s->vel, s->acc, s->omega, s->alpha, s->force, s->moment, s->mass,
                           s->inertia, np);
}

void xdo_run_steps(xdo_scene* s, unsigned nsteps)
{
    for (unsigned i = 0; i < nsteps; ++i) xdo_step(s);
}

/* ------------------------------------------------- reference CPU path */

/* grid_base::getCellNumber (grid_base.cpp:139-146) takes abs(floor(.)),
 * grid_base::getHash (grid_base.cpp:148-155). */
static unsigned cpu_hash(const xdo_params* prm, double x, double y, double z, int out[3])
{
    out[0] = abs((int)floor((x - prm->world_origin[0]) / prm->cell_size));
    out[1] = abs((int)floor((y - prm->world_origin[1]) / prm->cell_size));
    out[2] = abs((int)floor((z - prm->world_origin[2]) / prm->cell_size));
    return 0;
}

static unsigned cpu_get_hash(const xdo_params* prm, const int c[3])
{
    int gx = (int)prm->grid[0], gy = (int)prm->grid[1], gz = (int)prm->grid[2];
    int x = c[0] & (gx - 1), y = c[1] & (gy - 1), z = c[2] & (gz - 1);
    return (unsigned)((z * gy) * gx + (y * gx) + x);
}

/* contact::DHSModel (contact.cpp:20-46): F is assigned Fn + Ft, M = cp x Ft
 * only when |e| != 0 (otherwise M keeps its value). */
static void cpu_dhs(const fconst* c, double friction, double cdist, v3 cp, v3 dv, v3 unit,
                    double dt, v3* F, v3* M)
{
    v3 Fn, Ft = mk(0, 0, 0);
    double fsn = (-c->kn * pow(cdist, 1.5));
    double fsd = c->vn * dot(dv, unit);
    Fn = scl(fsn + 0.0 + fsd, unit);
    v3 e = sub(dv, scl(dot(dv, unit), unit));
    double mag_e = len(e);
    if (mag_e != 0.0) {
        v3 s_hat = dvd(e, mag_e);
        double ds = mag_e * dt;
        double ft1 = c->ks * ds + c->vs * dot(dv, s_hat);
        double ft2 = friction * len(Fn);
        Ft = scl(ft1 < ft2 ? ft1 : ft2, s_hat);
        *M = cross(cp, Ft);
    }
    *F = add(Fn, Ft);
}

/* One CPU step: velocity_verlet::updatePosition CPU branch
 * (velocity_verlet.cpp:22-33), neighborhood_cell::_detection
 * (neighborhood_cell.cpp:31-84), contactManager::hostCollision
 * (contactManager.cpp:208-277) with contact_particles_plane::singleCollision
 * (contact_particles_plane.cpp:209-236) and
 * contact_particles_particles::cppCollision
 * (contact_particles_particles.cpp:53-89), velocity_verlet::updateVelocity
 * CPU branch (velocity_verlet.cpp:44-66).  Triangle spheres join the grid
 * after the particles (neighborhood_cell.cpp:44-50) and grid entries k >= np
 * are polygon contacts, contact_particles_polygonObjects::cppolyCollision
 * (contact_particles_polygonObjects.cpp:202-256): closest point
 * (particle_polygon_contact_detection, :540-606), the face-winding normal,
 * moment arm rcon u with rcon = r - cdist / 2, wall velocity
 * v_body + w_body x (cp - origin), the reaction -F added to the body.  The
 * start/end loop of _detection reads one element past the sorted keys
 * (neighborhood_cell.cpp:76); the restatement treats that element as a key
 * that differs from the last one. */
static void cpu_poly_contact(const xdo_scene* s, unsigned t, double r, double m, v3 p, v3 v, v3 o, v3* F,
                             v3* M)
{
    const xdo_polygon* tri = s->poly + t;
    const unsigned b = (unsigned)tri->id;
    xdo_polygon_mass* pm = s->pmi + b;
    const xdo_contact_property* cp = s->cp_poly + b;
    v3 P = ld3(tri->P), Q = ld3(tri->Q), R = ld3(tri->R);
    v3 cpt = closest_pt_triangle(P, Q, R, p);
    v3 po2cp = sub(cpt, ld3(pm->origin));
    double cdist = r - len(sub(p, cpt));
    if (!(cdist > 0)) return;
    v3 u = neg(cross(sub(Q, P), sub(R, P)));
    u = dvd(u, len(u));
    double rcon = r - 0.5 * cdist;
    v3 dv = sub(add(ld3(pm->vel), cross(ld3(pm->omega), po2cp)), add(v, cross(o, scl(r, u))));
    fconst c = get_constant(r, 0.0, m, 0.0, cp);
    v3 mf, mm = mk(0, 0, 0);
    cpu_dhs(&c, cp->fric, cdist, scl(rcon, u), dv, u, s->prm.dt, &mf, &mm);
    *F = add(*F, mf);
    *M = add(*M, mm);
    acc3(pm->force, neg(mf));
}

void xdo_cpu_step(xdo_scene* s)
{
    xdo_params* prm = &s->prm;
    unsigned np = s->np;
    const unsigned ng = np + s->ntri;
    double dt = prm->dt;
    double sqt_dt = 0.5 * dt * dt;
    for (unsigned i = 0; i < np; i++) {
        double* p = s->pos + 4 * (size_t)i;
        v3 old_p = ld3(p);
        v3 new_p = add(add(old_p, scl(dt, ld3(s->vel + 3 * (size_t)i))), scl(sqt_dt, ld3(s->acc + 3 * (size_t)i)));
        p[0] = new_p.x; p[1] = new_p.y; p[2] = new_p.z;
    }
    for (unsigned i = 0; i < ng; i++) {
        int c[3];
        const double* p = i < np ? s->pos + 4 * (size_t)i : s->sphere + 4 * (size_t)(i - np);
        cpu_hash(prm, p[0], p[1], p[2], c);
        s->hash[i] = cpu_get_hash(prm, c);
        s->index[i] = i;
    }
    stable_sort_by_key(s->hash, s->index, ng);
    memset(s->cstart, 0xff, sizeof(unsigned) * (size_t)prm->ncell);
    memset(s->cend, 0, sizeof(unsigned) * (size_t)prm->ncell);
    for (unsigned i = 0; i < s->nbodies && s->ntri; ++i) {
        s->pmi[i].force[0] = s->pmi[i].force[1] = s->pmi[i].force[2] = 0.0;
    }
    for (unsigned b = 0; b < ng;) {
        unsigned e = b + 1;
        while (e < ng && s->hash[e] == s->hash[b]) e++;
        s->cstart[s->hash[b]] = b;
        s->cend[s->hash[b]] = e;
        for (unsigned j = b; j < e; j++) s->sorted[j] = s->index[j];
        b = e;
    }
    for (unsigned i = 0; i < np; i++) {
        v3 F = mk(0, 0, 0), M = mk(0, 0, 0);
        const double* p4 = s->pos + 4 * (size_t)i;
        v3 p = ld3(p4);
        v3 v = ld3(s->vel + 3 * (size_t)i);
        v3 o = ld3(s->omega + 3 * (size_t)i);
        double m = s->mass[i];
        double r = p4[3];
        for (unsigned w = 0; w < s->nplanes; ++w) {
            const xdo_plane* pe = s->planes + w;
            v3 dp = sub(p, ld3(pe->xw));
            v3 wp = mk(dot(dp, ld3(pe->u1)), dot(dp, ld3(pe->u2)), dot(dp, ld3(pe->uw)));
            v3 u = mk(0, 0, 0);
            double cdist = plane_detection(pe, p, wp, &u, r);
            if (cdist > 0) {
                double rcon = r - 0.5 * cdist;
                fconst c = get_constant(r, 0.0, m, 0.0, s->cp_planes + w);
                cpu_dhs(&c, s->cp_planes[w].fric, cdist, scl(rcon, u), neg(v), u, dt, &F, &M);
            }
        }
        int gp[3];
        cpu_hash(prm, p.x, p.y, p.z, gp);
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    int nb[3] = { gp[0] + x, gp[1] + y, gp[2] + z };
                    unsigned h = cpu_get_hash(prm, nb);
                    unsigned sid = s->cstart[h];
                    if (sid == 0xffffffffu) continue;
                    unsigned eid = s->cend[h];
                    for (unsigned j = sid; j < eid; j++) {
                        unsigned k = s->sorted[j];
                        if (k >= np) {
                            cpu_poly_contact(s, k - np, r, m, p, v, o, &F, &M);
                            continue;
                        }
                        if (i == k) continue;
                        const double* q4 = s->pos + 4 * (size_t)k;
                        v3 jp = ld3(q4);
                        double jr = q4[3];
                        v3 rp = sub(jp, p);
                        double dist = len(rp);
                        double cdist = (r + jr) - dist;
                        if (cdist > 0) {
                            v3 u = dvd(rp, dist);
                            double rcon = r - 0.5 * cdist;
                            v3 jv = ld3(s->vel + 3 * (size_t)k);
                            v3 jo = ld3(s->omega + 3 * (size_t)k);
                            v3 rv = sub(add(jv, cross(jo, scl(-jr, u))), add(v, cross(o, scl(r, u))));
                            fconst c = get_constant(r, jr, m, s->mass[k], s->cp_pp);
                            v3 mf, mm = mk(0, 0, 0);
                            cpu_dhs(&c, s->cp_pp->fric, cdist, scl(rcon, u), rv, u, dt, &mf, &mm);
                            F = add(F, mf);
                            M = add(M, mm);
                        }
                    }
                }
        acc3(s->force + 3 * (size_t)i, F);
        acc3(s->moment + 3 * (size_t)i, M);
    }
    v3 g = ld3(prm->gravity);
    for (unsigned i = 0; i < np; i++) {
        size_t o = 3 * (size_t)i;
        double inv_m = 1.0 / s->mass[i];
        double inv_i = 1.0 / s->inertia[i];
        v3 v = add(ld3(s->vel + o), scl(0.5 * dt, ld3(s->acc + o)));
        v3 w = add(ld3(s->omega + o), scl(0.5 * dt, ld3(s->alpha + o)));
        v3 a = scl(inv_m, ld3(s->force + o));
        v3 aa = scl(inv_i, ld3(s->moment + o));
        v = add(v, scl(0.5 * dt, a));
        w = add(w, scl(0.5 * dt, aa));
        st3(s->vel + o, v);
        st3(s->omega + o, w);
        st3(s->acc + o, a);
        st3(s->alpha + o, aa);
        st3(s->force + o, scl(s->mass[i], g));
        st3(s->moment + o, mk(0, 0, 0));
    }
}

void xdo_cpu_run_steps(xdo_scene* s, unsigned nsteps)
{
    for (unsigned i = 0; i < nsteps; ++i) xdo_cpu_step(s);
}
