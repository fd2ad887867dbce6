/*
 * xd_oracle: CPU restatement of the xdynamics DEM contact step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the CUDA library in
 * metakonga_gb300/csrc: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.  The product never links or calls it.
 *
 * Two semantics are restated:
 *   xdo_*      the reference's live FP64 GPU path (include/mphysics_cuda_impl.cuh,
 *              source/mphysics_cuda_def.cu), evaluated in IEEE double with no
 *              FMA contraction (build with -ffp-contract=off).  This is the
 *              parity oracle.
 *   xdo_cpu_*  the reference's CPU path (source/velocity_verlet.cpp,
 *              source/neighborhood_cell.cpp, source/contactManager.cpp,
 *              source/collision/contact*.cpp), single threaded like the
 *              reference; used as the timed CPU baseline.
 *
 * Pinning: the xdo_* functions are checked bit for bit against the reference's
 * own kernels compiled as host code (oracle/ref_driver.cpp -> oracle/_ref) and
 * against the golden fixtures generated from them (tests/golden).
 *
 * All arrays use the reference's boundary layouts: pos = double4 (x,y,z,r),
 * vel/acc/omega/alpha/force/moment = packed double3, mass/inertia = double.
 * The structs below have the byte layout of the reference's device structs
 * (include/mphysics_cuda_dec.cuh:17-88) so the same buffers feed the oracle,
 * the reference build and the CUDA library.
 */
#ifndef XD_ORACLE_H
#define XD_ORACLE_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* include/mphysics_cuda_dec.cuh:17-30 (device_parameters), 112 bytes */
typedef struct xdo_params {
    bool rolling;
    unsigned np;
    unsigned nsphere;
    unsigned ncell;
    unsigned grid[3];
    double dt;
    double half2dt;
    double cell_size;
    double cohesion;
    double gravity[3];
    double world_origin[3];
} xdo_params;

/* include/mphysics_cuda_dec.cuh:78-88 (device_contact_property), 88 bytes */
typedef struct xdo_contact_property {
    double Ei, Ej, pri, prj, Gi, Gj, rest, fric, rfric, coh, sratio;
} xdo_contact_property;

/* include/mphysics_cuda_dec.cuh:43-55 (device_plane_info), 232 bytes */
typedef struct xdo_plane {
    double l1, l2;
    double u1[3], u2[3], uw[3], xw[3], pa[3], pb[3], w2[3], w3[3], w4[3];
} xdo_plane;

/* include/mphysics_cuda_dec.cuh:67-76 (device_cylinder_info), 176 bytes */
typedef struct xdo_cylinder {
    double len, rbase, rtop;
    double pbase[3], ptop[3], origin[3], vel[3], omega[3];
    double ep[4];
} xdo_cylinder;

/* include/mphysics_cuda_dec.cuh:32-41 (device_polygon_info), 152 bytes */
typedef struct xdo_polygon {
    int id;
    double P[3], Q[3], R[3], V[3], W[3], N[3];
} xdo_polygon;

/* include/mphysics_cuda_dec.cuh:57-65 (device_polygon_mass_info), 160 bytes;
 * ep is a CUDA double4 (16-byte aligned). */
typedef struct xdo_polygon_mass {
    double origin[3];
    _Alignas(16) double ep[4];
    double vel[3], omega[3], force[3], moment[3];
} xdo_polygon_mass;

unsigned xdo_sizeof_params(void);
unsigned xdo_sizeof_plane(void);
unsigned xdo_sizeof_polygon(void);
unsigned xdo_sizeof_polygon_mass(void);
unsigned xdo_sizeof_contact_property(void);

/* ---- cell grid (impl:65-83, 137-212; def.cu:58-108) ---- */
void xdo_grid_pos(const xdo_params* prm, const double p[3], int out[3]);
unsigned xdo_grid_hash(const xdo_params* prm, const int c[3]);
void xdo_calculate_hash_and_index(const xdo_params* prm, unsigned* hash, unsigned* index,
                                  const double* pos, unsigned np);
void xdo_calculate_hash_and_index_polysphere(const xdo_params* prm, unsigned* hash,
                                             unsigned* index, unsigned sid, unsigned nsphere,
                                             const double* sphere);
void xdo_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart,
                                     unsigned* cend, unsigned* sorted_index, unsigned n,
                                     unsigned ncell);

/* ---- integrator (impl:85-134) ---- */
void xdo_vv_update_position(const xdo_params* prm, double* pos, const double* vel,
                            const double* acc, unsigned np);
void xdo_vv_update_velocity(const xdo_params* prm, double* vel, double* acc, double* omega,
                            double* alpha, double* force, double* moment, const double* mass,
                            const double* inertia, unsigned np);

/* ---- contact forces (impl:214-621, 837-1021) ---- */
void xdo_calculate_p2p(const xdo_params* prm, const double* pos, const double* vel,
                       const double* omega, double* force, double* moment, const double* mass,
                       const unsigned* sorted_index, const unsigned* cstart,
                       const unsigned* cend, const xdo_contact_property* cp, unsigned np);
void xdo_plane_contact_force(const xdo_params* prm, const xdo_plane* plane, const double* pos,
                             const double* vel, const double* omega, double* force,
                             double* moment, const double* mass, unsigned np,
                             const xdo_contact_property* cp);
void xdo_cylinder_contact_force(const xdo_params* prm, const xdo_cylinder* cy, const double* pos,
                                const double* vel, const double* omega, double* force, double* moment,
                                const double* mass, unsigned np, const xdo_contact_property* cp,
                                const double mpos[3], double* mf, double* mm);
void xdo_cube_contact_force(const xdo_params* prm, const xdo_plane* planes6, const double* pos,
                            const double* vel, const double* omega, double* force,
                            double* moment, const double* mass, unsigned np,
                            const xdo_contact_property* cp);
void xdo_particle_polygon_collision(const xdo_params* prm, const xdo_polygon* dpi,
                                    const double* sphere, xdo_polygon_mass* dpmi,
                                    const double* pos, const double* vel, const double* omega,
                                    double* force, double* moment, const double* mass,
                                    const unsigned* sorted_index, const unsigned* cstart,
                                    const unsigned* cend, const xdo_contact_property* cp,
                                    unsigned np);
void xdo_update_polygon_object_data(const xdo_polygon_mass* dpmi, const double* vlist,
                                    double* sphere, xdo_polygon* dpi, unsigned ntri);

/* Per-particle sum of contact force magnitudes, sum_c |Fn + Ft|, over the
 * particle-particle contacts (mag_pp) and the plane contacts (mag_planes),
 * added into mag[np]: the normaliser of the per-step force error. */
void xdo_contact_magnitudes(const xdo_params* prm, const double* pos, const double* vel,
                            const double* omega, const double* mass, const unsigned* sorted_index,
                            const unsigned* cstart, const unsigned* cend,
                            const xdo_contact_property* cp, unsigned np, const xdo_plane* planes,
                            const xdo_contact_property* cp_planes, unsigned nplanes, double* mag);

/* Contact pair list of one step: for every particle i (ascending) every
 * partner k found by the 27-cell search with cdist > 0, in search order.
 * Writes up to cap pairs as (i, k); returns the total number of pairs. */
unsigned long long xdo_pair_list(const xdo_params* prm, const double* pos,
                                 const unsigned* sorted_index, const unsigned* cstart,
                                 const unsigned* cend, unsigned np, unsigned* pairs,
                                 unsigned long long cap);

/* ---- tangential-spring history: an extension with no counterpart in the
 *      reference (its DHSModel, impl:379-401, keeps no state between steps).
 *      Each particle holds up to `slots` contacts keyed by partner: particle
 *      j -> j, plane w -> XDO_HIST_PLANE | w, triangle t -> XDO_HIST_TRI | t.
 *      Per contact and step, with vt the tangential relative velocity:
 *        d <- d - (d.u)u, rescaled to |d| (turned onto the new tangent plane)
 *        d <- d + vt dt;  Ft = ks d + vs vt
 *        if |Ft| > mu |Fn|: Ft <- (mu |Fn| / |Ft|) Ft, d <- (Ft - vs vt) / ks
 *        M = (ir u) x Ft  (ir = 0 for planes and triangles, as in the reference)
 *      A new contact starts from d = 0, so its first step gives the
 *      reference's DHS force; a contact that ends frees its entry. ---- */
#define XDO_HIST_EMPTY 0xffffffffu
#define XDO_HIST_PLANE 0x80000000u
#define XDO_HIST_TRI 0xC0000000u
#define XDO_HIST_MAX 32
typedef struct xdo_history {
    unsigned slots;                /* entries per particle, <= XDO_HIST_MAX */
    unsigned np;
    unsigned* key;                 /* key[s * np + i] */
    double* delta;                 /* delta[(s * np + i) * 3 + a] */
    unsigned long long overflow;   /* contacts that found no free entry (force without history) */
} xdo_history;

void xdo_hist_p2p(const xdo_params* prm, const double* pos, const double* vel,
                  const double* omega, double* force, double* moment, const double* mass,
                  const unsigned* sorted_index, const unsigned* cstart, const unsigned* cend,
                  const xdo_contact_property* cp, unsigned np, xdo_history* h);
void xdo_hist_planes(const xdo_params* prm, const xdo_plane* planes,
                     const xdo_contact_property* cps, unsigned nplanes, const double* pos,
                     const double* vel, const double* omega, double* force, double* moment,
                     const double* mass, unsigned np, xdo_history* h);
void xdo_hist_polygon(const xdo_params* prm, const xdo_polygon* dpi, xdo_polygon_mass* dpmi,
                      const double* pos, const double* vel, const double* omega, double* force,
                      double* moment, const double* mass, const unsigned* sorted_index,
                      const unsigned* cstart, const unsigned* cend, const xdo_contact_property* cp,
                      xdo_history* h);

/* Particle emitter, the reference's real-time creation
 * (dem_simulation.cpp:210-222 sets the period, :321-322 starts from no
 * particle, :449-450 adds a group before a step; particleManager.cpp:132-145
 * hands out the groups, or one particle at a time): the scene's np particles
 * are staged in memory and only the first `active` take part in a step.
 * Before step k (1-based, counted from when the emitter was set), when
 * period > 0, (k - 1) % period == 0 and active < np, active grows by the next
 * group size (by one when groups is NULL; by nothing once the groups are used
 * up), clamped to np.  The grid, the contacts and velocity-Verlet then run
 * over the active particles, and triangles sit at grid index active + t. */
typedef struct xdo_emitter {
    unsigned period;
    const unsigned* groups;
    unsigned ngroups;
    unsigned next;               /* next group to hand out */
    unsigned active;
    unsigned long long step;     /* steps run since the emitter was set */
} xdo_emitter;

/* Advances the emitter by one step and returns the active count of that step. */
unsigned xdo_emitter_before_step(xdo_emitter* e, unsigned np);

/* ---- one whole step in the reference's order (dem_simulation.cpp:447-469,
 *      contactManager.cpp:156-185) ---- */
typedef struct xdo_scene {
    xdo_params prm;
    unsigned np;
    double *pos, *vel, *acc, *omega, *alpha, *force, *moment, *mass, *inertia;
    /* grid work arrays: n = np + ntri entries, ncell cells */
    unsigned *hash, *index, *sorted, *cstart, *cend;
    const xdo_contact_property* cp_pp;
    unsigned nplanes;
    const xdo_plane* planes;             /* in contact-name order */
    const xdo_contact_property* cp_planes; /* one per plane */
    unsigned ntri;
    xdo_polygon* poly;
    double* sphere;
    xdo_polygon_mass* pmi;
    const xdo_contact_property* cp_poly; /* one per polygon object */
    xdo_history* hist;                   /* NULL: the reference's DHS, no history */
    /* kinematic bodies (an extension): when set, each step first moves every
     * polygon body by its own vel and omega over dt (xdo_advance_bodies) and
     * the triangles with it (xdo_update_polygon_object_data) */
    int kinematic;
    unsigned nbodies;
    const double* vlist;                 /* body-frame vertices [ntri][9] */
    xdo_emitter* emit;                   /* NULL: every particle takes part */
} xdo_scene;

/* One step of prescribed body motion: origin += dt vel; the Euler parameters
 * (e0 scalar) turned by the rotation of angle |omega| dt about omega,
 * p <- q (x) p with q = (cos(|omega| dt / 2), sin(|omega| dt / 2) omega / |omega|),
 * then normalised.  An extension: the reference moves bodies through its
 * multibody solver on the host. */
void xdo_advance_bodies(xdo_polygon_mass* pmi, unsigned nbodies, double dt);

void xdo_step(xdo_scene* s);
void xdo_run_steps(xdo_scene* s, unsigned nsteps);

/* ---- the reference CPU path (timed baseline) ---- */
void xdo_cpu_step(xdo_scene* s);
void xdo_cpu_run_steps(xdo_scene* s, unsigned nsteps);

#ifdef __cplusplus
}
#endif

#endif
