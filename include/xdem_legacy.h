/*
 * xdem_legacy.h -- C ABI of the legacy DEM interface of the xdynamics
 * reference (include/cu_dem_dec.cuh, launchers source/cu_dem_def.cu, kernels
 * include/cu_dem_impl.cuh), the one the parSIM classes (dem_force,
 * cell_grid, Verlet_integrator, geometry) call.  Implemented by libxdem
 * (metakonga_gb300/csrc/xd_legacy.cu); the C++ names of cu_dem_dec.cuh are in
 * libxdem_legacy.so (metakonga_gb300/csrc/shim_legacy.cpp).
 *
 * The legacy interface differs from the live one (xdem.h): its parameter
 * block carries the contact constants (kn, vn, ks, vs, mu, cohesive); vel,
 * acc, omega and alpha are double4 rows with the mass in acc.w and the
 * inertia in alpha.w; force and moment are packed double3; every kernel runs
 * over the parameter block's np (the launchers' np only sizes the launch and,
 * for the hash call, the sort); the hash call sorts; triangle contact goes
 * through mesh vertices placed in the grid after the particles.
 *
 * Behaviour kept from the reference, as the drop-in requires:
 *   - a particle-particle contact adds only its normal force to the particle,
 *     the shear force only through the moment (calForce, impl:231-252);
 *   - with cohesive != 0, particles within the 27 cells but apart get the
 *     cohesion terms of impl:211-229;
 *   - vector / scalar is a multiplication by the reciprocal (impl:68-72);
 *   - xd_legacy_reorder_and_find_cell_start resets cstart only, not cend
 *     (def.cu:71-90);
 *   - the shape call zeroes force and moment, adds the first face contact of
 *     each particle, else its first edge or vertex contact, and returns the
 *     sum of the particle forces (def.cu:140-232).
 * All pointers are DEVICE pointers unless noted; every call takes a stream
 * and returns XD_OK or an XD_ERR_* code (xdem.h).
 */
#ifndef XDEM_LEGACY_H
#define XDEM_LEGACY_H

#include <stdbool.h>

#include "xdem.h"

#ifdef __cplusplus
extern "C" {
#endif

/* device_parameters (cu_dem_dec.cuh:41-60), 144 bytes */
typedef struct xd_legacy_parameters {
    unsigned int np;
    unsigned int nsp;
    unsigned int ncell;
    unsigned int grid_size[3];
    double dt;
    double half2dt;
    double cell_size;
    double gravity[3];
    double world_origin[3];
    double kn, vn, ks, vs, mu;
    double cohesive;
} xd_legacy_parameters;

/* device_plane_info (cu_dem_dec.cuh:62-71), 160 bytes */
typedef struct xd_legacy_plane_info {
    double l1, l2;
    double u1[3], u2[3], uw[3], xw[3], pa[3], pb[3];
} xd_legacy_plane_info;

/* cu_polygon (cu_dem_dec.cuh:73-81), 144 bytes */
typedef struct xd_legacy_polygon {
    double P[3], Q[3], R[3], V[3], W[3], N[3];
} xd_legacy_polygon;

/* cu_mass_info (cu_dem_dec.cuh:83-87), 48 bytes */
typedef struct xd_legacy_mass_info {
    double pos[3];
    double vel[3];
} xd_legacy_mass_info;

/* setSymbolicParameter (cu_dem_dec.cuh:95; def.cu:25-28) */
int xd_legacy_set_symbolic_parameter(const xd_legacy_parameters* h_params);

/* vv_update_position (cu_dem_dec.cuh:98; def.cu:30-37; impl:93-107):
 * pos.xyz += dt vel.xyz + half2dt acc.xyz. */
int xd_legacy_vv_update_position(double* pos, const double* vel, const double* acc, unsigned np,
                                 void* stream);

/* vv_update_velocity (cu_dem_dec.cuh:99; def.cu:39-49; impl:109-140): a = F / acc.w,
 * alpha = M / alpha.w, half-step velocity updates; force and moment are kept. */
int xd_legacy_vv_update_velocity(double* vel, double* acc, double* omega, double* alpha,
                                 const double* force, const double* moment, unsigned np,
                                 void* stream);

/* cu_calculateHashAndIndex (cu_dem_dec.cuh:102; def.cu:57-69; impl:142-154): hash
 * and index of the parameter block's np + nsp rows of pos, then a stable sort
 * of the first np (argument) entries by hash. */
int xd_legacy_calculate_hash_and_index(unsigned* hash, unsigned* index, const double* pos,
                                       unsigned np, void* stream);

/* cu_reorderDataAndFindCellStart (cu_dem_dec.cuh:103; def.cu:71-90; impl:156-196). */
int xd_legacy_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart,
                                          unsigned* cend, unsigned* sorted_index, unsigned np,
                                          unsigned nc, void* stream);

/* cu_calculate_p2p (cu_dem_dec.cuh:106; def.cu:92-107; impl:198-327): force +=
 * m g + the normal contact forces, moment += the shear moments. */
int xd_legacy_calculate_p2p(const double* pos, const double* vel, const double* acc,
                            const double* omega, const double* alpha, double* force,
                            double* moment, const unsigned* sorted_index, const unsigned* cstart,
                            const unsigned* cend, unsigned np, unsigned cRun, void* stream);

/* cu_cube_hertzian_contact_force (cu_dem_dec.cuh:109; def.cu:109-138; impl:329-378):
 * the face contacts of six planes; isLineContact is not used. */
int xd_legacy_cube_hertzian_contact_force(const xd_legacy_plane_info* planes, double kn, double vn,
                                          double ks, double vs, double mu, bool* isLineContact,
                                          const double* pos, const double* vel,
                                          const double* omega, double* force, double* moment,
                                          unsigned np, void* stream);

/* cu_shape_hertzian_contact_force (cu_dem_dec.cuh:110; def.cu:140-232; impl:380-762).
 * Grid entries >= np are mesh vertices; poly_start/poly_end[v] delimit the
 * polygons of vertex v in id_set; minfo holds the body's velocity.  The sum
 * of the particle forces is written to out[3] (host); bforce is not used. */
int xd_legacy_shape_hertzian_contact_force(const xd_legacy_mass_info* minfo,
                                           const xd_legacy_polygon* polygons,
                                           const unsigned* id_set, const unsigned* poly_start,
                                           const unsigned* poly_end, double kn, double vn,
                                           double ks, double vs, double mu, bool* isLineContact,
                                           const double* pos, const double* vel,
                                           const double* omega, double* force, double* moment,
                                           double* bforce, unsigned np,
                                           const unsigned* sorted_id, const unsigned* cell_start,
                                           const unsigned* cell_end, double out[3], void* stream);

/* cu_update_polygons_position (cu_dem_dec.cuh:111; def.cu:234-238; impl:764-780):
 * pos[v] = mpos + A local_vertice[v] (A row-major 3x3, mpos one double3). */
int xd_legacy_update_polygons_position(const double* mpos, const double* A,
                                       const double* local_vertice, unsigned nvertex, double* pos,
                                       void* stream);

/* cu_update_polygons_information (cu_dem_dec.cuh:112; def.cu:240-244; impl:798-817). */
int xd_legacy_update_polygons_information(xd_legacy_polygon* polygons, const unsigned* indice,
                                          const double* pos, unsigned ni, void* stream);

/* cu_mergedata (cu_dem_dec.cuh:113; def.cu:51-55; impl:782-796): data = the np
 * particles then the snp vertices as (x, y, z, -1). */
int xd_legacy_mergedata(double* data, const double* pos, unsigned np, const double* vertice,
                        unsigned snp, void* stream);

#ifdef __cplusplus
}
#endif

#endif
