/*
 * xdem.h -- C ABI of libxdem, the GB300 (sm_103a) DEM contact-step library.
 *
 * libxdem replaces the CUDA library of the xdynamics reference (the launchers
 * in source/mphysics_cuda_def.cu declared by include/mphysics_cuda_dec.cuh).
 * Every entry point below names the reference function it replaces.  The
 * arguments keep the reference's meaning and order; three things are added:
 *   - an explicit CUDA stream (`stream`, a cudaStream_t; 0 = legacy default
 *     stream, which is what the reference uses);
 *   - an int status return (XD_OK or an XD_ERR_* code) instead of `void` +
 *     exit() (the reference's checkCudaErrors), with the first failure also
 *     kept for xd_last_error();
 *   - plain C types only: device pointers, sizes and the POD structs below,
 *     whose byte layouts equal the reference's device structs.
 *
 * All pointer arguments of the compute calls are DEVICE pointers owned by the
 * caller, in the reference's layouts: pos and triangle spheres are double4
 * (x, y, z, r) rows; vel, acc, omega, alpha, force and moment are packed
 * double3 rows (24-byte stride); mass and inertia are double.
 *
 * Calls on the same stream are ordered like the reference's default-stream
 * launches.  The stateless calls share one library workspace (for the radix
 * sort) and the parameter block set by xd_set_symbolic_parameter; like the
 * reference they are meant for one host thread and one stream at a time.
 * Independent scenes run concurrently through xd_scene_* handles, which own
 * their parameters and workspace.
 */
#ifndef XDEM_H
#define XDEM_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XDEM_VERSION "0.1.0"

#ifdef __cplusplus
#define XD_ALIGN16 alignas(16)
#else
#define XD_ALIGN16 _Alignas(16)
#endif

/* status codes */
enum {
    XD_OK = 0,
    XD_ERR_INVALID = 1,      /* bad argument (null pointer, size, layout) */
    XD_ERR_CUDA = 2,         /* a CUDA runtime call or launch failed */
    XD_ERR_NOMEM = 3,        /* device allocation failed */
    XD_ERR_CAPACITY = 4,     /* a fixed-capacity buffer would overflow */
    XD_ERR_TIMEOUT = 5,      /* a bounded device-side wait ran out */
    XD_ERR_STATE = 6         /* call out of order (e.g. no parameters set) */
};

/* device_parameters (mphysics_cuda_dec.cuh:17-30), 112 bytes */
typedef struct xd_device_parameters {
    bool rollingCondition;
    unsigned int np;
    unsigned int nsphere;
    unsigned int ncell;
    unsigned int grid_size[3];
    double dt;
    double half2dt;
    double cell_size;
    double cohesion;
    double gravity[3];
    double world_origin[3];
} xd_device_parameters;

/* device_contact_property (mphysics_cuda_dec.cuh:78-88), 88 bytes */
typedef struct xd_contact_property {
    double Ei, Ej, pri, prj, Gi, Gj, rest, fric, rfric, coh, sratio;
} xd_contact_property;

/* device_plane_info (mphysics_cuda_dec.cuh:43-55), 232 bytes */
typedef struct xd_plane_info {
    double l1, l2;
    double u1[3], u2[3], uw[3], xw[3], pa[3], pb[3], w2[3], w3[3], w4[3];
} xd_plane_info;

/* device_cylinder_info (mphysics_cuda_dec.cuh:67-76), 176 bytes (ep at
 * offset 144: the reference's double4 is 16-byte aligned) */
typedef struct xd_cylinder_info {
    double len, rbase, rtop;
    double pbase[3], ptop[3], origin[3], vel[3], omega[3];
    double ep[4];
} xd_cylinder_info;

/* device_polygon_info (mphysics_cuda_dec.cuh:32-41), 152 bytes */
typedef struct xd_polygon_info {
    int id;
    double P[3], Q[3], R[3], V[3], W[3], N[3];
} xd_polygon_info;

/* device_polygon_mass_info (mphysics_cuda_dec.cuh:57-65), 160 bytes; ep is a
 * CUDA double4 and therefore 16-byte aligned. */
typedef struct xd_polygon_mass_info {
    double origin[3];
    XD_ALIGN16 double ep[4];
    double vel[3], omega[3], force[3], moment[3];
} xd_polygon_mass_info;

/* Single-precision twins of the structs (mphysics_cuda_dec.cuh:165-246). */
typedef struct xd_device_parameters_f {   /* device_parameters_f, 64 bytes */
    unsigned int np;
    unsigned int nsphere;
    unsigned int ncell;
    unsigned int grid_size[3];
    float dt;
    float half2dt;
    float cell_size;
    float cohesion;
    float gravity[3];
    float world_origin[3];
} xd_device_parameters_f;

typedef struct xd_contact_property_f {    /* device_contact_property_f, 44 bytes */
    float Ei, Ej, pri, prj, Gi, Gj, rest, fric, rfric, coh, sratio;
} xd_contact_property_f;

typedef struct xd_plane_info_f {          /* device_plane_info_f, 116 bytes */
    float l1, l2;
    float u1[3], u2[3], uw[3], xw[3], pa[3], pb[3], w2[3], w3[3], w4[3];
} xd_plane_info_f;

typedef struct xd_polygon_info_f {        /* device_polygon_info_f, 76 bytes */
    int id;
    float P[3], Q[3], R[3], V[3], W[3], N[3];
} xd_polygon_info_f;

typedef struct xd_polygon_mass_info_f {   /* device_polygon_mass_info_f, 80 bytes; ep a float4 */
    float origin[3];
    XD_ALIGN16 float ep[4];
    float vel[3], omega[3], force[3], moment[3];
} xd_polygon_mass_info_f;

/* ------------------------------------------------------------ library */

const char* xd_version(void);
const char* xd_status_string(int status);
/* First failure since the last xd_clear_error(), with a message. */
int xd_last_error(char* msg, size_t msg_len);
void xd_clear_error(void);
/* sizeof of each ABI struct, for binding-side layout checks. */
size_t xd_sizeof(const char* struct_name);
/* Record XD_ERR_INVALID ("<what>: not provided") for a declared entry point
 * that this build does not implement (used by the reference-API shim);
 * returns XD_ERR_INVALID. */
int xd_report_unsupported(const char* what);
/* Free the shared workspace of the stateless calls. */
int xd_release_workspace(void);

/* setSymbolicParameter (mphysics_cuda_dec.cuh:110; mphysics_cuda_def.cu:13-16).
 * Copies the host struct; later calls read it at launch time. */
int xd_set_symbolic_parameter(const xd_device_parameters* h_params);

/* ------------------------------------------------------------ integrator */

/* vv_update_position (mphysics_cuda_dec.cuh:112; def.cu:33-41;
 * kernel mphysics_cuda_impl.cuh:85-96): pos.xyz += dt*vel + half2dt*acc. */
int xd_vv_update_position(double* pos, const double* vel, const double* acc, unsigned np,
                          void* stream);

/* vv_update_velocity (mphysics_cuda_dec.cuh:113; def.cu:43-56;
 * kernel impl:98-134): a' = F/m, alpha' = M/I, v += dt/2 (a + a'),
 * w += dt/2 (alpha + alpha'); then force = m*gravity, moment = 0. */
int xd_vv_update_velocity(double* vel, double* acc, double* omega, double* alpha, double* force,
                          double* moment, const double* mass, const double* inertia, unsigned np,
                          void* stream);

/* Fused step boundary: vv_update_velocity of step t followed by
 * vv_update_position of step t+1 in one pass (same arithmetic, one read of
 * the state instead of two).  No reference counterpart as a single call; it
 * equals the reference's consecutive vv_update_velocity / vv_update_position
 * (dem_simulation.cpp:467 then :454 of the next step). */
int xd_vv_update_velocity_position(double* pos, double* vel, double* acc, double* omega,
                                   double* alpha, double* force, double* moment,
                                   const double* mass, const double* inertia, unsigned np,
                                   void* stream);

/* ------------------------------------------------------------ cell grid */

/* cu_calculateHashAndIndex (mphysics_cuda_dec.cuh:115; def.cu:58-66;
 * kernel impl:137-151). */
int xd_calculate_hash_and_index(unsigned* hash, unsigned* index, const double* pos, unsigned np,
                                void* stream);

/* cu_calculateHashAndIndexForPolygonSphere (mphysics_cuda_dec.cuh:116-118;
 * def.cu:68-77; kernel impl:153-164): entries sid .. sid+nsphere-1. */
int xd_calculate_hash_and_index_polysphere(unsigned* hash, unsigned* index, unsigned sid,
                                           unsigned nsphere, const double* sphere,
                                           void* stream);

/* cu_reorderDataAndFindCellStart (mphysics_cuda_dec.cuh:119; def.cu:80-108;
 * kernel impl:166-212): stable sort of (hash, index) by hash in place,
 * cstart = 0xffffffff / cend = 0 for every cell without entries, cstart/cend
 * = [first, one past last) sorted position of each occupied cell, and
 * sorted_index = index after the sort.  n = np + nsphere entries. */
int xd_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart,
                                   unsigned* cend, unsigned* sorted_index, unsigned n,
                                   unsigned ncell, void* stream);

/* Allocation-free variant of xd_reorder_and_find_cell_start; no counterpart
 * in the reference.  For callers that may not allocate device memory while
 * they run (an application that hands out all device memory from its own
 * pool at start-up, or a process held to a fixed memory budget): the sort
 * scratch comes from a fixed device array inside the library instead of
 * cudaMalloc, and the call allocates nothing.  Limits and rules:
 *   - at most XD_NOALLOC_MAX_ENTRIES entries (n); larger n -> XD_ERR_CAPACITY;
 *   - the array (about 9.4 MB) stays on every device that uses it until the
 *     process exits.  Under lazy module loading (the CUDA default) the driver
 *     reserves it at the first call on a device, so a caller whose own pool
 *     takes the device's memory makes one call first (n = 0 only clears the
 *     cell arrays and serves as that set-up) or sets
 *     CUDA_MODULE_LOADING=EAGER; later calls reserve nothing;
 *   - all calls share the array: calls that overlap on the GPU (other
 *     streams or host threads) race, so serialise them;
 *   - every call looks up the array's device address on the current device;
 *     make a device's first call before any stream capture on that device.
 * Same arguments, results and status codes as xd_reorder_and_find_cell_start. */
#define XD_NOALLOC_MAX_ENTRIES (1u << 20)
int xd_reorder_and_find_cell_start_noalloc(unsigned* hash, unsigned* index, unsigned* cstart,
                                           unsigned* cend, unsigned* sorted_index, unsigned n,
                                           unsigned ncell, void* stream);

/* Stable LSD radix sort of 32-bit (key, value) pairs by the low key_bits of
 * the key (the sort inside cu_reorderDataAndFindCellStart, def.cu:92-94,
 * where the reference calls thrust::sort_by_key).  In place. */
int xd_radix_sort_pairs(unsigned* keys, unsigned* values, unsigned n, unsigned key_bits,
                        void* stream);

/* ------------------------------------------------------------ contacts */

/* cu_calculate_p2p (mphysics_cuda_dec.cuh:121-126; def.cu:110-136;
 * kernel impl:403-485), tcm = 1 (the DHS model the application runs;
 * contact_particles_particles.cpp:135).  cp is a device pointer. */
int xd_calculate_p2p(int tcm, const double* pos, const double* vel, const double* omega,
                     double* force, double* moment, const double* mass,
                     const unsigned* sorted_index, const unsigned* cstart, const unsigned* cend,
                     const xd_contact_property* cp, unsigned np, void* stream);

/* cu_plane_contact_force (mphysics_cuda_dec.cuh:129-133; def.cu:138-156;
 * kernel impl:572-621).  plane and cp are device pointers. */
int xd_plane_contact_force(int tcm, const xd_plane_info* plane, const double* pos,
                           const double* vel, const double* omega, double* force, double* moment,
                           const double* mass, unsigned np, const xd_contact_property* cp,
                           void* stream);

/* cu_cylinder_hertzian_contact_force (mphysics_cuda_dec.cuh:149-155;
 * def.cu:181-200; cylinder_hertzian_contact_force_kernel, impl:652-760): one
 * cylinder (device pointer) against every particle, DHS with Meq = m and
 * Req = r, the contact depth rounded to FP32 as the reference's detection
 * returns it.  Adds to force/moment; writes each particle's reaction on the
 * cylinder to mf[i] = -Fn and mm[i] = (cp - mpos) x -Fn (mpos: one double[3]
 * on the device).  The reference also zeroes mf[0] and mm[0] from every
 * thread, racing with particle 0's store; here slot 0 holds particle 0's
 * reaction.  Its _mf/_mm outputs are never written by the reference and have
 * no counterpart here. */
int xd_cylinder_contact_force(int tcm, const xd_cylinder_info* cyl, const double* pos,
                              const double* vel, const double* omega, double* force, double* moment,
                              const double* mass, unsigned np, const xd_contact_property* cp,
                              const double* mpos, double* mf, double* mm, void* stream);

/* cu_cube_contact_force (mphysics_cuda_dec.cuh:135-139; def.cu:158-179):
 * the six planes of a cube (device array of 6), applied in order. */
int xd_cube_contact_force(int tcm, const xd_plane_info* planes6, const double* pos,
                          const double* vel, const double* omega, double* force, double* moment,
                          const double* mass, unsigned np, const xd_contact_property* cp,
                          void* stream);

/* Several planes in one pass, applied in array order with the same
 * per-plane accumulation as nplanes consecutive cu_plane_contact_force calls
 * (contactManager.cpp:167-174 iterates plane contacts in name order).
 * planes and cps are device arrays of nplanes entries. */
int xd_planes_contact_force(int tcm, const xd_plane_info* planes, const xd_contact_property* cps,
                            unsigned nplanes, const double* pos, const double* vel,
                            const double* omega, double* force, double* moment,
                            const double* mass, unsigned np, void* stream);

/* cu_particle_polygonObject_collision (mphysics_cuda_dec.cuh:142-147;
 * def.cu:203-221; kernel impl:923-1021).  Grid entries k >= np are
 * triangles k - np.  The reaction on each polygon body is added to
 * dpmi[body].force / .moment by a deterministic reduction (the reference
 * adds it with unsynchronised +=, impl:1010-1011). */
int xd_particle_polygon_collision(int tcm, const xd_polygon_info* dpi, const double* dsph,
                                  xd_polygon_mass_info* dpmi, const double* pos,
                                  const double* vel, const double* omega, double* force,
                                  double* moment, const double* mass, const unsigned* sidx,
                                  const unsigned* cstart, const unsigned* cend,
                                  const xd_contact_property* cp, unsigned np, unsigned nbodies,
                                  void* stream);

/* cu_updatePolygonObjectData (mphysics_cuda_dec.cuh:296-298; def.cu:469-475;
 * kernel impl:1911-1956): move body-frame triangle vertices vList (9 doubles
 * per triangle) by the body's origin and Euler parameters, write P, Q, R and
 * the circumcentre into sphere.xyz. */
int xd_update_polygon_object_data(const xd_polygon_mass_info* dpmi, const double* vList,
                                  double* sphere, xd_polygon_info* dpi, unsigned ntriangle,
                                  void* stream);

/* reductionD3 (mphysics_cuda_dec.cuh:157; def.cu:223-242): sum of n double3
 * rows, returned to the host in out[3] (deterministic order). */
int xd_reduction_d3(const double* in, unsigned n, double out[3], void* stream);

/* Contact pair list: for every particle i (ascending) the partners k with
 * (r_i + r_k) - |x_k - x_i| > 0 found by the 27-cell search, in search order,
 * written as (i, k) pairs.  counts[np] receives the per-particle counts;
 * pairs must hold `cap` pairs.  *total gets the total pair count (may exceed
 * cap, in which case XD_ERR_CAPACITY is returned).  Diagnostic call. */
int xd_pair_list(const double* pos, const unsigned* sorted_index, const unsigned* cstart,
                 const unsigned* cend, unsigned np, unsigned* counts, unsigned* pairs,
                 unsigned long long cap, unsigned long long* total, void* stream);

/* ------------------------------------------------------------ single precision
 *
 * The FP32 twins of the live API (mphysics_cuda_dec.cuh:248-300, launchers
 * mphysics_cuda_def.cu:254-466, kernels mphysics_cuda_impl.cuh:1094-1895):
 * pos and triangle spheres are float4 rows (16-byte aligned), vel, acc,
 * omega, alpha, force and moment packed float3 rows (12-byte stride), mass
 * and inertia float.  The arithmetic follows the reference's float kernels
 * expression by expression, with their mixed float/double constants.
 * Reference behaviour kept on purpose:
 *   - the cell hash wraps with the grid size of the FP64 parameter block
 *     (calcGridHash, impl:65-72, reads cte.grid_size, which only
 *     setSymbolicParameter sets): set it with xd_set_symbolic_parameter too,
 *     or, as when the reference runs in single precision without it, the
 *     grid size is 0 and the hash is the x cell index alone;
 *   - particle-particle forces always include the rotation terms (the float
 *     parameter block has no rolling switch);
 *   - a triangle contact adds only its normal force to the particle and no
 *     moment, while the body takes -(Fn + Ft) (impl:1880-1888);
 *   - planes apply no moment (DHSModel with ir = 0, impl:1553-1561).
 * The body reaction, summed racily by the reference kernel, is summed here in
 * a fixed order.  Only tcm = 1 (DHS) is provided, as for FP64. */

/* setSymbolicParameter_f (mphysics_cuda_dec.cuh:248; def.cu:255-258). */
int xd_set_symbolic_parameter_f(const xd_device_parameters_f* h_params);

/* vv_update_position(float*) (dec.cuh:250; def.cu:260-267; impl:1105-1116). */
int xd_vv_update_position_f(float* pos, const float* vel, const float* acc, unsigned np, void* stream);

/* vv_update_velocity(float*) (dec.cuh:251; def.cu:269-282; impl:1118-1153). */
int xd_vv_update_velocity_f(float* vel, float* acc, float* omega, float* alpha, float* force,
                            float* moment, const float* mass, const float* inertia, unsigned np,
                            void* stream);

/* cu_calculateHashAndIndex(float*) (dec.cuh:253; def.cu:284-292; impl:1156-1168). */
int xd_calculate_hash_and_index_f(unsigned* hash, unsigned* index, const float* pos, unsigned np,
                                  void* stream);

/* cu_calculateHashAndIndexForPolygonSphere(float*) (dec.cuh:254; def.cu:294-302;
 * impl:1170-1182). */
int xd_calculate_hash_and_index_polysphere_f(unsigned* hash, unsigned* index, unsigned sid,
                                             unsigned nsphere, const float* sphere, void* stream);

/* cu_reorderDataAndFindCellStart_f (dec.cuh:255-258; def.cu:305-333;
 * impl:1184-1227): the same integer work as the FP64 call. */
int xd_reorder_and_find_cell_start_f(unsigned* hash, unsigned* index, unsigned* cstart,
                                     unsigned* cend, unsigned* sorted_index, unsigned n,
                                     unsigned ncell, void* stream);

/* cu_calculate_p2p(float*) (dec.cuh:260-266; def.cu:335-361; impl:1345-1425). */
int xd_calculate_p2p_f(int tcm, const float* pos, const float* vel, const float* omega,
                       float* force, float* moment, const float* mass,
                       const unsigned* sorted_index, const unsigned* cstart, const unsigned* cend,
                       const xd_contact_property_f* cp, unsigned np, void* stream);

/* cu_plane_contact_force(float*) (dec.cuh:268-272; def.cu:363-381; impl:1427-1564). */
int xd_plane_contact_force_f(int tcm, const xd_plane_info_f* plane, const float* pos,
                             const float* vel, const float* omega, float* force, float* moment,
                             const float* mass, unsigned np, const xd_contact_property_f* cp,
                             void* stream);

/* cu_cube_contact_force(float*) (dec.cuh:274-279; def.cu:383-404): the six
 * planes in order, one shared property. */
int xd_cube_contact_force_f(int tcm, const xd_plane_info_f* planes6, const float* pos,
                            const float* vel, const float* omega, float* force, float* moment,
                            const float* mass, unsigned np, const xd_contact_property_f* cp,
                            void* stream);

/* cu_particle_polygonObject_collision(float*) (dec.cuh:281-286; def.cu:428-446;
 * impl:1808-1895).  Entries of sidx >= np are triangles (index - np); the
 * reaction -(Fn + Ft) and its moment are added to dpmi[body]: for nbodies
 * bodies (at most 8) in a fixed order, or with atomics when nbodies = 0. */
int xd_particle_polygon_collision_f(int tcm, const xd_polygon_info_f* dpi, const float* dsph,
                                    xd_polygon_mass_info_f* dpmi, const float* pos,
                                    const float* vel, const float* omega, float* force,
                                    float* moment, const float* mass, const unsigned* sidx,
                                    const unsigned* cstart, const unsigned* cend,
                                    const xd_contact_property_f* cp, unsigned np,
                                    unsigned nbodies, void* stream);

/* reductionD3(float3*) (dec.cuh:300; def.cu:448-466): sum of n float3 rows,
 * returned to the host in out[3] (deterministic order). */
int xd_reduction_f3(const float* in, unsigned n, float out[3], void* stream);

/* ------------------------------------------------------------ scenes
 *
 * A scene owns one DEM system on the device: its state arrays, grid work
 * arrays, walls, triangle mesh and workspace, and advances whole steps in the
 * reference's order (dem_simulation::oneStepAnalysis,
 * dem_simulation.cpp:447-469; contactManager::deviceCollision,
 * contactManager.cpp:156-185):
 *   VV position -> hash (+ triangle spheres) -> sort / cell ranges ->
 *   particle-particle -> planes in array order -> triangles -> VV velocity.
 * Scenes hold no global state, so independent scenes may run on different
 * streams at the same time.
 */
typedef struct xd_scene xd_scene;

enum {
    XD_MODE_FP64 = 0,  /* the reference's FP64 arithmetic and loop order */
    XD_MODE_MIXED = 1  /* FP64 state and integration, exact integer contact
                          decisions, FP32 contact forces; the scene's own grid
                          (cell 2 r_max, sized to the initial bounding box) */
};

typedef struct xd_scene_desc {
    xd_device_parameters params;             /* grid, dt, gravity, rolling; params.np = np */
    unsigned np;                             /* particles */
    int mode;                                /* XD_MODE_* */
    xd_contact_property cp_pp;               /* particle-particle property */
    unsigned nplanes;
    const xd_plane_info* planes;             /* host array, contact-name order */
    const xd_contact_property* cp_planes;    /* host array, one per plane */
    unsigned ntri;                           /* triangles of all polygon bodies */
    unsigned nbodies;                        /* polygon bodies */
    const xd_polygon_info* poly;             /* host array [ntri] */
    const double* sphere;                    /* host array [ntri][4] */
    const double* vlist;                     /* host array [ntri][9] body-frame vertices */
    const xd_polygon_mass_info* pmi;         /* host array [nbodies] */
    const xd_contact_property* cp_poly;      /* host array [nbodies] */
} xd_scene_desc;

/* Allocates the scene's device memory.  No reference counterpart: the
 * reference allocates these arrays in dem_simulation::allocationMemory
 * (dem_simulation.cpp:174-199) and contact::cudaMemoryAlloc (contact.cpp:107-116). */
int xd_scene_create(const xd_scene_desc* desc, xd_scene** out);
int xd_scene_destroy(xd_scene* scene);

/* Host <-> device state copies (reference layouts; any argument may be NULL
 * to skip that array).  Synchronous with respect to `stream`. */
int xd_scene_upload(xd_scene* scene, const double* pos, const double* vel, const double* acc,
                    const double* omega, const double* alpha, const double* force,
                    const double* moment, const double* mass, const double* inertia,
                    void* stream);
int xd_scene_download(xd_scene* scene, double* pos, double* vel, double* acc, double* omega,
                      double* alpha, double* force, double* moment, void* stream);
/* The same copies queued on `stream` without waiting for them: the host
 * arrays must stay untouched (upload) or unread (download) until the stream
 * has passed this point; with pinned host memory the copies overlap the
 * host's next calls.  A scene's first upload sets its grid up and waits. */
int xd_scene_upload_async(xd_scene* scene, const double* pos, const double* vel, const double* acc,
                          const double* omega, const double* alpha, const double* force,
                          const double* moment, const double* mass, const double* inertia,
                          void* stream);
int xd_scene_download_async(xd_scene* scene, double* pos, double* vel, double* acc, double* omega,
                            double* alpha, double* force, double* moment, void* stream);

/* Device pointers of the scene's state, in the reference layouts (for
 * zero-copy access); any output may be NULL. */
int xd_scene_device_state(xd_scene* scene, double** pos, double** vel, double** acc,
                          double** omega, double** alpha, double** force, double** moment,
                          double** mass, double** inertia);
/* Device pointers of the grid arrays after the last step's sort. */
int xd_scene_device_grid(xd_scene* scene, unsigned** hash, unsigned** index, unsigned** sorted,
                         unsigned** cstart, unsigned** cend);

/* Host copies of the grid arrays after the last step's sort (any may be NULL):
 * hash/index/sorted hold np + ntri entries, cstart/cend ncell. */
int xd_scene_download_grid(xd_scene* scene, unsigned* hash, unsigned* index, unsigned* sorted,
                           unsigned* cstart, unsigned* cend, void* stream);

/* Replace the polygon bodies' motion (origin, Euler parameters, velocity,
 * angular velocity) from a host array [nbodies]; the triangles are moved by
 * cu_updatePolygonObjectData semantics before the next step's hashing.
 * Reaction force/moment fields of the uploaded records are kept. */
int xd_scene_set_bodies(xd_scene* scene, const xd_polygon_mass_info* pmi, void* stream);
int xd_scene_get_bodies(xd_scene* scene, xd_polygon_mass_info* pmi, void* stream);
/* Replace the planes (same count and order as the description) from a host
 * array, as contact_particles_plane::cuda_collision re-uploads a moving
 * plane's device_plane_info (collision/contact_particles_plane.cpp:33-51).
 * The plane contact has no wall velocity, as in the reference.  The mixed
 * form re-bins before its next step (the planes in reach change). */
int xd_scene_set_planes(xd_scene* scene, const xd_plane_info* planes, void* stream);

/* Advance nsteps whole steps on `stream`.  Returns after enqueueing; a
 * device-side error word is checked (with a synchronisation) only when
 * `check` is non-zero.  Both forms replay the steps as CUDA graphs captured
 * at the scene's first call (the FP64 form for calls of four steps or more);
 * XDEM_NO_GRAPHS=1 in the environment launches the same kernels directly. */
int xd_scene_step(xd_scene* scene, unsigned nsteps, int check, void* stream);

/* Per-phase timing with CUDA events recorded on the step's stream.  Phases:
 * 0 VV update, 1 hash, 2 sort + cell ranges, 3 particle-particle,
 * 4 planes, 5 triangles, 6 reorder (mixed mode).  xd_scene_phase_times
 * synchronises the events and returns the summed milliseconds and launch
 * counts since timing was last enabled. */
#define XD_SCENE_PHASES 7
int xd_scene_set_timing(xd_scene* scene, int enable);
int xd_scene_phase_times(xd_scene* scene, double* ms, unsigned long long* launches);

/* Contact forces and moments (without gravity) of the current state, in the
 * original particle order, written to host arrays [np][3]: the
 * particle-particle and wall terms that the next step would add.  Diagnostic
 * call (synchronous); the state is not advanced. */
int xd_scene_eval_contacts(xd_scene* scene, double* force, double* moment, void* stream);

/* Contact partners of the current state (mixed mode): for every particle i
 * (original order) counts[i] partners written to partners[i * cap + k] as
 * original indices, in search order.  Diagnostic call (synchronous). */
int xd_scene_pair_list(xd_scene* scene, unsigned cap, unsigned* counts, unsigned* partners,
                       void* stream);

/* Mixed-mode counters: [0] particles the contact pass visits (those with a
 * Verlet neighbour or a plane within reach at the last list build),
 * [1] pairs decided by the FP64 guard-band test (cumulative), [2] normal
 * forces formed in FP64 because the elastic and damping terms nearly cancel
 * (cumulative), [3] slips formed in FP64 because the rotation term cancels
 * most of the tangential velocity (cumulative). */
int xd_scene_counters(xd_scene* scene, unsigned long long out[4], void* stream);

/* Mixed-mode diagnostics (no counterpart in the reference), the first
 * `count` of: [0..3] as xd_scene_counters; [4] wall contacts (planes and
 * triangles) decided by the FP64 region test instead of the FP64 plane
 * distance of a clear face contact (cumulative); [5] re-binnings
 * (cumulative); [6] listed particles with triangles in reach; [7] Verlet
 * lists and [8] triangle lists over their capacity at the last build (those
 * particles' contacts are searched in the cells); [9] Verlet-list and [10]
 * triangle-list entries at the last build.  Zeros for an FP64 scene. */
#define XD_STATS_COUNT 11
int xd_scene_stats(xd_scene* scene, unsigned long long* out, unsigned count, void* stream);

/* Mixed-mode tuning (no counterpart in the reference, whose grid and launch
 * shapes are fixed: dem_simulation.cpp:259-261): the skin width over the
 * largest radius (cells are 2 r_max + skin wide; a larger skin re-bins less
 * often but lists more neighbours), the Verlet-list and triangle-list
 * capacities per particle (a fuller list makes that particle's contact pass
 * search its cells instead), and the contact pass's block size.  Set before
 * the scene's first upload (XD_ERR_STATE after); a batch launches its
 * contact pass with its first scene's block size and pair pass.  Defaults:
 * 0.1, 48, 16, 64, 1.
 * metakonga_gb300.tune chooses them per scene shape. */
typedef struct xd_tuning {
    float skin_factor;          /* [0.02, 1] */
    unsigned verlet_cap;        /* [8, 256] */
    unsigned triangle_cap;      /* [4, 128] */
    unsigned contact_threads;   /* 32, 64 or 128 */
    unsigned contact_mode;      /* pair pass: 0 a thread per listed particle, 1 warp-cooperative (the
                                   warp's contacts spread one per lane, summed per particle in list
                                   order: the same bits as 0) */
} xd_tuning;
int xd_scene_set_tuning(xd_scene* scene, const xd_tuning* tuning);
int xd_scene_get_tuning(xd_scene* scene, xd_tuning* tuning);

/* Number of kernel launches one xd_scene_step of nsteps issues, not counting
 * the cell re-binnings the mixed mode decides on the device (see
 * xd_scene_rebuilds); the FP64 mode's count is exact. */
unsigned long long xd_scene_launches(xd_scene* scene, unsigned nsteps);

/* Mixed mode: cell re-binnings so far (*count, cumulative) and the kernel
 * launches each one issues (*launches_each).  A mixed scene keeps every
 * particle in its assigned cell while it stays within half a skin of it and
 * re-bins all cells in the step where one leaves; the FP64 mode re-bins every
 * step as the reference does and reports 0 here.  No counterpart in the
 * reference. */
int xd_scene_rebuilds(xd_scene* scene, unsigned long long* count, unsigned long long* launches_each,
                      void* stream);

/* Kinematic polygon bodies, an extension (the reference moves its bodies
 * through its multibody solver on the host, one D2H/H2D round trip per
 * step): with enable != 0, every step first moves each body by its own vel
 * and omega (as set by xd_scene_set_bodies) over dt -- origin += dt vel, the
 * Euler parameters p <- q (x) p with q the rotation of angle |omega| dt about
 * omega, normalised -- and the triangles with it
 * (cu_updatePolygonObjectData semantics), all on the device.  The mixed form
 * re-bins when a vertex has moved half the skin. */
int xd_scene_set_kinematic_bodies(xd_scene* scene, int enable);

/* Particle emitter: the reference's real-time particle creation
 * (dem_simulation.cpp:210-222 and :321-322 set it up with no particle yet,
 * :449-450 adds a group before a step; particleManager.cpp:132-145 hands out
 * the groups made by its plane and circle creators, or one particle at a
 * time).  The scene's particles are all uploaded (staged at their creation
 * positions); only the first `active` take part in a step -- the cell grid,
 * every contact, velocity-Verlet, and the triangle offset in the grid.  Before
 * the k-th step after this call (k from 1), when period > 0,
 * (k - 1) % period == 0 and particles remain, the next of the `ngroups` group
 * sizes joins (one particle when ngroups is 0), up to the particle count.  An
 * emitted particle starts from its uploaded state.  period = 0 with active =
 * np turns the emitter off.  Deliberate difference: the reference keeps the
 * parameter block's np at the total, so until every particle is out its
 * polygon kernel reads the triangles' grid entries (active + t) as particles
 * or as the wrong triangle; here the triangles take part from the first step.
 * Downloads return every particle, the staged ones unchanged;
 * xd_scene_eval_contacts gives them zero rows. */
int xd_scene_set_emitter(xd_scene* scene, unsigned active, unsigned period, const unsigned* groups,
                         unsigned ngroups, void* stream);
/* The particles that take part in the next step (before its emission). */
int xd_scene_active(xd_scene* scene, unsigned* active);

/* FP64 form: a grid of its own for the particles (power-of-two dimensions,
 * cell size, origin), while the triangles stay on the scene's grid.  The
 * reference hashes particles and triangle circumspheres into one grid whose
 * cell must hold the largest circumsphere (dem_simulation.cpp:259-261), so a
 * mesh of large triangles makes every particle search cells many times its
 * size; with this call the particle pairs are searched in cells of the
 * particles' own size (at least the largest diameter: the caller's choice,
 * as the reference's cell size is) and the triangles as before.  The pair
 * sums then run in another order: results equal the reference's within the
 * FP64 rounding of a reordered sum.  No counterpart in the reference. */
int xd_scene_set_particle_grid(xd_scene* scene, const unsigned grid[3], double cell_size, const double origin[3]);

/* Tangential-spring history, an extension: the reference's DHSModel
 * (mphysics_cuda_impl.cuh:379-401) keeps no state between steps.  With
 * slots > 0 (at most 32) every particle keeps up to `slots` contacts keyed
 * by partner (particle j -> j, plane w -> 0x80000000 | w, triangle t ->
 * 0xC0000000 | t) with an FP64 tangential spring d.  Per contact and step,
 * with u the contact normal and vt the tangential relative velocity:
 *   d <- d - (d.u)u, rescaled to |d|;  d <- d + vt dt;  Ft = ks d + vs vt;
 *   if |Ft| > mu |Fn|:  Ft <- mu |Fn| Ft / |Ft|,  d <- (Ft - vs vt) / ks;
 *   the moment is (ir u) x Ft with ir = 0 for walls, as in the reference.
 * A new contact starts from d = 0, so its first step has the reference's DHS
 * force; a contact that ends frees its entry; a contact that finds no free
 * entry is counted as overflow and computed without history.  The normal
 * force is the reference's.  slots = 0 restores the reference model.  The
 * call empties the tables. */
int xd_scene_set_tangential_history(xd_scene* scene, unsigned slots);

/* The history tables in original particle order: keys[s * np + i] (0xffffffff
 * empty) and delta[(s * np + i) * 3 + a], and the overflow count.  Any
 * pointer may be NULL.  Synchronous. */
int xd_scene_download_history(xd_scene* scene, unsigned* keys, double* delta,
                              unsigned long long* overflow, void* stream);

/* Advance `count` independent scenes (scenes[i] by nsteps[i] steps) side by
 * side on the current device: the scenes are spread over a pool of 32
 * library streams that start after the work queued on `stream` and that
 * `stream` waits for on return, so the batch is ordered on `stream` like one
 * xd_scene_step.  The streams overlap on the device up to the
 * CUDA_DEVICE_MAX_CONNECTIONS hardware queues (set it to 32 before the CUDA
 * context is created).  Each scene's result is bit for bit the one xd_scene_step
 * gives it alone.  Two scenes of one call must not be the same scene.  With
 * `check` non-zero the call synchronises `stream`.  No counterpart in the
 * reference, which runs one model per process. */
int xd_scene_step_many(xd_scene* const* scenes, const unsigned* nsteps, unsigned count, int check,
                       void* stream);

/* Device memory the scene holds, in bytes (state, grid, lists, meshes,
 * workspace).  No counterpart in the reference. */
int xd_scene_device_bytes(xd_scene* scene, unsigned long long* bytes);

/* Batches (no counterpart in the reference): mixed-form scenes advanced
 * together, a step of all of them being one CUDA graph -- one advance launch
 * over every scene's particles, a re-binning per scene that needs one (a
 * conditional node per group of 32 scenes, then per scene), one contact
 * launch over every scene's listed particles.  Each scene's result is the
 * same, bit for bit, as when it is stepped alone; what a batch saves is the
 * launch and graph-node cost per scene, which bounds many small scenes.  The
 * scenes must be uploaded, in the mixed form, without tangential history,
 * kinematic bodies or an emitter; a batch re-captures itself when one of its
 * scenes changes (planes, bodies' kinematics, history), and must be
 * destroyed before its scenes. */
typedef struct xd_batch xd_batch;
int xd_batch_create(xd_scene* const* scenes, unsigned count, xd_batch** out);
/* nsteps whole steps of every scene of the batch, queued on `stream`. */
int xd_batch_step(xd_batch* batch, unsigned nsteps, int check, void* stream);
int xd_batch_destroy(xd_batch* batch);
/* Kernel timing of a batch: while enabled, xd_batch_step launches the step's
 * kernels directly (the same kernels; the re-binning flags are read on the
 * host) with CUDA events around the advance of every step but a call's first
 * and around every contact launch.  xd_batch_kernel_times returns their
 * summed milliseconds and launch counts, [0] advance, [1] pair pass (the
 * whole contact pass in contact_mode 0) and [2] wall pass, since timing was
 * enabled.  XDEM_NO_GRAPHS=1 in the environment also makes a batch
 * launch directly (profilers list no kernel inside a graph with conditional
 * nodes). */
int xd_batch_set_timing(xd_batch* batch, int enable);
int xd_batch_kernel_times(xd_batch* batch, double ms[3], unsigned long long launches[3]);

#ifdef __cplusplus
}
#endif

#endif
