/*
 * mphysics_cuda_dec.cuh -- drop-in declaration of the xdynamics DEM CUDA
 * library, implemented by libxdem_mphysics.so on top of libxdem (xdem.h).
 *
 * The declarations keep the names, C++ signatures, argument meaning and
 * struct layouts of the reference's include/mphysics_cuda_dec.cuh (cited per
 * item) so that the reference's host code (dem_simulation, neighborhood_cell,
 * velocity_verlet, contactManager, the contact_* classes) compiles and links
 * against this library unchanged.  Behaviour:
 *   - every function launches on the legacy default stream, like the
 *     reference's launchers (source/mphysics_cuda_def.cu);
 *   - the functions return void like the reference; a failure (bad
 *     argument, CUDA error) is recorded and can be read with xd_last_error()
 *     (xdem.h) instead of exiting the process;
 *   - tcm = 1 (the DHS model the application runs) is the only contact model.
 * The single-precision overloads (mphysics_cuda_dec.cuh:164-300) run the
 * xd_*_f twins, except cu_cylinder_hertzian_contact_force(float*), whose
 * declaration names the FP64 cylinder struct (the reference defines it with
 * the float one): it records XD_ERR_INVALID ("not provided").  The double-precision
 * cu_updatePolygonObjectData(device_polygon_mass_info*, ...) declared among
 * them (:296-298) is the mesh update the application calls and is provided.
 */
#ifndef MPHYSICS_CUDA_DEC_CUH
#define MPHYSICS_CUDA_DEC_CUH

#include <cuda_runtime.h>
#include <vector_types.h>

#if defined(__GNUC__)
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wdeprecated-declarations"
#endif

/* mphysics_cuda_dec.cuh:17-30 */
struct device_parameters
{
    bool rollingCondition;
    unsigned int np;
    unsigned int nsphere;
    unsigned int ncell;
    uint3 grid_size;
    double dt;
    double half2dt;
    double cell_size;
    double cohesion;
    double3 gravity;
    double3 world_origin;
};

/* mphysics_cuda_dec.cuh:32-41 */
struct device_polygon_info
{
    int id;
    double3 P;
    double3 Q;
    double3 R;
    double3 V;
    double3 W;
    double3 N;
};

/* mphysics_cuda_dec.cuh:43-55 */
struct device_plane_info
{
    double l1, l2;
    double3 u1;
    double3 u2;
    double3 uw;
    double3 xw;
    double3 pa;
    double3 pb;
    double3 w2;
    double3 w3;
    double3 w4;
};

/* mphysics_cuda_dec.cuh:57-65 */
struct device_polygon_mass_info
{
    double3 origin;
    double4 ep;
    double3 vel;
    double3 omega;
    double3 force;
    double3 moment;
};

/* mphysics_cuda_dec.cuh:67-76 */
struct device_cylinder_info
{
    double len, rbase, rtop;
    double3 pbase;
    double3 ptop;
    double3 origin;
    double3 vel;
    double3 omega;
    double4 ep;
};

/* mphysics_cuda_dec.cuh:78-88 */
struct device_contact_property
{
    double Ei, Ej;
    double pri, prj;
    double Gi, Gj;
    double rest;
    double fric;
    double rfric;
    double coh;
    double sratio;
};

/* mphysics_cuda_dec.cuh:91-108 */
struct device_force_constant
{
    double kn;
    double vn;
    double ks;
    double vs;
    double mu;
    double ms;
};

struct device_force_constant_d
{
    double kn;
    double vn;
    double ks;
    double vs;
    double mu;
};

/* mphysics_cuda_dec.cuh:110-160 */
void setSymbolicParameter(device_parameters *h_paras);

void vv_update_position(double *pos, double *vel, double *acc, unsigned int np);
void vv_update_velocity(double *vel, double *acc, double *omega, double *alpha, double *force, double *moment, double* mass, double* iner, unsigned int np);

void cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, double *pos, unsigned int np);
void cu_calculateHashAndIndexForPolygonSphere(
    unsigned int* hash, unsigned int* index,
    unsigned int sid, unsigned int nsphere, double *sphere);
void cu_reorderDataAndFindCellStart(unsigned int* hash, unsigned int* index, unsigned int* cstart, unsigned int* cend, unsigned int* sorted_index, unsigned int np, unsigned int ncell);

void cu_calculate_p2p(
    const int tcm, double* pos, double* vel,
    double* omega, double* force,
    double* moment, double* mass,
    unsigned int* sorted_index, unsigned int* cstart,
    unsigned int* cend, device_contact_property* cp, unsigned int np);

void cu_plane_contact_force(
    const int tcm, device_plane_info* plan,
    double* pos, double* vel, double* omega,
    double* force, double* moment, double* mass,
    unsigned int np, device_contact_property *cp);

void cu_cube_contact_force(
    const int tcm, device_plane_info* plan,
    double* pos, double* vel, double* omega,
    double* force, double* moment, double* mass,
    unsigned int np, device_contact_property *cp);

void cu_particle_polygonObject_collision(
    const int tcm, device_polygon_info* dpi, double* dsph, device_polygon_mass_info* dpmi,
    double* pos, double* vel, double* omega,
    double* force, double* moment, double* mass,
    unsigned int* sidx, unsigned int* cstart, unsigned int* cend, device_contact_property *cp,
    unsigned int np);

void cu_cylinder_hertzian_contact_force(
    const int tcm, device_cylinder_info* cyl,
    double* pos, double* vel, double* omega,
    double* force, double* moment, double* mass,
    unsigned int np, device_contact_property* cp,
    double3* mpos, double3* mf, double3* mm, double3& _mf, double3& _mm);

double3 reductionD3(double3* in, unsigned int np);
void cu_updatePolygonObjectData(
    double *vList, double* sph, device_polygon_info* poly,
    device_polygon_mass_info* dpmi, unsigned int np);

/* single precision (mphysics_cuda_dec.cuh:164-300): the xd_*_f twins */
struct device_parameters_f
{
    unsigned int np;
    unsigned int nsphere;
    unsigned int ncell;
    uint3 grid_size;
    float dt;
    float half2dt;
    float cell_size;
    float cohesion;
    float3 gravity;
    float3 world_origin;
};

struct device_polygon_info_f
{
    int id;
    float3 P;
    float3 Q;
    float3 R;
    float3 V;
    float3 W;
    float3 N;
};

struct device_plane_info_f
{
    float l1, l2;
    float3 u1;
    float3 u2;
    float3 uw;
    float3 xw;
    float3 pa;
    float3 pb;
    float3 w2;
    float3 w3;
    float3 w4;
};

struct device_polygon_mass_info_f
{
    float3 origin;
    float4 ep;
    float3 vel;
    float3 omega;
    float3 force;
    float3 moment;
};

struct device_cylinder_info_f
{
    float len, rbase, rtop;
    float3 pbase;
    float3 ptop;
    float3 origin;
    float3 vel;
    float3 omega;
    float4 ep;
};

struct device_contact_property_f
{
    float Ei, Ej;
    float pri, prj;
    float Gi, Gj;
    float rest;
    float fric;
    float rfric;
    float coh;
    float sratio;
};

struct device_force_constant_f
{
    float kn;
    float vn;
    float ks;
    float vs;
    float mu;
    float ms;
};

void setSymbolicParameter_f(device_parameters_f *h_paras);
void vv_update_position(float *pos, float *vel, float *acc, unsigned int np);
void vv_update_velocity(float *vel, float *acc, float *omega, float *alpha, float *force, float *moment, float* mass, float* iner, unsigned int np);
void cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, float *pos, unsigned int np);
void cu_calculateHashAndIndexForPolygonSphere(unsigned int* hash, unsigned int* index, unsigned int sid, unsigned int nsphere, float *sphere);
void cu_reorderDataAndFindCellStart_f(
    unsigned int* hash, unsigned int* index,
    unsigned int* cstart, unsigned int* cend,
    unsigned int* sorted_index, unsigned int np, unsigned int ncell);
void cu_calculate_p2p(
    const int tcm, float* pos, float* vel,
    float* omega, float* force,
    float* moment, float* mass,
    unsigned int* sorted_index, unsigned int* cstart,
    unsigned int* cend, device_contact_property_f* cp, unsigned int np);
void cu_plane_contact_force(
    const int tcm, device_plane_info_f* plan,
    float* pos, float* vel, float* omega,
    float* force, float* moment, float* mass,
    unsigned int np, device_contact_property_f *cp);
void cu_cube_contact_force(
    const int tcm, device_plane_info_f* plan,
    float* pos, float* vel, float* omega,
    float* force, float* moment, float* mass,
    unsigned int np, device_contact_property_f *cp);
void cu_particle_polygonObject_collision(
    const int tcm, device_polygon_info_f* dpi, float* dsph, device_polygon_mass_info_f* dpmi,
    float* pos, float* vel, float* omega,
    float* force, float* moment, float* mass,
    unsigned int* sidx, unsigned int* cstart, unsigned int* cend, device_contact_property_f *cp,
    unsigned int np);
void cu_cylinder_hertzian_contact_force(
    const int tcm, device_cylinder_info* cyl,
    float* pos, float* vel, float* omega,
    float* force, float* moment, float* mass,
    unsigned int np, device_contact_property_f* cp,
    float3* mpos, float3* mf, float3* mm, float3& _mf, float3& _mm);
/* provided (double precision): cu_updatePolygonObjectData, def.cu:469-475 */
void cu_updatePolygonObjectData(
    device_polygon_mass_info *dpmi, double* vList,
    double* sphere, device_polygon_info* dpi, unsigned int ntriangle);
float3 reductionD3(float3* in, unsigned int np);

#if defined(__GNUC__)
#pragma GCC diagnostic pop
#endif

#endif
