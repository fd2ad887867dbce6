/*
 * cu_dem_dec.cuh -- the legacy DEM launcher interface of the xdynamics
 * reference (include/cu_dem_dec.cuh:41-113), with the same struct layouts and
 * C++ signatures, so that the parSIM classes (dem_force, cell_grid,
 * Verlet_integrator, geometry) compile and link unchanged against
 * libxdem_legacy.so.  It is a separate header and library because its
 * device_parameters and device_plane_info differ from the live interface's
 * (mphysics_cuda_dec.cuh).  Behaviour: include/xdem_legacy.h.
 */
#ifndef CU_DEM_DEC_CUH
#define CU_DEM_DEC_CUH

#include <vector_types.h>

struct device_parameters
{
    unsigned int np;
    unsigned int nsp;
    unsigned int ncell;
    uint3 grid_size;
    double dt;
    double half2dt;
    double cell_size;
    double3 gravity;
    double3 world_origin;

    double kn;
    double vn;
    double ks;
    double vs;
    double mu;

    double cohesive;
};

struct device_plane_info
{
    double l1, l2;
    double3 u1;
    double3 u2;
    double3 uw;
    double3 xw;
    double3 pa;
    double3 pb;
};

struct cu_polygon
{
    double3 P;
    double3 Q;
    double3 R;
    double3 V;
    double3 W;
    double3 N;
};

struct cu_mass_info
{
    double3 pos;
    double3 vel;
};

struct cu_contact_info
{
    double penetration;
    double3 unit;
};

void setSymbolicParameter(device_parameters *h_paras);

void vv_update_position(double *pos, double *vel, double *acc, unsigned int np);
void vv_update_velocity(double *vel, double *acc, double *omega, double *alpha, double *force, double *moment, unsigned int np);

void cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, double *pos, unsigned int np);
void cu_reorderDataAndFindCellStart(unsigned int* hash, unsigned int* index, unsigned int* cstart, unsigned int* cend, unsigned int* sorted_index, unsigned int np, unsigned int nc);

void cu_calculate_p2p(double* pos, double* vel, double* acc, double* omega, double* alpha, double* force, double* moment, unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend, unsigned int np, unsigned int cRun = 0);

void cu_cube_hertzian_contact_force(device_plane_info* plans, double kn, double vn, double ks, double vs, double mu, bool* isLineContact, double* pos, double* vel, double* omega, double* force, double* moment, unsigned int np);
double3 cu_shape_hertzian_contact_force(cu_mass_info *minfo, cu_polygon* polygons, unsigned int *id_set, unsigned int *poly_start, unsigned int *poly_end, double kn, double vn, double ks, double vs, double mu, bool* isLineContact, double* pos, double* vel, double* omega, double* force, double* moment, double3* bforce, unsigned int np, unsigned int* sorted_id, unsigned int* cell_start, unsigned int* cell_end);
void cu_update_polygons_position(double3* mpos, double* A, double3* local_vertice, unsigned int nvertex, double3* pos);
void cu_update_polygons_information(cu_polygon* polygons, uint3 *indice, double3* pos, unsigned int ni);
void cu_mergedata(double* data, double* pos, unsigned int np, double3* vertice, unsigned int snp);

#endif
