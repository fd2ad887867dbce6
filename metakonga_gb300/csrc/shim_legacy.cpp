// libxdem_legacy.so: the reference's legacy DEM launcher interface
// (include/cu_dem_dec.cuh) implemented on libxdem's legacy C ABI
// (include/xdem_legacy.h).  Every call launches on the legacy default stream
// like the reference's launchers (source/cu_dem_def.cu); failures are kept
// for xd_last_error().
#include <cuda_runtime.h>

#include "cu_dem_dec.cuh"
#include "xdem_legacy.h"

static_assert(sizeof(device_parameters) == sizeof(xd_legacy_parameters), "legacy device_parameters layout");
static_assert(sizeof(device_plane_info) == sizeof(xd_legacy_plane_info), "legacy device_plane_info layout");
static_assert(sizeof(cu_polygon) == sizeof(xd_legacy_polygon), "cu_polygon layout");
static_assert(sizeof(cu_mass_info) == sizeof(xd_legacy_mass_info), "cu_mass_info layout");

namespace {
void* const kDefaultStream = nullptr;
}

void setSymbolicParameter(device_parameters* h_paras)
{
    xd_legacy_set_symbolic_parameter(reinterpret_cast<const xd_legacy_parameters*>(h_paras));
}

void vv_update_position(double* pos, double* vel, double* acc, unsigned int np)
{
    xd_legacy_vv_update_position(pos, vel, acc, np, kDefaultStream);
}

void vv_update_velocity(double* vel, double* acc, double* omega, double* alpha, double* force, double* moment,
                        unsigned int np)
{
    xd_legacy_vv_update_velocity(vel, acc, omega, alpha, force, moment, np, kDefaultStream);
}

void cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, double* pos, unsigned int np)
{
    xd_legacy_calculate_hash_and_index(hash, index, pos, np, kDefaultStream);
}

void cu_reorderDataAndFindCellStart(unsigned int* hash, unsigned int* index, unsigned int* cstart,
                                    unsigned int* cend, unsigned int* sorted_index, unsigned int np,
                                    unsigned int nc)
{
    xd_legacy_reorder_and_find_cell_start(hash, index, cstart, cend, sorted_index, np, nc, kDefaultStream);
}

void cu_calculate_p2p(double* pos, double* vel, double* acc, double* omega, double* alpha, double* force,
                      double* moment, unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend,
                      unsigned int np, unsigned int cRun)
{
    xd_legacy_calculate_p2p(pos, vel, acc, omega, alpha, force, moment, sorted_index, cstart, cend, np, cRun,
                            kDefaultStream);
}

void cu_cube_hertzian_contact_force(device_plane_info* plans, double kn, double vn, double ks, double vs,
                                    double mu, bool* isLineContact, double* pos, double* vel, double* omega,
                                    double* force, double* moment, unsigned int np)
{
    xd_legacy_cube_hertzian_contact_force(reinterpret_cast<const xd_legacy_plane_info*>(plans), kn, vn, ks, vs, mu,
                                          isLineContact, pos, vel, omega, force, moment, np, kDefaultStream);
}

double3 cu_shape_hertzian_contact_force(cu_mass_info* minfo, cu_polygon* polygons, unsigned int* id_set,
                                        unsigned int* poly_start, unsigned int* poly_end, double kn, double vn,
                                        double ks, double vs, double mu, bool* isLineContact, double* pos,
                                        double* vel, double* omega, double* force, double* moment,
                                        double3* bforce, unsigned int np, unsigned int* sorted_id,
                                        unsigned int* cell_start, unsigned int* cell_end)
{
    double out[3] = { 0.0, 0.0, 0.0 };
    xd_legacy_shape_hertzian_contact_force(reinterpret_cast<const xd_legacy_mass_info*>(minfo),
                                           reinterpret_cast<const xd_legacy_polygon*>(polygons), id_set,
                                           poly_start, poly_end, kn, vn, ks, vs, mu, isLineContact, pos, vel,
                                           omega, force, moment, reinterpret_cast<double*>(bforce), np, sorted_id,
                                           cell_start, cell_end, out, kDefaultStream);
    double3 r;
    r.x = out[0];
    r.y = out[1];
    r.z = out[2];
    return r;
}

void cu_update_polygons_position(double3* mpos, double* A, double3* local_vertice, unsigned int nvertex,
                                 double3* pos)
{
    xd_legacy_update_polygons_position(reinterpret_cast<const double*>(mpos), A,
                                       reinterpret_cast<const double*>(local_vertice), nvertex,
                                       reinterpret_cast<double*>(pos), kDefaultStream);
}

void cu_update_polygons_information(cu_polygon* polygons, uint3* indice, double3* pos, unsigned int ni)
{
    xd_legacy_update_polygons_information(reinterpret_cast<xd_legacy_polygon*>(polygons),
                                          reinterpret_cast<const unsigned*>(indice),
                                          reinterpret_cast<const double*>(pos), ni, kDefaultStream);
}

void cu_mergedata(double* data, double* pos, unsigned int np, double3* vertice, unsigned int snp)
{
    xd_legacy_mergedata(data, pos, np, reinterpret_cast<const double*>(vertice), snp, kDefaultStream);
}
