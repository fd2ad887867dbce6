// libxdem_mphysics.so: the reference's C++ DEM library interface
// (include/mphysics_cuda_dec.cuh) and host classes (include/xdem_host.h)
// implemented on libxdem's C ABI (include/xdem.h).  Every call launches on
// the legacy default stream like the reference's launchers
// (source/mphysics_cuda_def.cu); failures are kept for xd_last_error().
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>

#include "mphysics_cuda_dec.cuh"
#include "xdem.h"
#include "xdem_host.h"

static_assert(sizeof(device_parameters) == sizeof(xd_device_parameters), "device_parameters layout");
static_assert(sizeof(device_plane_info) == sizeof(xd_plane_info), "device_plane_info layout");
static_assert(sizeof(device_cylinder_info) == sizeof(xd_cylinder_info) && offsetof(device_cylinder_info, ep) == 144,
              "device_cylinder_info layout");
static_assert(sizeof(device_polygon_info) == sizeof(xd_polygon_info), "device_polygon_info layout");
static_assert(sizeof(device_polygon_mass_info) == sizeof(xd_polygon_mass_info), "mass info layout");
static_assert(sizeof(device_contact_property) == sizeof(xd_contact_property), "property layout");

namespace {
void* const kDefaultStream = nullptr;

void not_provided(const char* name) { xd_report_unsupported(name); }
}  // namespace

// ---------------------------------------------------------------- FP64 API

void setSymbolicParameter(device_parameters* h_paras)
{
    xd_set_symbolic_parameter(reinterpret_cast<const xd_device_parameters*>(h_paras));
}

void vv_update_position(double* pos, double* vel, double* acc, unsigned int np)
{
    xd_vv_update_position(pos, vel, acc, np, kDefaultStream);
}

void vv_update_velocity(double* vel, double* acc, double* omega, double* alpha, double* force,
                        double* moment, double* mass, double* iner, unsigned int np)
{
    xd_vv_update_velocity(vel, acc, omega, alpha, force, moment, mass, iner, np, kDefaultStream);
}

void cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, double* pos, unsigned int np)
{
    xd_calculate_hash_and_index(hash, index, pos, np, kDefaultStream);
}

void cu_calculateHashAndIndexForPolygonSphere(unsigned int* hash, unsigned int* index,
                                              unsigned int sid, unsigned int nsphere, double* sphere)
{
    xd_calculate_hash_and_index_polysphere(hash, index, sid, nsphere, sphere, kDefaultStream);
}

void cu_reorderDataAndFindCellStart(unsigned int* hash, unsigned int* index, unsigned int* cstart,
                                    unsigned int* cend, unsigned int* sorted_index, unsigned int np,
                                    unsigned int ncell)
{
    xd_reorder_and_find_cell_start(hash, index, cstart, cend, sorted_index, np, ncell, kDefaultStream);
}

void cu_calculate_p2p(const int tcm, double* pos, double* vel, double* omega, double* force,
                      double* moment, double* mass, unsigned int* sorted_index,
                      unsigned int* cstart, unsigned int* cend, device_contact_property* cp,
                      unsigned int np)
{
    xd_calculate_p2p(tcm, pos, vel, omega, force, moment, mass, sorted_index, cstart, cend,
                     reinterpret_cast<const xd_contact_property*>(cp), np, kDefaultStream);
}

void cu_plane_contact_force(const int tcm, device_plane_info* plan, double* pos, double* vel,
                            double* omega, double* force, double* moment, double* mass,
                            unsigned int np, device_contact_property* cp)
{
    xd_plane_contact_force(tcm, reinterpret_cast<const xd_plane_info*>(plan), pos, vel, omega, force,
                           moment, mass, np, reinterpret_cast<const xd_contact_property*>(cp),
                           kDefaultStream);
}

void cu_cube_contact_force(const int tcm, device_plane_info* plan, double* pos, double* vel,
                           double* omega, double* force, double* moment, double* mass,
                           unsigned int np, device_contact_property* cp)
{
    xd_cube_contact_force(tcm, reinterpret_cast<const xd_plane_info*>(plan), pos, vel, omega, force,
                          moment, mass, np, reinterpret_cast<const xd_contact_property*>(cp),
                          kDefaultStream);
}

void cu_particle_polygonObject_collision(const int tcm, device_polygon_info* dpi, double* dsph,
                                         device_polygon_mass_info* dpmi, double* pos, double* vel,
                                         double* omega, double* force, double* moment,
                                         double* mass, unsigned int* sidx, unsigned int* cstart,
                                         unsigned int* cend, device_contact_property* cp,
                                         unsigned int np)
{
    // the body count is not part of the reference signature: reactions are
    // added with atomics (nbodies = 0)
    xd_particle_polygon_collision(tcm, reinterpret_cast<const xd_polygon_info*>(dpi), dsph,
                                  reinterpret_cast<xd_polygon_mass_info*>(dpmi), pos, vel, omega,
                                  force, moment, mass, sidx, cstart, cend,
                                  reinterpret_cast<const xd_contact_property*>(cp), np, 0,
                                  kDefaultStream);
}

void cu_cylinder_hertzian_contact_force(const int tcm, device_cylinder_info* cyl, double* pos, double* vel,
                                        double* omega, double* force, double* moment, double* mass,
                                        unsigned int np, device_contact_property* cp, double3* mpos,
                                        double3* mf, double3* mm, double3&, double3&)
{
    // the reference's wrapper leaves _mf and _mm unwritten (def.cu:181-200)
    xd_cylinder_contact_force(tcm, reinterpret_cast<const xd_cylinder_info*>(cyl), pos, vel, omega, force,
                              moment, mass, np, reinterpret_cast<const xd_contact_property*>(cp),
                              reinterpret_cast<const double*>(mpos), reinterpret_cast<double*>(mf),
                              reinterpret_cast<double*>(mm), kDefaultStream);
}

double3 reductionD3(double3* in, unsigned int np)
{
    double out[3] = { 0.0, 0.0, 0.0 };
    xd_reduction_d3(reinterpret_cast<const double*>(in), np, out, kDefaultStream);
    return make_double3(out[0], out[1], out[2]);
}

// mphysics_cuda_def.cu:244-251 launches an empty kernel (impl:1063-1092)
void cu_updatePolygonObjectData(double*, double*, device_polygon_info*, device_polygon_mass_info*,
                                unsigned int)
{
}

// mphysics_cuda_def.cu:469-475
void cu_updatePolygonObjectData(device_polygon_mass_info* dpmi, double* vList, double* sphere,
                                device_polygon_info* dpi, unsigned int ntriangle)
{
    xd_update_polygon_object_data(reinterpret_cast<const xd_polygon_mass_info*>(dpmi), vList,
                                  sphere, reinterpret_cast<xd_polygon_info*>(dpi), ntriangle,
                                  kDefaultStream);
}

// ---------------------------------------------------------------- FP32 API

static_assert(sizeof(device_parameters_f) == sizeof(xd_device_parameters_f), "device_parameters_f layout");
static_assert(sizeof(device_plane_info_f) == sizeof(xd_plane_info_f), "device_plane_info_f layout");
static_assert(sizeof(device_polygon_info_f) == sizeof(xd_polygon_info_f), "device_polygon_info_f layout");
static_assert(sizeof(device_polygon_mass_info_f) == sizeof(xd_polygon_mass_info_f), "mass info f layout");
static_assert(sizeof(device_contact_property_f) == sizeof(xd_contact_property_f), "property f layout");

void setSymbolicParameter_f(device_parameters_f* h_paras)
{
    xd_set_symbolic_parameter_f(reinterpret_cast<const xd_device_parameters_f*>(h_paras));
}

void vv_update_position(float* pos, float* vel, float* acc, unsigned int np)
{
    xd_vv_update_position_f(pos, vel, acc, np, kDefaultStream);
}

void vv_update_velocity(float* vel, float* acc, float* omega, float* alpha, float* force, float* moment,
                        float* mass, float* iner, unsigned int np)
{
    xd_vv_update_velocity_f(vel, acc, omega, alpha, force, moment, mass, iner, np, kDefaultStream);
}

void cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, float* pos, unsigned int np)
{
    xd_calculate_hash_and_index_f(hash, index, pos, np, kDefaultStream);
}

void cu_calculateHashAndIndexForPolygonSphere(unsigned int* hash, unsigned int* index, unsigned int sid,
                                              unsigned int nsphere, float* sphere)
{
    xd_calculate_hash_and_index_polysphere_f(hash, index, sid, nsphere, sphere, kDefaultStream);
}

void cu_reorderDataAndFindCellStart_f(unsigned int* hash, unsigned int* index, unsigned int* cstart,
                                      unsigned int* cend, unsigned int* sorted_index, unsigned int np,
                                      unsigned int ncell)
{
    xd_reorder_and_find_cell_start_f(hash, index, cstart, cend, sorted_index, np, ncell, kDefaultStream);
}

void cu_calculate_p2p(const int tcm, float* pos, float* vel, float* omega, float* force, float* moment,
                      float* mass, unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend,
                      device_contact_property_f* cp, unsigned int np)
{
    xd_calculate_p2p_f(tcm, pos, vel, omega, force, moment, mass, sorted_index, cstart, cend,
                       reinterpret_cast<const xd_contact_property_f*>(cp), np, kDefaultStream);
}

void cu_plane_contact_force(const int tcm, device_plane_info_f* plan, float* pos, float* vel, float* omega,
                            float* force, float* moment, float* mass, unsigned int np,
                            device_contact_property_f* cp)
{
    xd_plane_contact_force_f(tcm, reinterpret_cast<const xd_plane_info_f*>(plan), pos, vel, omega, force,
                             moment, mass, np, reinterpret_cast<const xd_contact_property_f*>(cp),
                             kDefaultStream);
}

void cu_cube_contact_force(const int tcm, device_plane_info_f* plan, float* pos, float* vel, float* omega,
                           float* force, float* moment, float* mass, unsigned int np,
                           device_contact_property_f* cp)
{
    xd_cube_contact_force_f(tcm, reinterpret_cast<const xd_plane_info_f*>(plan), pos, vel, omega, force,
                            moment, mass, np, reinterpret_cast<const xd_contact_property_f*>(cp),
                            kDefaultStream);
}

void cu_particle_polygonObject_collision(const int tcm, device_polygon_info_f* dpi, float* dsph,
                                         device_polygon_mass_info_f* dpmi, float* pos, float* vel,
                                         float* omega, float* force, float* moment, float* mass,
                                         unsigned int* sidx, unsigned int* cstart, unsigned int* cend,
                                         device_contact_property_f* cp, unsigned int np)
{
    // the body count is not part of the reference signature: reactions are
    // added with atomics (nbodies = 0)
    xd_particle_polygon_collision_f(tcm, reinterpret_cast<const xd_polygon_info_f*>(dpi), dsph,
                                    reinterpret_cast<xd_polygon_mass_info_f*>(dpmi), pos, vel, omega, force,
                                    moment, mass, sidx, cstart, cend,
                                    reinterpret_cast<const xd_contact_property_f*>(cp), np, 0, kDefaultStream);
}

void cu_cylinder_hertzian_contact_force(const int, device_cylinder_info*, float*, float*, float*,
                                        float*, float*, float*, unsigned int,
                                        device_contact_property_f*, float3*, float3*, float3*,
                                        float3&, float3&)
{
    // no caller in the reference application, and declared with the FP64
    // cylinder struct but defined with the float one (def.cu:406-426)
    not_provided("cu_cylinder_hertzian_contact_force(float)");
}

float3 reductionD3(float3* in, unsigned int np)
{
    float out[3] = { 0.f, 0.f, 0.f };
    xd_reduction_f3(reinterpret_cast<const float*>(in), np, out, kDefaultStream);
    return make_float3(out[0], out[1], out[2]);
}

// ------------------------------------------------------------ host classes

VEC3D grid_base::wo;
double grid_base::cs = 0.0;
VEC3UI grid_base::gs;

grid_base::grid_base()
    : type(NEIGHBORHOOD), d_sorted_id(NULL), d_cell_id(NULL), d_body_id(NULL), d_cell_start(NULL),
      d_cell_end(NULL), nse(0), ng(0)
{
}

grid_base::grid_base(Type t)
    : type(t), d_sorted_id(NULL), d_cell_id(NULL), d_body_id(NULL), d_cell_start(NULL),
      d_cell_end(NULL), nse(0), ng(0)
{
}

grid_base::~grid_base() { clear(); }

// grid_base::clear (grid_base.cpp:59-77), GPU branch
void grid_base::clear()
{
    if (d_cell_id) cudaFree(d_cell_id);
    if (d_body_id) cudaFree(d_body_id);
    if (d_sorted_id) cudaFree(d_sorted_id);
    if (d_cell_start) cudaFree(d_cell_start);
    if (d_cell_end) cudaFree(d_cell_end);
    d_cell_id = d_body_id = d_sorted_id = d_cell_start = d_cell_end = NULL;
}

// grid_base::initialize (grid_base.cpp:79-92), GPU branch
void grid_base::initialize(unsigned int np) { cuAllocMemory(np); }

void grid_base::allocMemory(unsigned int n) { cuAllocMemory(n); }

// grid_base::cuAllocMemory (grid_base.cpp:105-114)
void grid_base::cuAllocMemory(unsigned int n)
{
    clear();
    ng = gs.x * gs.y * gs.z;
    size_t m = n ? n : 1;
    cudaMalloc((void**)&d_cell_id, sizeof(unsigned int) * m);
    cudaMalloc((void**)&d_body_id, sizeof(unsigned int) * m);
    cudaMalloc((void**)&d_sorted_id, sizeof(unsigned int) * m);
    cudaMalloc((void**)&d_cell_start, sizeof(unsigned int) * (ng ? ng : 1));
    cudaMalloc((void**)&d_cell_end, sizeof(unsigned int) * (ng ? ng : 1));
    nse = n;
}

// grid_base::getCellNumber (grid_base.cpp:139-146): the host path keeps abs(floor(.))
VEC3I grid_base::getCellNumber(double x, double y, double z)
{
    return VEC3I(static_cast<int>(std::abs(std::floor((x - wo.x) / cs))),
                 static_cast<int>(std::abs(std::floor((y - wo.y) / cs))),
                 static_cast<int>(std::abs(std::floor((z - wo.z) / cs))));
}

// grid_base::getHash (grid_base.cpp:148-155)
unsigned int grid_base::getHash(VEC3I& c3)
{
    int x = c3.x & (int)(gs.x - 1), y = c3.y & (int)(gs.y - 1), z = c3.z & (int)(gs.z - 1);
    return (unsigned)((z * (int)gs.y) * (int)gs.x + (y * (int)gs.x) + x);
}

neighborhood_cell::neighborhood_cell() : grid_base(NEIGHBORHOOD) {}
neighborhood_cell::~neighborhood_cell() {}

// neighborhood_cell::detection (neighborhood_cell.cpp:91-107), GPU branch
void neighborhood_cell::detection(double* pos, double* spos, unsigned int np, unsigned int snp)
{
    cu_calculateHashAndIndex(d_cell_id, d_body_id, pos, np);
    if (snp && spos) cu_calculateHashAndIndexForPolygonSphere(d_cell_id, d_body_id, np, snp, spos);
    cu_reorderDataAndFindCellStart(d_cell_id, d_body_id, d_cell_start, d_cell_end, d_sorted_id,
                                   np + snp, ng);
}

void neighborhood_cell::detection_f(float*, float*, unsigned int, unsigned int)
{
    not_provided("neighborhood_cell::detection_f");
}

// velocity_verlet (velocity_verlet.cpp:18-43), GPU branch
void velocity_verlet::updatePosition(double* dpos, double* dvel, double* dacc, unsigned int np)
{
    vv_update_position(dpos, dvel, dacc, np);
}

void velocity_verlet::updateVelocity(double* dvel, double* dacc, double* domega, double* dalpha,
                                     double* dforce, double* dmoment, double* dmass,
                                     double* dinertia, unsigned int np)
{
    vv_update_velocity(dvel, dacc, domega, dalpha, dforce, dmoment, dmass, dinertia, np);
}

void velocity_verlet::updatePosition(float* dpos, float* dvel, float* dacc, unsigned int np)
{
    vv_update_position(dpos, dvel, dacc, np);
}

void velocity_verlet::updateVelocity(float* dvel, float* dacc, float* domega, float* dalpha,
                                     float* dforce, float* dmoment, float* dmass, float* dinertia,
                                     unsigned int np)
{
    vv_update_velocity(dvel, dacc, domega, dalpha, dforce, dmoment, dmass, dinertia, np);
}
