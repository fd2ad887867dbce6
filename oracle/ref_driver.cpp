/*
 * Launch emulator around the reference's own FP64 (and FP32) DEM kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
 * reference's include/mphysics_cuda_impl.cuh, read where it lies in the
 * reference tree (see oracle/build_ref.sh), using the host stand-in headers
 * under oracle/refshim.  The result, oracle/_ref/libxdref.so, runs the
 * reference kernels sequentially on the CPU (one call per emulated thread, in
 * ascending thread order per block) and is used only to pin the C restatement
 * in oracle/xd_oracle.c and to generate the golden fixtures in tests/golden.
 *
 * Each entry point mirrors one launcher of the reference's
 * source/mphysics_cuda_def.cu (line numbers cited per function): same block
 * size, same kernel, same arguments.  thrust::sort_by_key (def.cu:92-94) is
 * restated as a stable sort of (key, value) pairs by key, which is what
 * thrust's radix sort produces for 32-bit keys.
 */
#include "mphysics_cuda_impl.cuh"

#include <algorithm>
#include <numeric>
#include <vector>

uint3 blockIdx;
uint3 threadIdx;
uint3 blockDim;
uint3 gridDim;
uint sharedHash[1024 + 1];

namespace {

template <typename F>
void launch(unsigned n, unsigned block, F&& body)
{
    if (n == 0) return;
    unsigned nt = std::min(block, n);
    unsigned nb = (n + nt - 1) / nt;
    blockDim = make_uint3(nt, 1, 1);
    gridDim = make_uint3(nb, 1, 1);
    for (unsigned b = 0; b < nb; ++b) {
        blockIdx = make_uint3(b, 0, 0);
        for (unsigned t = 0; t < nt; ++t) {
            threadIdx = make_uint3(t, 0, 0);
            body();
        }
    }
}

void stable_sort_by_key(unsigned* key, unsigned* val, unsigned n)
{
    std::vector<unsigned> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](unsigned a, unsigned b) { return key[a] < key[b]; });
    std::vector<unsigned> k(n), v(n);
    for (unsigned i = 0; i < n; ++i) { k[i] = key[order[i]]; v[i] = val[order[i]]; }
    std::copy(k.begin(), k.end(), key);
    std::copy(v.begin(), v.end(), val);
}

}  // namespace

extern "C" {

/* def.cu:13-16 */
void xdref_set_params(const device_parameters* p) { cte = *p; }
void xdref_set_params_f(const device_parameters_f* p) { cte_f = *p; }
unsigned xdref_sizeof_params() { return sizeof(device_parameters); }
unsigned xdref_sizeof_params_f() { return sizeof(device_parameters_f); }
unsigned xdref_sizeof_plane() { return sizeof(device_plane_info); }
unsigned xdref_sizeof_polygon() { return sizeof(device_polygon_info); }
unsigned xdref_sizeof_polygon_mass() { return sizeof(device_polygon_mass_info); }
unsigned xdref_sizeof_contact_property() { return sizeof(device_contact_property); }

/* def.cu:33-41 */
void xdref_vv_update_position(double* pos, double* vel, double* acc, unsigned np)
{
    launch(np, 512, [&] { vv_update_position_kernel((double4*)pos, (double3*)vel, (double3*)acc, np); });
}

/* def.cu:43-56 */
void xdref_vv_update_velocity(double* vel, double* acc, double* omega, double* alpha,
                              double* force, double* moment, double* mass, double* iner,
                              unsigned np)
{
    launch(np, 512, [&] {
        vv_update_velocity_kernel((double3*)vel, (double3*)acc, (double3*)omega, (double3*)alpha,
                                  (double3*)force, (double3*)moment, mass, iner, np);
    });
}

/* def.cu:58-66 */
void xdref_calculate_hash_and_index(unsigned* hash, unsigned* index, double* pos, unsigned np)
{
    launch(np, 512, [&] { calculateHashAndIndex_kernel(hash, index, (double4*)pos, np); });
}

/* def.cu:68-77 */
void xdref_calculate_hash_and_index_polysphere(unsigned* hash, unsigned* index, unsigned sid,
                                               unsigned nsphere, double* sphere)
{
    launch(nsphere, 512, [&] {
        calculateHashAndIndexForPolygonSphere_kernel(hash, index, sid, nsphere, (double4*)sphere);
    });
}

/* def.cu:80-108: sort, memset cstart=~0 / cend=0 over all cells, boundary kernel */
void xdref_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart,
                                       unsigned* cend, unsigned* sorted_index, unsigned np,
                                       unsigned ncell)
{
    stable_sort_by_key(hash, index, np);
    std::memset(cstart, 0xff, sizeof(unsigned) * ncell);
    std::memset(cend, 0, sizeof(unsigned) * ncell);
    launch(np, 512, [&] {
        reorderDataAndFindCellStart_kernel(hash, index, cstart, cend, sorted_index, np);
    });
}

/* def.cu:110-136 (tcm = 1, the model the application runs) */
void xdref_calculate_p2p(int tcm, double* pos, double* vel, double* omega, double* force,
                         double* moment, double* mass, unsigned* sorted_index, unsigned* cstart,
                         unsigned* cend, device_contact_property* cp, unsigned np)
{
    if (tcm == 0)
        launch(np, 256, [&] {
            calculate_p2p_kernel<0>((double4*)pos, (double3*)vel, (double3*)omega, (double3*)force,
                                    (double3*)moment, mass, sorted_index, cstart, cend, cp, np);
        });
    else
        launch(np, 256, [&] {
            calculate_p2p_kernel<1>((double4*)pos, (double3*)vel, (double3*)omega, (double3*)force,
                                    (double3*)moment, mass, sorted_index, cstart, cend, cp, np);
        });
}

/* def.cu:138-156 */
void xdref_plane_contact_force(int tcm, device_plane_info* plane, double* pos, double* vel,
                               double* omega, double* force, double* moment, double* mass,
                               unsigned np, device_contact_property* cp)
{
    (void)tcm;
    launch(np, 256, [&] {
        plane_contact_force_kernel<1>(plane, (double4*)pos, (double3*)vel, (double3*)omega,
                                      (double3*)force, (double3*)moment, cp, mass, np);
    });
}

/* def.cu:158-179: six launches over the cube's planes */
void xdref_cube_contact_force(int tcm, device_plane_info* planes, double* pos, double* vel,
                              double* omega, double* force, double* moment, double* mass,
                              unsigned np, device_contact_property* cp)
{
    for (int i = 0; i < 6; ++i)
        xdref_plane_contact_force(tcm, planes + i, pos, vel, omega, force, moment, mass, np, cp);
}

/* def.cu:181-200 (cu_cylinder_hertzian_contact_force, TCM = 1): mf and mm
 * are per-particle rows; every thread also zeroes row 0 (impl:732-733), so
 * after the sequential launch row 0 holds zero unless np == 1. */
void xdref_cylinder_contact_force(device_cylinder_info* cyl, double* pos, double* vel, double* omega,
                                  double* force, double* moment, double* mass, unsigned np,
                                  device_contact_property* cp, double* mpos, double* mf, double* mm)
{
    launch(np, 512, [&] {
        cylinder_hertzian_contact_force_kernel<1>(cyl, (double4*)pos, (double3*)vel, (double3*)omega,
                                                  (double3*)force, (double3*)moment, cp, mass, (double3*)mpos,
                                                  (double3*)mf, (double3*)mm, np);
    });
}

/* def.cu:203-221 */
void xdref_particle_polygon_collision(int tcm, device_polygon_info* dpi, double* dsph,
                                      device_polygon_mass_info* dpmi, double* pos, double* vel,
                                      double* omega, double* force, double* moment, double* mass,
                                      unsigned* sorted_index, unsigned* cstart, unsigned* cend,
                                      device_contact_property* cp, unsigned np)
{
    (void)tcm;
    launch(np, 512, [&] {
        particle_polygonObject_collision_kernel<1>(dpi, (double4*)dsph, dpmi, (double4*)pos,
                                                   (double3*)vel, (double3*)omega, (double3*)force,
                                                   (double3*)moment, mass, sorted_index, cstart,
                                                   cend, cp, np);
    });
}

/* def.cu:469-475 */
void xdref_update_polygon_object_data(device_polygon_mass_info* dpmi, double* vList,
                                      double* sphere, device_polygon_info* dpi, unsigned ntri)
{
    launch(ntri, 512, [&] {
        updatePolygonObjectData_kernel(dpmi, vList, (double4*)sphere, dpi, ntri);
    });
}

/* ---------------- FP32 twins (def.cu:255-475) ---------------- */

void xdref_vv_update_position_f(float* pos, float* vel, float* acc, unsigned np)
{
    launch(np, 512, [&] { vv_update_position_kernel((float4*)pos, (float3*)vel, (float3*)acc, np); });
}

void xdref_vv_update_velocity_f(float* vel, float* acc, float* omega, float* alpha, float* force,
                                float* moment, float* mass, float* iner, unsigned np)
{
    launch(np, 512, [&] {
        vv_update_velocity_kernel((float3*)vel, (float3*)acc, (float3*)omega, (float3*)alpha,
                                  (float3*)force, (float3*)moment, mass, iner, np);
    });
}

void xdref_calculate_hash_and_index_f(unsigned* hash, unsigned* index, float* pos, unsigned np)
{
    launch(np, 512, [&] { calculateHashAndIndex_kernel(hash, index, (float4*)pos, np); });
}

/* def.cu:294-302 */
void xdref_calculate_hash_and_index_polysphere_f(unsigned* hash, unsigned* index, unsigned sid,
                                                 unsigned nsphere, float* sphere)
{
    launch(nsphere, 512, [&] {
        calculateHashAndIndexForPolygonSphere_kernel(hash, index, sid, nsphere, (float4*)sphere);
    });
}

/* def.cu:305-333 */
void xdref_reorder_and_find_cell_start_f(unsigned* hash, unsigned* index, unsigned* cstart,
                                         unsigned* cend, unsigned* sorted_index, unsigned np,
                                         unsigned ncell)
{
    stable_sort_by_key(hash, index, np);
    std::memset(cstart, 0xff, sizeof(unsigned) * ncell);
    std::memset(cend, 0, sizeof(unsigned) * ncell);
    launch(np, 512, [&] {
        reorderDataAndFindCellStart_kernel_f(hash, index, cstart, cend, sorted_index, np);
    });
}

/* def.cu:335-361 (tcm = 1) */
void xdref_calculate_p2p_f(float* pos, float* vel, float* omega, float* force, float* moment,
                           float* mass, unsigned* sorted_index, unsigned* cstart, unsigned* cend,
                           device_contact_property_f* cp, unsigned np)
{
    launch(np, 512, [&] {
        calculate_p2p_kernel<1>((float4*)pos, (float3*)vel, (float3*)omega, (float3*)force,
                                (float3*)moment, mass, sorted_index, cstart, cend, cp, np);
    });
}

/* def.cu:363-381 (tcm = 1) */
void xdref_plane_contact_force_f(device_plane_info_f* plane, float* pos, float* vel, float* omega,
                                 float* force, float* moment, float* mass, unsigned np,
                                 device_contact_property_f* cp)
{
    launch(np, 512, [&] {
        plane_contact_force_kernel<1>(plane, (float4*)pos, (float3*)vel, (float3*)omega,
                                      (float3*)force, (float3*)moment, cp, mass, np);
    });
}

/* def.cu:383-404: six launches over the cube's planes */
void xdref_cube_contact_force_f(device_plane_info_f* planes, float* pos, float* vel, float* omega,
                                float* force, float* moment, float* mass, unsigned np,
                                device_contact_property_f* cp)
{
    for (int i = 0; i < 6; ++i)
        xdref_plane_contact_force_f(planes + i, pos, vel, omega, force, moment, mass, np, cp);
}

/* def.cu:428-446 (tcm = 1); the body reaction's += runs in thread order here */
void xdref_particle_polygon_collision_f(device_polygon_info_f* dpi, float* dsph,
                                        device_polygon_mass_info_f* dpmi, float* pos, float* vel,
                                        float* omega, float* force, float* moment, float* mass,
                                        unsigned* sorted_index, unsigned* cstart, unsigned* cend,
                                        device_contact_property_f* cp, unsigned np)
{
    launch(np, 512, [&] {
        particle_polygonObject_collision_kernel<1>(dpi, (float4*)dsph, dpmi, (float4*)pos,
                                                   (float3*)vel, (float3*)omega, (float3*)force,
                                                   (float3*)moment, mass, sorted_index, cstart,
                                                   cend, cp, np);
    });
}

}  // extern "C"
