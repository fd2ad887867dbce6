/*
 * Launch emulator around the reference's own legacy DEM kernels
 * (include/cu_dem_impl.cuh, the interface of include/cu_dem_dec.cuh).
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled with the reference's header where it
 * lies in the reference tree, using the host stand-ins under oracle/refshim
 * (oracle/Makefile, target ref), into oracle/_ref/libxdref_legacy.so; used to
 * generate the legacy golden fixtures (tests/golden/make_golden_legacy.py).
 * Each entry point mirrors one launcher of source/cu_dem_def.cu (cited per
 * function): block size 256, the same kernel and arguments, threads run in
 * ascending order.  thrust::sort_by_key is a stable sort of (key, value) by
 * key; the shape call's reduce6 + host block sum (def.cu:210-229) is a plain
 * sum of the force rows in particle order.
 */
#include "cu_dem_impl.cuh"

#include <algorithm>
#include <numeric>
#include <vector>

uint3 blockIdx;
uint3 threadIdx;
uint3 blockDim;
uint3 gridDim;
uint sharedHash[256 + 1];

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
    std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) { return key[a] < key[b]; });
    std::vector<unsigned> k(n), v(n);
    for (unsigned i = 0; i < n; ++i) { k[i] = key[order[i]]; v[i] = val[order[i]]; }
    std::copy(k.begin(), k.end(), key);
    std::copy(v.begin(), v.end(), val);
}

}  // namespace

extern "C" {

unsigned xdrefl_sizeof_params() { return sizeof(device_parameters); }
unsigned xdrefl_sizeof_plane() { return sizeof(device_plane_info); }
unsigned xdrefl_sizeof_polygon() { return sizeof(cu_polygon); }
unsigned xdrefl_sizeof_mass_info() { return sizeof(cu_mass_info); }

/* def.cu:25-28 */
void xdrefl_set_params(const device_parameters* p) { cte = *p; }

/* def.cu:30-37 */
void xdrefl_vv_update_position(double* pos, double* vel, double* acc, unsigned np)
{
    launch(np, 256, [&] { vv_update_position_kernel((double4*)pos, (double4*)vel, (double4*)acc); });
}

/* def.cu:39-49 */
void xdrefl_vv_update_velocity(double* vel, double* acc, double* omega, double* alpha, double* force,
                               double* moment, unsigned np)
{
    launch(np, 256, [&] {
        vv_update_velocity_kernel((double4*)vel, (double4*)acc, (double4*)omega, (double4*)alpha,
                                  (double3*)force, (double3*)moment);
    });
}

/* def.cu:51-55 */
void xdrefl_mergedata(double* data, double* pos, unsigned np, double* vertice, unsigned snp)
{
    launch(np + snp, 256, [&] { mergedata_kernel((double4*)data, (double4*)pos, np, (double3*)vertice, snp); });
}

/* def.cu:57-69 */
void xdrefl_calculate_hash_and_index(unsigned* hash, unsigned* index, double* pos, unsigned np)
{
    launch(np, 256, [&] { calculateHashAndIndex_kernel(hash, index, (double4*)pos); });
    stable_sort_by_key(hash, index, np);
}

/* def.cu:71-90: cstart reset, cend kept */
void xdrefl_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart,
                                        unsigned* cend, unsigned* sorted_index, unsigned np,
                                        unsigned nc)
{
    std::memset(cstart, 0xff, sizeof(unsigned) * nc);
    launch(np, 256, [&] { reorderDataAndFindCellStart_kernel(hash, index, cstart, cend, sorted_index); });
}

/* def.cu:92-107 */
void xdrefl_calculate_p2p(double* pos, double* vel, double* acc, double* omega, double* alpha,
                          double* force, double* moment, unsigned* sorted_index, unsigned* cstart,
                          unsigned* cend, unsigned np, unsigned cRun)
{
    launch(np, 256, [&] {
        calculate_p2p_kernel((double4*)pos, (double4*)vel, (double4*)acc, (double4*)omega,
                             (double4*)alpha, (double3*)force, (double3*)moment, sorted_index, cstart,
                             cend, cRun);
    });
}

/* def.cu:109-138 */
void xdrefl_cube_hertzian_contact_force(device_plane_info* planes, double kn, double vn, double ks,
                                        double vs, double mu, bool* isLineContact, double* pos,
                                        double* vel, double* omega, double* force, double* moment,
                                        unsigned np)
{
    launch(np, 256, [&] {
        cube_hertzian_contact_force_kernel(planes, kn, vn, ks, vs, mu, isLineContact, (double4*)pos,
                                           (double4*)vel, (double4*)omega, (double3*)force,
                                           (double3*)moment);
    });
}

/* def.cu:140-232 */
void xdrefl_shape_hertzian_contact_force(cu_mass_info* minfo, cu_polygon* polygons, unsigned* id_set,
                                         unsigned* poly_start, unsigned* poly_end, double kn, double vn,
                                         double ks, double vs, double mu, bool* isLineContact,
                                         double* pos, double* vel, double* omega, double* force,
                                         double* moment, unsigned np, unsigned* sorted_id,
                                         unsigned* cell_start, unsigned* cell_end, double* out)
{
    std::memset(force, 0, sizeof(double) * 3 * np);
    std::memset(moment, 0, sizeof(double) * 3 * np);
    launch(np, 256, [&] {
        shpae_hertzian_contact_force_kernel(minfo, polygons, id_set, poly_start, poly_end, kn, vn, ks,
                                            vs, mu, isLineContact, (double4*)pos, (double4*)vel,
                                            (double4*)omega, (double3*)force, (double3*)moment,
                                            sorted_id, cell_start, cell_end);
    });
    launch(np, 256, [&] {
        shape_line_or_edge_contact_force_kernel(minfo, polygons, id_set, poly_start, poly_end, kn, vn,
                                                ks, vs, mu, isLineContact, (double4*)pos,
                                                (double4*)vel, (double4*)omega, (double3*)force,
                                                (double3*)moment, sorted_id, cell_start, cell_end);
    });
    out[0] = out[1] = out[2] = 0.0;
    for (unsigned i = 0; i < np; ++i)
        for (int c = 0; c < 3; ++c) out[c] += force[3 * (size_t)i + c];
}

/* def.cu:234-238 */
void xdrefl_update_polygons_position(double* mpos, double* A, double* local_vertice, unsigned nvertex,
                                     double* pos)
{
    launch(nvertex, 256, [&] {
        update_polygons_position((double3*)mpos, A, (double3*)local_vertice, nvertex, (double3*)pos);
    });
}

/* def.cu:240-244 */
void xdrefl_update_polygons_information(cu_polygon* polygons, unsigned* indice, double* pos, unsigned ni)
{
    launch(ni, 256, [&] { update_polygons_information(polygons, (uint3*)indice, (double3*)pos, ni); });
}

}  // extern "C"
