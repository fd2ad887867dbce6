// Internal launch helpers shared between libxdem's translation units.
#pragma once

#include <cuda_runtime.h>

#include "xd_internal.cuh"

namespace xd {

// cell grid (xd_grid.cu)
unsigned key_bits_for(unsigned ncell);
size_t reorder_scratch_bytes(unsigned n);
struct HistTable;   // xd_physics64.cuh: tangential-spring history of a scene

int launch_hash(const Params& P, unsigned* hash, unsigned* index, const double* pos, unsigned n,
                unsigned sid, cudaStream_t s);
int launch_fill_cells(unsigned* cstart, unsigned* cend, unsigned ncell, cudaStream_t s);
// The cell ranges of n keys already sorted in hash (with their values in
// index): cstart/cend at the runs' ends, sorted_index = index; a key >= ncell
// is skipped and raises *err.  Cells without keys are left as they are.
int launch_cell_bounds_sorted(unsigned* hash, unsigned* index, unsigned* cstart, unsigned* cend,
                              unsigned* sorted_index, unsigned n, unsigned ncell, unsigned* err, cudaStream_t s);
int reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart, unsigned* cend,
                                unsigned* sorted_index, unsigned n, unsigned ncell, void* scratch,
                                cudaStream_t s, bool check);

// integrator (xd_integrate.cu)
int launch_vv_position(const Params& P, double* pos, const double* vel, const double* acc,
                       unsigned np, cudaStream_t s);
int launch_vv_velocity(const Params& P, double* vel, double* acc, double* omega, double* alpha,
                       double* force, double* moment, const double* mass, const double* inertia,
                       unsigned np, cudaStream_t s);
int launch_vv_velocity_position(const Params& P, double* pos, double* vel, double* acc,
                                double* omega, double* alpha, double* force, double* moment,
                                const double* mass, const double* inertia, unsigned np,
                                cudaStream_t s);

// FP64 contacts (xd_contact64.cu)
int launch_p2p(const Params& P, const double* pos, const double* vel, const double* omega,
               double* force, double* moment, const double* mass, const unsigned* sorted,
               const unsigned* cstart, const unsigned* cend, const xd_contact_property* cp,
               unsigned np, cudaStream_t s, const HistTable* ht = nullptr);
int launch_cylinder(const Params& P, const xd_cylinder_info* cyl, const xd_contact_property* cp,
                    const double* pos, const double* vel, const double* omega, double* force,
                    double* moment, const double* mass, unsigned np, const double* mpos, double* mf,
                    double* mm, cudaStream_t s);
int launch_planes(const Params& P, const xd_plane_info* planes, const xd_contact_property* cps,
                  unsigned cp_stride, unsigned nplanes, const double* pos, const double* vel,
                  const double* omega, double* force, double* moment, const double* mass,
                  unsigned np, cudaStream_t s, const HistTable* ht = nullptr);
size_t polygon_scratch_bytes(unsigned np, unsigned nbodies);
int launch_polygon(const Params& P, const xd_polygon_info* dpi, xd_polygon_mass_info* dpmi,
                   const double* pos, const double* vel, const double* omega, double* force,
                   double* moment, const double* mass, const unsigned* sidx,
                   const unsigned* cstart, const unsigned* cend, const xd_contact_property* cp,
                   unsigned nbodies, void* scratch, cudaStream_t s, const HistTable* ht = nullptr);
int launch_body_advance(xd_polygon_mass_info* pmi, unsigned nbodies, double dt, cudaStream_t s);
int launch_update_polygon(const xd_polygon_mass_info* dpmi, const double* vlist, double* sphere,
                          xd_polygon_info* dpi, unsigned ntri, cudaStream_t s);
// The mesh update with the mixed form's moved check in one launch (see
// k_mesh_move): *flag raised when a vertex moved disp2 or more from ref; rec
// (nullable) receives the triangle records of the new pose.
struct TriRec;
int launch_mesh_move(const xd_polygon_mass_info* dpmi, const double* vlist, double* sphere, xd_polygon_info* dpi,
                     unsigned ntri, const float* ref, const double wo[3], float disp2, unsigned* flag,
                     TriRec* rec, cudaStream_t s);
// The mixed form's triangle records of a mesh as it stands.
int launch_tri_records(const xd_polygon_info* dpi, unsigned ntri, TriRec* rec, cudaStream_t s);
int reduction_d3(const double* in, unsigned n, double out[3], void* scratch, cudaStream_t s);
size_t reduction_scratch_bytes(unsigned n);
size_t pair_list_scratch_bytes(unsigned np);
int pair_list(const Params& P, const double* pos, const unsigned* sorted, const unsigned* cstart,
              const unsigned* cend, unsigned np, unsigned* counts, unsigned* pairs,
              unsigned long long cap, unsigned long long* total, void* scratch, cudaStream_t s);

}  // namespace xd
