// Internal interface of the mixed-precision scene path (xd_mixed.cu).
#pragma once

#include <cuda_runtime.h>

#include "xd_internal.cuh"

namespace xd {

// Phase hooks for event timing: begin/end of phase p on stream q.
struct Phases {
    void* ctx = nullptr;
    void (*fn)(void*, int, bool, cudaStream_t) = nullptr;
    void begin(int p, cudaStream_t q) const { if (fn) fn(ctx, p, true, q); }
    void end(int p, cudaStream_t q) const { if (fn) fn(ctx, p, false, q); }
};

struct MixedScene;

int mixed_create(const xd_scene_desc& d, MixedScene** out);
void mixed_destroy(MixedScene* s);
int mixed_upload(MixedScene* s, const double* pos, const double* vel, const double* acc,
                 const double* omega, const double* alpha, const double* mass,
                 const double* inertia, cudaStream_t q, bool sync = true);
int mixed_download(MixedScene* s, double* pos, double* vel, double* acc, double* omega,
                   double* alpha, double* force, double* moment, cudaStream_t q, bool sync = true);
int mixed_step(MixedScene* s, unsigned nsteps, cudaStream_t q, const Phases& ph);
unsigned long long mixed_launches(MixedScene* s, unsigned nsteps);
unsigned long long mixed_rebuild_launches(MixedScene* s);
int mixed_rebuilds(MixedScene* s, unsigned long long* out, cudaStream_t q);
int mixed_eval_contacts(MixedScene* s, double* force, double* moment, cudaStream_t q);
int mixed_pair_list(MixedScene* s, unsigned cap_per_particle, unsigned* counts, unsigned* partners,
                    cudaStream_t q);
int mixed_counters(MixedScene* s, unsigned long long* out, cudaStream_t q);
int mixed_stats(MixedScene* s, unsigned long long* out, cudaStream_t q);
int mixed_set_tuning(MixedScene* s, const xd_tuning* t);
void mixed_get_tuning(const MixedScene* s, xd_tuning* t);
unsigned long long mixed_device_bytes(MixedScene* s);
int mixed_set_history(MixedScene* s, unsigned slots);
int mixed_set_kinematic(MixedScene* s, bool enable);
// Emitter support: the particles that take part in a step (slots [active,
// particle count) keep the staged ones in id order).  restore: first put every
// particle back in id order (when the emitter is set).
int mixed_set_active(MixedScene* s, unsigned active, bool restore, cudaStream_t q);
unsigned mixed_active(MixedScene* s);

// Batches: scenes advanced together by shared launches, each with the results
// it has when stepped alone.  Scenes with history or kinematic bodies are not
// batched.
struct MixedBatch;
int mixed_batch_create(MixedScene* const* scenes, unsigned count, MixedBatch** out);
void mixed_batch_destroy(MixedBatch* b);
int mixed_batch_step(MixedBatch* b, unsigned nsteps, cudaStream_t q);
int mixed_batch_set_timing(MixedBatch* b, bool enable);
void mixed_batch_kernel_times(MixedBatch* b, double ms[3], unsigned long long launches[3]);
int mixed_download_history(MixedScene* s, unsigned* keys, double* delta, unsigned long long* overflow,
                           cudaStream_t q);
int mixed_set_bodies(MixedScene* s, const xd_polygon_mass_info* pmi, cudaStream_t q);
int mixed_set_planes(MixedScene* s, const xd_plane_info* planes, cudaStream_t q);
int mixed_get_bodies(MixedScene* s, xd_polygon_mass_info* pmi, cudaStream_t q);

}  // namespace xd
