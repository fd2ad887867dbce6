// Scenes: device-resident DEM systems stepped in the reference's order
// (dem_simulation::oneStepAnalysis, dem_simulation.cpp:447-469).
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "xd_grid.cuh"
#include "xd_internal.cuh"
#include "xd_mixed.cuh"
#include "xd_physics64.cuh"

using namespace xd;

struct xd_scene {
    xd_scene_desc desc;
    Params P;
    unsigned np = 0, ntri = 0, nbodies = 0, nplanes = 0, ncell = 0;
    // state (reference layouts)
    double *pos = nullptr, *vel = nullptr, *acc = nullptr, *omega = nullptr, *alpha = nullptr;
    double *force = nullptr, *moment = nullptr, *mass = nullptr, *inertia = nullptr;
    // grid
    unsigned *hash = nullptr, *index = nullptr, *sorted = nullptr, *cstart = nullptr, *cend = nullptr;
    // FP64 form with a grid of its own for the particles (xd_scene_set_particle_grid): the
    // particles hashed, sorted and searched on Pp's cells, the triangles on the scene's grid
    bool split = false;
    Params Pp;
    unsigned ncell_p = 0;
    unsigned *pcstart = nullptr, *pcend = nullptr;
    // walls / mesh
    xd_plane_info* planes = nullptr;
    xd_contact_property* cp_planes = nullptr;
    xd_contact_property* cp_pp = nullptr;
    xd_polygon_info* poly = nullptr;
    double* sphere = nullptr;
    double* vlist = nullptr;
    xd_polygon_mass_info* pmi = nullptr;
    xd_contact_property* cp_poly = nullptr;
    // workspace
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    void* poly_scratch = nullptr;
    bool bodies_dirty = false;
    bool kinematic = false;   // bodies moved by their own vel and omega every step
    std::vector<void*> allocs;
    unsigned long long bytes = 0;   // device memory held by the FP64 form
    // phase timing
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> spans;
    double phase_ms[XD_SCENE_PHASES] = {};
    unsigned long long phase_n[XD_SCENE_PHASES] = {};
    cudaEvent_t pending[XD_SCENE_PHASES] = {};
    MixedScene* mixed = nullptr;
    // tangential-spring history (FP64 form; the mixed form keeps its own)
    unsigned hist_slots = 0;
    unsigned* hist_key = nullptr;
    double* hist_delta = nullptr;
    unsigned long long* hist_overflow = nullptr;
    // particle emitter: only the first `active` particles take part in a step
    unsigned active = 0;
    unsigned emit_period = 0;            // steps between creations; 0: none
    std::vector<unsigned> emit_groups;   // empty: one particle per creation
    unsigned emit_next = 0;              // next group to hand out
    unsigned long long emit_step = 0;    // steps run since the emitter was set
    // FP64 step graphs: 8 middle steps, one middle step, the last step of a
    // call; captured for `graphs_np` particles and the history setting
    cudaGraphExec_t graphs[3] = {};
    unsigned graphs_np = ~0u;
    bool use_graphs = true;
};

namespace {

// An NVTX range over a host call (profilers show the library's calls on the
// timeline; without a profiler attached it costs a function-pointer check).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

template <typename T>
int dalloc(xd_scene* s, T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) return XD_OK;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * count);
    if (e != cudaSuccess) return cuda_status(e, "scene allocation");
    s->allocs.push_back(q);
    s->bytes += sizeof(T) * count;
    *p = static_cast<T*>(q);
    return XD_OK;
}

int h2d(void* dst, const void* src, size_t bytes, cudaStream_t st)
{
    if (!src || !dst || bytes == 0) return XD_OK;
    return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), "scene upload");
}

int d2h(void* dst, const void* src, size_t bytes, cudaStream_t st)
{
    if (!src || !dst || bytes == 0) return XD_OK;
    return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st), "scene download");
}

void free_history(xd_scene* s)
{
    if (s->hist_key) cudaFree(s->hist_key);
    if (s->hist_delta) cudaFree(s->hist_delta);
    if (s->hist_overflow) cudaFree(s->hist_overflow);
    s->hist_key = nullptr;
    s->hist_delta = nullptr;
    s->hist_overflow = nullptr;
    s->hist_slots = 0;
}

HistTable history_of(xd_scene* s)
{
    HistTable h;
    h.key = s->hist_key;
    h.delta = s->hist_delta;
    h.slots = s->hist_slots;
    h.n = s->np;
    h.overflow = s->hist_overflow;
    return h;
}

void free_fp64_graphs(xd_scene* s)
{
    for (auto& g : s->graphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    s->graphs_np = ~0u;
}

void free_scene(xd_scene* s)
{
    free_fp64_graphs(s);
    free_history(s);
    if (s->mixed) mixed_destroy(s->mixed);
    s->mixed = nullptr;
    for (void* p : s->allocs) cudaFree(p);
    s->allocs.clear();
    for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
    s->ev_pool.clear();
}

cudaEvent_t next_event(xd_scene* s)
{
    if (s->ev_used == s->ev_pool.size()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        s->ev_pool.push_back(e);
    }
    return s->ev_pool[s->ev_used++];
}

// Phase hook for the mixed path.
void phase_hook(void* ctx, int phase, bool begin, cudaStream_t q)
{
    xd_scene* s = static_cast<xd_scene*>(ctx);
    if (!s->timing || phase < 0 || phase >= XD_SCENE_PHASES) return;
    cudaEvent_t e = next_event(s);
    if (!e) return;
    cudaEventRecord(e, q);
    if (begin) {
        s->pending[phase] = e;
    } else if (s->pending[phase]) {
        s->spans.push_back({ phase, { s->pending[phase], e } });
        s->pending[phase] = nullptr;
    }
}

// No hook while timing is off: the mixed path then runs its steps as CUDA
// graphs and decides re-binning on the device.
Phases phases_of(xd_scene* s)
{
    Phases p;
    p.ctx = s;
    p.fn = s->timing ? phase_hook : nullptr;
    return p;
}

// Records a [begin, end) event pair around one phase when timing is on.
struct PhaseSpan {
    xd_scene* s;
    int phase;
    cudaStream_t q;
    cudaEvent_t b = nullptr;
    PhaseSpan(xd_scene* s_, int ph, cudaStream_t q_) : s(s_), phase(ph), q(q_)
    {
        if (s->timing && (b = next_event(s))) cudaEventRecord(b, q);
    }
    ~PhaseSpan()
    {
        if (!b) return;
        cudaEvent_t e = next_event(s);
        if (!e) return;
        cudaEventRecord(e, q);
        s->spans.push_back({ phase, { b, e } });
    }
};

// Streams on which xd_scene_step_many runs its scenes side by side: kPoolStreams
// non-blocking streams per device, made on first use and kept for the
// process; the calls that use them take the mutex.  The device runs streams
// truly side by side only up to CUDA_DEVICE_MAX_CONNECTIONS hardware queues
// (8 unless the variable is set before the context is made; 32 at most).
constexpr int kPoolStreams = 32;
constexpr int kPoolDevices = 64;

struct StreamPool {
    cudaStream_t s[kPoolStreams] = {};
    cudaEvent_t done[kPoolStreams] = {};
    cudaEvent_t start = nullptr;
    bool ready = false;
};

std::mutex g_pool_mutex;
StreamPool g_pools[kPoolDevices];

int pool_of_current_device(StreamPool** out)
{
    int dev = 0;
    int st = cuda_status(cudaGetDevice(&dev), "step_many device");
    if (st != XD_OK) return st;
    if (dev < 0 || dev >= kPoolDevices) return set_error(XD_ERR_INVALID, "step_many: device ordinal out of range");
    StreamPool& p = g_pools[dev];
    if (!p.ready) {
        st = cuda_status(cudaEventCreateWithFlags(&p.start, cudaEventDisableTiming), "step_many events");
        for (int k = 0; k < kPoolStreams && st == XD_OK; ++k) {
            st = cuda_status(cudaStreamCreateWithFlags(&p.s[k], cudaStreamNonBlocking), "step_many streams");
            if (st == XD_OK)
                st = cuda_status(cudaEventCreateWithFlags(&p.done[k], cudaEventDisableTiming), "step_many events");
        }
        if (st != XD_OK) return st;
        p.ready = true;
    }
    *out = &p;
    return XD_OK;
}

}  // namespace

extern "C" {

int xd_scene_create(const xd_scene_desc* d, xd_scene** out)
{
    if (!d || !out) return set_error(XD_ERR_INVALID, "scene_create: null argument");
    *out = nullptr;
    if (d->mode != XD_MODE_FP64 && d->mode != XD_MODE_MIXED)
        return set_error(XD_ERR_INVALID, "scene_create: unknown mode %d", d->mode);
    if (d->mode == XD_MODE_MIXED) {
        xd_scene* s = new (std::nothrow) xd_scene();
        if (!s) return set_error(XD_ERR_NOMEM, "scene_create: host allocation");
        s->desc = *d;
        s->np = d->np;
        s->active = d->np;
        s->nplanes = d->nplanes;
        int st = mixed_create(*d, &s->mixed);
        if (st != XD_OK) {
            delete s;
            return st;
        }
        *out = s;
        return XD_OK;
    }
    const xd_device_parameters& h = d->params;
    unsigned gx = h.grid_size[0], gy = h.grid_size[1], gz = h.grid_size[2];
    if (!gx || !gy || !gz || (gx & (gx - 1)) || (gy & (gy - 1)) || (gz & (gz - 1)))
        return set_error(XD_ERR_INVALID, "scene_create: grid sizes must be powers of two");
    if ((unsigned long long)gx * gy * gz != h.ncell)
        return set_error(XD_ERR_INVALID, "scene_create: ncell must equal the grid size product");
    if (h.cell_size <= 0.0) return set_error(XD_ERR_INVALID, "scene_create: cell_size must be > 0");
    if (d->nplanes && (!d->planes || !d->cp_planes))
        return set_error(XD_ERR_INVALID, "scene_create: planes given without arrays");
    if (d->ntri && (!d->poly || !d->sphere || !d->vlist || !d->pmi || !d->cp_poly || !d->nbodies))
        return set_error(XD_ERR_INVALID, "scene_create: triangles given without mesh arrays");

    xd_scene* s = new (std::nothrow) xd_scene();
    if (!s) return set_error(XD_ERR_NOMEM, "scene_create: host allocation");
    s->desc = *d;
    s->desc.planes = nullptr;
    s->desc.cp_planes = nullptr;
    s->desc.poly = nullptr;
    s->desc.sphere = nullptr;
    s->desc.vlist = nullptr;
    s->desc.pmi = nullptr;
    s->desc.cp_poly = nullptr;
    s->np = d->np;
    s->active = d->np;
    s->ntri = d->ntri;
    {
        const char* ng = getenv("XDEM_NO_GRAPHS");
        s->use_graphs = !(ng && ng[0] && ng[0] != '0');
    }
    s->nbodies = d->ntri ? d->nbodies : 0;
    s->nplanes = d->nplanes;
    s->ncell = h.ncell;
    xd_device_parameters hp = h;
    hp.np = d->np;
    s->P = to_params(hp);

    const size_t n = (size_t)s->np, ng = (size_t)s->np + s->ntri;
    int st = XD_OK;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    A(dalloc(s, &s->pos, 4 * n));
    A(dalloc(s, &s->vel, 3 * n));
    A(dalloc(s, &s->acc, 3 * n));
    A(dalloc(s, &s->omega, 3 * n));
    A(dalloc(s, &s->alpha, 3 * n));
    A(dalloc(s, &s->force, 3 * n));
    A(dalloc(s, &s->moment, 3 * n));
    A(dalloc(s, &s->mass, n));
    A(dalloc(s, &s->inertia, n));
    A(dalloc(s, &s->hash, ng));
    A(dalloc(s, &s->index, ng));
    A(dalloc(s, &s->sorted, ng));
    A(dalloc(s, &s->cstart, s->ncell));
    A(dalloc(s, &s->cend, s->ncell));
    A(dalloc(s, &s->cp_pp, 1));
    A(dalloc(s, &s->planes, s->nplanes));
    A(dalloc(s, &s->cp_planes, s->nplanes));
    A(dalloc(s, &s->poly, s->ntri));
    A(dalloc(s, &s->sphere, 4 * (size_t)s->ntri));
    A(dalloc(s, &s->vlist, 9 * (size_t)s->ntri));
    A(dalloc(s, &s->pmi, s->nbodies));
    A(dalloc(s, &s->cp_poly, s->nbodies));
    s->scratch_bytes = reorder_scratch_bytes((unsigned)ng);
    char* scr = nullptr;
    A(dalloc(s, &scr, s->scratch_bytes));
    s->scratch = scr;
    size_t pb = polygon_scratch_bytes(s->np, s->nbodies);
    char* pscr = nullptr;
    if (s->ntri) A(dalloc(s, &pscr, pb ? pb : 256));
    s->poly_scratch = pscr;
    if (st != XD_OK) {
        free_scene(s);
        delete s;
        return st;
    }
    cudaStream_t q = 0;
    A(h2d(s->cp_pp, &d->cp_pp, sizeof(xd_contact_property), q));
    A(h2d(s->planes, d->planes, sizeof(xd_plane_info) * s->nplanes, q));
    A(h2d(s->cp_planes, d->cp_planes, sizeof(xd_contact_property) * s->nplanes, q));
    A(h2d(s->poly, d->poly, sizeof(xd_polygon_info) * s->ntri, q));
    A(h2d(s->sphere, d->sphere, sizeof(double) * 4 * s->ntri, q));
    A(h2d(s->vlist, d->vlist, sizeof(double) * 9 * s->ntri, q));
    A(h2d(s->pmi, d->pmi, sizeof(xd_polygon_mass_info) * s->nbodies, q));
    A(h2d(s->cp_poly, d->cp_poly, sizeof(xd_contact_property) * s->nbodies, q));
    if (st == XD_OK) A(cuda_status(cudaStreamSynchronize(q), "scene_create upload"));
    if (st != XD_OK) {
        free_scene(s);
        delete s;
        return st;
    }
    *out = s;
    return XD_OK;
}

int xd_scene_destroy(xd_scene* s)
{
    if (!s) return XD_OK;
    cudaError_t e = cudaDeviceSynchronize();
    free_scene(s);
    delete s;
    return cuda_status(e, "scene_destroy");
}

static int scene_upload(xd_scene* s, const double* pos, const double* vel, const double* acc,
                        const double* omega, const double* alpha, const double* force,
                    const double* moment, const double* mass, const double* inertia, void* stream, bool sync)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_upload: null scene");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    if (s->mixed) return mixed_upload(s->mixed, pos, vel, acc, omega, alpha, mass, inertia, q, sync);
    size_t n = s->np;
    int st = XD_OK;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    A(h2d(s->pos, pos, sizeof(double) * 4 * n, q));
    A(h2d(s->vel, vel, sizeof(double) * 3 * n, q));
    A(h2d(s->acc, acc, sizeof(double) * 3 * n, q));
    A(h2d(s->omega, omega, sizeof(double) * 3 * n, q));
    A(h2d(s->alpha, alpha, sizeof(double) * 3 * n, q));
    A(h2d(s->force, force, sizeof(double) * 3 * n, q));
    A(h2d(s->moment, moment, sizeof(double) * 3 * n, q));
    A(h2d(s->mass, mass, sizeof(double) * n, q));
    A(h2d(s->inertia, inertia, sizeof(double) * n, q));
    if (st == XD_OK && sync) A(cuda_status(cudaStreamSynchronize(q), "scene_upload"));
    return st;
}

int xd_scene_upload(xd_scene* s, const double* pos, const double* vel, const double* acc, const double* omega,
                    const double* alpha, const double* force, const double* moment, const double* mass,
                    const double* inertia, void* stream)
{
    return scene_upload(s, pos, vel, acc, omega, alpha, force, moment, mass, inertia, stream, true);
}

int xd_scene_upload_async(xd_scene* s, const double* pos, const double* vel, const double* acc, const double* omega,
                          const double* alpha, const double* force, const double* moment, const double* mass,
                          const double* inertia, void* stream)
{
    return scene_upload(s, pos, vel, acc, omega, alpha, force, moment, mass, inertia, stream, false);
}

static int scene_download(xd_scene* s, double* pos, double* vel, double* acc, double* omega,
                      double* alpha, double* force, double* moment, void* stream, bool sync)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_download: null scene");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    if (s->mixed) return mixed_download(s->mixed, pos, vel, acc, omega, alpha, force, moment, q, sync);
    size_t n = s->np;
    int st = XD_OK;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    A(d2h(pos, s->pos, sizeof(double) * 4 * n, q));
    A(d2h(vel, s->vel, sizeof(double) * 3 * n, q));
    A(d2h(acc, s->acc, sizeof(double) * 3 * n, q));
    A(d2h(omega, s->omega, sizeof(double) * 3 * n, q));
    A(d2h(alpha, s->alpha, sizeof(double) * 3 * n, q));
    A(d2h(force, s->force, sizeof(double) * 3 * n, q));
    A(d2h(moment, s->moment, sizeof(double) * 3 * n, q));
    if (st == XD_OK && sync) A(cuda_status(cudaStreamSynchronize(q), "scene_download"));
    return st;
}

int xd_scene_download(xd_scene* s, double* pos, double* vel, double* acc, double* omega, double* alpha,
                      double* force, double* moment, void* stream)
{
    return scene_download(s, pos, vel, acc, omega, alpha, force, moment, stream, true);
}

int xd_scene_download_async(xd_scene* s, double* pos, double* vel, double* acc, double* omega, double* alpha,
                            double* force, double* moment, void* stream)
{
    return scene_download(s, pos, vel, acc, omega, alpha, force, moment, stream, false);
}

int xd_scene_device_state(xd_scene* s, double** pos, double** vel, double** acc, double** omega,
                          double** alpha, double** force, double** moment, double** mass,
                          double** inertia)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_device_state: null scene");
    if (s->mixed) return set_error(XD_ERR_STATE, "scene_device_state: not available in mixed mode (state is kept in cell order)");
    if (pos) *pos = s->pos;
    if (vel) *vel = s->vel;
    if (acc) *acc = s->acc;
    if (omega) *omega = s->omega;
    if (alpha) *alpha = s->alpha;
    if (force) *force = s->force;
    if (moment) *moment = s->moment;
    if (mass) *mass = s->mass;
    if (inertia) *inertia = s->inertia;
    return XD_OK;
}

int xd_scene_device_grid(xd_scene* s, unsigned** hash, unsigned** index, unsigned** sorted,
                         unsigned** cstart, unsigned** cend)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_device_grid: null scene");
    if (s->mixed) return set_error(XD_ERR_STATE, "scene_device_grid: not available in mixed mode (state is kept in cell order)");
    if (hash) *hash = s->hash;
    if (index) *index = s->index;
    if (sorted) *sorted = s->sorted;
    if (cstart) *cstart = s->cstart;
    if (cend) *cend = s->cend;
    return XD_OK;
}

int xd_scene_download_grid(xd_scene* s, unsigned* hash, unsigned* index, unsigned* sorted,
                           unsigned* cstart, unsigned* cend, void* stream)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_download_grid: null scene");
    if (s->mixed) return set_error(XD_ERR_STATE, "scene_download_grid: not available in mixed mode (state is kept in cell order)");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    size_t ng = (size_t)s->np + s->ntri;
    int st = XD_OK;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    A(d2h(hash, s->hash, sizeof(unsigned) * ng, q));
    A(d2h(index, s->index, sizeof(unsigned) * ng, q));
    A(d2h(sorted, s->sorted, sizeof(unsigned) * ng, q));
    A(d2h(cstart, s->cstart, sizeof(unsigned) * s->ncell, q));
    A(d2h(cend, s->cend, sizeof(unsigned) * s->ncell, q));
    if (st == XD_OK) A(cuda_status(cudaStreamSynchronize(q), "scene_download_grid"));
    return st;
}

int xd_scene_set_bodies(xd_scene* s, const xd_polygon_mass_info* pmi, void* stream)
{
    if (!s || !pmi) return set_error(XD_ERR_INVALID, "scene_set_bodies: null argument");
    if (s->mixed) return mixed_set_bodies(s->mixed, pmi, static_cast<cudaStream_t>(stream));
    if (!s->nbodies) return set_error(XD_ERR_STATE, "scene_set_bodies: scene has no polygon bodies");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    int st = h2d(s->pmi, pmi, sizeof(xd_polygon_mass_info) * s->nbodies, q);
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_set_bodies");
    s->bodies_dirty = true;
    return st;
}

int xd_scene_set_planes(xd_scene* s, const xd_plane_info* planes, void* stream)
{
    if (!s || !planes) return set_error(XD_ERR_INVALID, "scene_set_planes: null argument");
    if (!s->nplanes) return set_error(XD_ERR_STATE, "scene_set_planes: scene has no planes");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    if (s->mixed) return mixed_set_planes(s->mixed, planes, q);
    int st = h2d(s->planes, planes, sizeof(xd_plane_info) * s->nplanes, q);
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_set_planes");
    return st;
}

int xd_scene_get_bodies(xd_scene* s, xd_polygon_mass_info* pmi, void* stream)
{
    if (!s || !pmi) return set_error(XD_ERR_INVALID, "scene_get_bodies: null argument");
    if (s->mixed) return mixed_get_bodies(s->mixed, pmi, static_cast<cudaStream_t>(stream));
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    int st = d2h(pmi, s->pmi, sizeof(xd_polygon_mass_info) * s->nbodies, q);
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_get_bodies");
    return st;
}

int xd_scene_eval_contacts(xd_scene* s, double* force, double* moment, void* stream)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_eval_contacts: null scene");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    if (s->mixed) return mixed_eval_contacts(s->mixed, force, moment, q);
    // FP64 mode: contacts added onto zeroed force/moment copies (rows of
    // particles not emitted yet stay zero)
    const size_t n = s->np, na = s->active, ng = na + s->ntri;
    double *f0 = nullptr, *m0 = nullptr;
    int st = cuda_status(cudaMalloc(&f0, sizeof(double) * 6 * (n ? n : 1)), "scene_eval_contacts");
    if (st != XD_OK) return st;
    m0 = f0 + 3 * n;
    auto A = [&](int r) { if (st == XD_OK) st = r; };
    A(cuda_status(cudaMemsetAsync(f0, 0, sizeof(double) * 6 * n, q), "scene_eval_contacts"));
    Params P = s->P;
    P.np = (unsigned)na;
    if (na) {
        A(launch_hash(P, s->hash, s->index, s->pos, P.np, 0, q));
        if (s->ntri) A(launch_hash(P, s->hash, s->index, s->sphere, s->ntri, P.np, q));
        if (st == XD_OK)
            A(reorder_and_find_cell_start(s->hash, s->index, s->cstart, s->cend, s->sorted, (unsigned)ng,
                                          s->ncell, s->scratch, q, false));
        if (st == XD_OK)
            A(launch_p2p(P, s->pos, s->vel, s->omega, f0, m0, s->mass, s->sorted, s->cstart, s->cend,
                         s->cp_pp, P.np, q));
        if (st == XD_OK && s->nplanes)
            A(launch_planes(P, s->planes, s->cp_planes, 1, s->nplanes, s->pos, s->vel, s->omega, f0, m0,
                            s->mass, P.np, q));
    }
    if (st == XD_OK && s->ntri && na) {
        // the reaction on the bodies is not part of this diagnostic: work on a copy
        xd_polygon_mass_info* tmp = nullptr;
        A(cuda_status(cudaMalloc(&tmp, sizeof(xd_polygon_mass_info) * s->nbodies), "scene_eval_contacts"));
        if (st == XD_OK) {
            A(cuda_status(cudaMemcpyAsync(tmp, s->pmi, sizeof(xd_polygon_mass_info) * s->nbodies,
                                          cudaMemcpyDeviceToDevice, q), "scene_eval_contacts"));
            A(launch_polygon(P, s->poly, tmp, s->pos, s->vel, s->omega, f0, m0, s->mass, s->sorted,
                             s->cstart, s->cend, s->cp_poly, s->nbodies, s->poly_scratch, q));
            cudaStreamSynchronize(q);
            cudaFree(tmp);
        }
    }
    if (st == XD_OK && force) A(d2h(force, f0, sizeof(double) * 3 * n, q));
    if (st == XD_OK && moment) A(d2h(moment, m0, sizeof(double) * 3 * n, q));
    if (st == XD_OK) A(cuda_status(cudaStreamSynchronize(q), "scene_eval_contacts"));
    cudaFree(f0);
    return st;
}

int xd_scene_pair_list(xd_scene* s, unsigned cap, unsigned* counts, unsigned* partners, void* stream)
{
    if (!s || !counts || !partners) return set_error(XD_ERR_INVALID, "scene_pair_list: null argument");
    if (!s->mixed) return set_error(XD_ERR_STATE, "scene_pair_list: mixed mode only (use xd_pair_list)");
    return mixed_pair_list(s->mixed, cap, counts, partners, static_cast<cudaStream_t>(stream));
}

int xd_scene_counters(xd_scene* s, unsigned long long out[4], void* stream)
{
    if (!s || !out) return set_error(XD_ERR_INVALID, "scene_counters: null argument");
    if (!s->mixed) {
        for (int i = 0; i < 4; ++i) out[i] = 0;
        return XD_OK;
    }
    return mixed_counters(s->mixed, out, static_cast<cudaStream_t>(stream));
}

int xd_scene_stats(xd_scene* s, unsigned long long* out, unsigned count, void* stream)
{
    if (!s || (!out && count)) return set_error(XD_ERR_INVALID, "scene_stats: null argument");
    if (count > XD_STATS_COUNT) return set_error(XD_ERR_INVALID, "scene_stats: at most %d values", XD_STATS_COUNT);
    unsigned long long v[XD_STATS_COUNT] = {};
    if (s->mixed) {
        const int st = mixed_stats(s->mixed, v, static_cast<cudaStream_t>(stream));
        if (st != XD_OK) return st;
    }
    for (unsigned i = 0; i < count; ++i) out[i] = v[i];
    return XD_OK;
}

int xd_scene_set_tuning(xd_scene* s, const xd_tuning* t)
{
    if (!s || !t) return set_error(XD_ERR_INVALID, "scene_set_tuning: null argument");
    if (!s->mixed) return set_error(XD_ERR_STATE, "scene_set_tuning: an FP64 scene has no tunable parameters");
    return mixed_set_tuning(s->mixed, t);
}

int xd_scene_get_tuning(xd_scene* s, xd_tuning* t)
{
    if (!s || !t) return set_error(XD_ERR_INVALID, "scene_get_tuning: null argument");
    if (!s->mixed) return set_error(XD_ERR_STATE, "scene_get_tuning: an FP64 scene has no tunable parameters");
    mixed_get_tuning(s->mixed, t);
    return XD_OK;
}

int xd_scene_rebuilds(xd_scene* s, unsigned long long* count, unsigned long long* launches_each,
                      void* stream)
{
    if (!s || !count || !launches_each) return set_error(XD_ERR_INVALID, "scene_rebuilds: null argument");
    if (!s->mixed) {
        *count = 0;
        *launches_each = 0;
        return XD_OK;
    }
    *launches_each = mixed_rebuild_launches(s->mixed);
    return mixed_rebuilds(s->mixed, count, static_cast<cudaStream_t>(stream));
}

int xd_scene_set_timing(xd_scene* s, int enable)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_set_timing: null scene");
    cudaError_t e = cudaDeviceSynchronize();
    s->timing = enable != 0;
    s->spans.clear();
    s->ev_used = 0;
    for (int i = 0; i < XD_SCENE_PHASES; ++i) {
        s->phase_ms[i] = 0.0;
        s->phase_n[i] = 0;
        s->pending[i] = nullptr;
    }
    return cuda_status(e, "scene_set_timing");
}

int xd_scene_phase_times(xd_scene* s, double* ms, unsigned long long* launches)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_phase_times: null scene");
    for (auto& sp : s->spans) {
        cudaError_t e = cudaEventSynchronize(sp.second.second);
        if (e != cudaSuccess) return cuda_status(e, "scene_phase_times");
        float t = 0.f;
        e = cudaEventElapsedTime(&t, sp.second.first, sp.second.second);
        if (e != cudaSuccess) return cuda_status(e, "scene_phase_times");
        s->phase_ms[sp.first] += t;
        s->phase_n[sp.first] += 1;
    }
    s->spans.clear();
    s->ev_used = 0;
    for (int i = 0; i < XD_SCENE_PHASES; ++i) {
        if (ms) ms[i] = s->phase_ms[i];
        if (launches) launches[i] = s->phase_n[i];
    }
    return XD_OK;
}

unsigned long long xd_scene_launches(xd_scene* s, unsigned nsteps)
{
    if (!s || nsteps == 0) return 0;
    if (s->mixed) return mixed_launches(s->mixed, nsteps);
    unsigned ng = s->np + s->ntri;
    unsigned passes = (key_bits_for(s->ncell) + 7) / 8;
    unsigned long long per = 0;
    per += 1 + (s->ntri ? 1 : 0);                 // hash (+ triangle spheres)
    per += ng > 1 ? 5ull * passes : 0;            // radix sort
    per += 2;                                     // fill + cell bounds
    per += 1;                                     // particle-particle
    per += s->nplanes ? 1 : 0;                    // planes
    per += s->ntri ? 2 : 0;                       // triangles + reaction
    per += 1;                                     // VV velocity(+position)
    unsigned long long total = per * nsteps;
    if (s->bodies_dirty && s->ntri) total += 1;   // mesh update
    total += 1;                                   // first VV position
    // kinematic bodies: pose and mesh before every step; the step boundary
    // is then velocity and position as two launches
    if (s->kinematic && s->ntri) total += 2ull * nsteps + (nsteps - 1);
    return total;
}

namespace {

// nsteps whole FP64 steps over the active particles (no emission inside).
int fp64_steps(xd_scene* s, unsigned nsteps, cudaStream_t q)
{
    Params P = s->P;
    P.np = s->active;
    const unsigned np = s->active, ng = np + s->ntri;
    const HistTable ht = history_of(s);
    const HistTable* hp = s->hist_slots ? &ht : nullptr;
    int st = XD_OK;
    if (s->bodies_dirty && s->ntri) {
        st = launch_update_polygon(s->pmi, s->vlist, s->sphere, s->poly, s->ntri, q);
        if (st != XD_OK) return st;
        s->bodies_dirty = false;
    }
    const bool kin = s->kinematic && s->ntri;
    auto move_bodies = [&]() {
        int r = launch_body_advance(s->pmi, s->nbodies, P.dt, q);
        if (r == XD_OK) r = launch_update_polygon(s->pmi, s->vlist, s->sphere, s->poly, s->ntri, q);
        return r;
    };
    if (np == 0) {   // nothing emitted yet: only the prescribed body motion
        for (unsigned t = 0; t < nsteps && kin && st == XD_OK; ++t) st = move_bodies();
        return st;
    }
    if (kin) st = move_bodies();
    if (st != XD_OK) return st;
    // VV position of the first step (later ones are fused into the velocity pass)
    {
        PhaseSpan ps(s, 0, q);
        st = launch_vv_position(P, s->pos, s->vel, s->acc, np, q);
    }
    if (st != XD_OK) return st;
    // one step: grid, contacts, and the velocity update, fused with the next
    // step's position update unless `last`
    Params Pp = s->Pp;
    Pp.np = np;
    // the particles' grid: the scene's, or their own (then the triangles'
    // hashes, sorted order and cell ranges sit after the particles' in
    // hash/index/sorted and in cstart/cend of the scene's grid)
    const Params& PG = s->split ? Pp : P;
    unsigned* const gcs = s->split ? s->pcstart : s->cstart;
    unsigned* const gce = s->split ? s->pcend : s->cend;
    auto one_step = [&](bool last, cudaStream_t qq) {
        int r = XD_OK;
        {
            PhaseSpan ps(s, 1, qq);
            r = launch_hash(PG, s->hash, s->index, s->pos, np, 0, qq);
            if (r == XD_OK && s->ntri) r = launch_hash(P, s->hash, s->index, s->sphere, s->ntri, np, qq);
        }
        if (r == XD_OK) {
            PhaseSpan ps(s, 2, qq);
            if (!s->split) {
                r = reorder_and_find_cell_start(s->hash, s->index, s->cstart, s->cend, s->sorted, ng, s->ncell,
                                                s->scratch, qq, false);
            } else {
                r = reorder_and_find_cell_start(s->hash, s->index, s->pcstart, s->pcend, s->sorted, np,
                                                s->ncell_p, s->scratch, qq, false);
                if (r == XD_OK && s->ntri)
                    r = reorder_and_find_cell_start(s->hash + np, s->index + np, s->cstart, s->cend,
                                                    s->sorted + np, s->ntri, s->ncell, s->scratch, qq, false);
            }
        }
        if (r == XD_OK) {
            PhaseSpan ps(s, 3, qq);
            r = launch_p2p(PG, s->pos, s->vel, s->omega, s->force, s->moment, s->mass, s->sorted, gcs, gce,
                           s->cp_pp, np, qq, hp);
        }
        if (r == XD_OK && s->nplanes) {
            PhaseSpan ps(s, 4, qq);
            r = launch_planes(P, s->planes, s->cp_planes, 1, s->nplanes, s->pos, s->vel, s->omega, s->force,
                              s->moment, s->mass, np, qq, hp);
        }
        if (r == XD_OK && s->ntri) {
            PhaseSpan ps(s, 5, qq);
            r = launch_polygon(P, s->poly, s->pmi, s->pos, s->vel, s->omega, s->force, s->moment, s->mass,
                               s->split ? s->sorted + np : s->sorted, s->cstart, s->cend, s->cp_poly,
                               s->nbodies, s->poly_scratch, qq, hp);
        }
        if (r == XD_OK) {
            PhaseSpan ps(s, 0, qq);
            if (!last && !kin) {
                r = launch_vv_velocity_position(P, s->pos, s->vel, s->acc, s->omega, s->alpha, s->force,
                                                s->moment, s->mass, s->inertia, np, qq);
            } else {
                r = launch_vv_velocity(P, s->vel, s->acc, s->omega, s->alpha, s->force, s->moment, s->mass,
                                       s->inertia, np, qq);
                // moving bodies come before the next step's position update
                if (r == XD_OK && !last) r = move_bodies();
                if (r == XD_OK && !last) r = launch_vv_position(P, s->pos, s->vel, s->acc, np, qq);
            }
        }
        return r;
    };
    if (!s->use_graphs || s->timing || kin || nsteps < 4) {
        for (unsigned t = 0; t < nsteps && st == XD_OK; ++t) st = one_step(t + 1 == nsteps, q);
        return st;
    }
    // the steps as CUDA graphs (no host decision inside a step): captured at
    // the first call and whenever the particle count changed
    if (s->graphs_np != np) {
        free_fp64_graphs(s);
        for (int kind = 0; kind < 3 && st == XD_OK; ++kind) {
            cudaStream_t cs = nullptr;
            st = cuda_status(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "scene graph stream");
            if (st != XD_OK) break;
            st = cuda_status(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "scene graph capture");
            const unsigned count = kind == 0 ? 8u : 1u;
            for (unsigned k = 0; k < count && st == XD_OK; ++k) st = one_step(kind == 2, cs);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(cs, &g);
            if (st == XD_OK) st = cuda_status(e, "scene graph capture");
            if (st == XD_OK) st = cuda_status(cudaGraphInstantiate(&s->graphs[kind], g, 0), "scene graph instantiate");
            if (g) cudaGraphDestroy(g);
            cudaStreamDestroy(cs);
        }
        if (st != XD_OK) {
            free_fp64_graphs(s);
            return st;
        }
        s->graphs_np = np;
    }
    unsigned mid = nsteps - 1;
    for (; mid >= 8 && st == XD_OK; mid -= 8) st = cuda_status(cudaGraphLaunch(s->graphs[0], q), "scene graph launch");
    for (; mid > 0 && st == XD_OK; --mid) st = cuda_status(cudaGraphLaunch(s->graphs[1], q), "scene graph launch");
    if (st == XD_OK) st = cuda_status(cudaGraphLaunch(s->graphs[2], q), "scene graph launch");
    if (st != XD_OK) return st;
    return XD_OK;
}

// Emission before the scene's next step, if one is due (particleManager's
// groups handed out every emit_period steps, dem_simulation.cpp:449-450).
int emit_before_step(xd_scene* s, cudaStream_t q)
{
    const unsigned long long k = s->emit_step + 1;
    if (!s->emit_period || (k - 1) % s->emit_period != 0 || s->active >= s->np) return XD_OK;
    unsigned add = 1;
    if (!s->emit_groups.empty()) add = s->emit_next < s->emit_groups.size() ? s->emit_groups[s->emit_next++] : 0;
    const unsigned next = add > s->np - s->active ? s->np : s->active + add;
    if (next == s->active) return XD_OK;
    s->active = next;
    return s->mixed ? mixed_set_active(s->mixed, next, false, q) : XD_OK;
}

// Steps from the scene's next step to the next emission (all of `left` when
// none can come).
unsigned steps_to_emission(const xd_scene* s, unsigned left)
{
    const bool more = s->emit_period && s->active < s->np &&
                      (s->emit_groups.empty() || s->emit_next < s->emit_groups.size());
    if (!more) return left;
    const unsigned long long k = s->emit_step + 1;   // the next step, 1-based
    const unsigned long long to = s->emit_period - (k - 1) % s->emit_period;
    return (unsigned)std::min<unsigned long long>(left, to);
}

}  // namespace

int xd_scene_step(xd_scene* s, unsigned nsteps, int check, void* stream)
{
    NvtxRange range("xd_scene_step");
    if (!s) return set_error(XD_ERR_INVALID, "scene_step: null scene");
    if (nsteps == 0) return XD_OK;
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    // A call is split at the steps that emit particles: each piece ends with
    // the velocity update of the particles that took part, and the next one
    // starts with the position update of the grown set, the reference's order.
    int st = XD_OK;
    for (unsigned left = nsteps; left && st == XD_OK;) {
        st = emit_before_step(s, q);
        if (st != XD_OK) break;
        const unsigned run = steps_to_emission(s, left);
        st = s->mixed ? mixed_step(s->mixed, run, q, phases_of(s)) : fp64_steps(s, run, q);
        s->emit_step += run;
        left -= run;
    }
    if (st != XD_OK) return st;
    if (s->mixed) {
        if (check) st = cuda_status(cudaStreamSynchronize(q), "scene_step");
        return st;
    }
    if (check) {
        unsigned herr = 0;
        cudaError_t e = cudaMemcpyAsync(&herr, s->scratch, sizeof(unsigned), cudaMemcpyDeviceToHost, q);
        if (e == cudaSuccess) e = cudaStreamSynchronize(q);
        if (e != cudaSuccess) return cuda_status(e, "scene_step check");
        if (herr) return set_error(XD_ERR_INVALID, "scene_step: a hash value was >= ncell");
    }
    return XD_OK;
}

int xd_scene_set_kinematic_bodies(xd_scene* s, int enable)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_set_kinematic_bodies: null scene");
    if (s->mixed) return mixed_set_kinematic(s->mixed, enable != 0);
    if (enable && !s->nbodies) return set_error(XD_ERR_STATE, "scene_set_kinematic_bodies: no polygon bodies");
    s->kinematic = enable != 0;
    return XD_OK;
}

int xd_scene_set_emitter(xd_scene* s, unsigned active, unsigned period, const unsigned* groups, unsigned ngroups,
                         void* stream)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_set_emitter: null scene");
    if (active > s->np) return set_error(XD_ERR_INVALID, "scene_set_emitter: active %u above the %u particles", active, s->np);
    if (ngroups && !groups) return set_error(XD_ERR_INVALID, "scene_set_emitter: groups is null");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    if (s->mixed) {
        int st = mixed_set_active(s->mixed, active, true, q);
        if (st != XD_OK) return st;
    }
    s->active = active;
    s->emit_period = period;
    s->emit_groups.assign(groups, groups + ngroups);
    s->emit_next = 0;
    s->emit_step = 0;
    return XD_OK;
}

int xd_scene_active(xd_scene* s, unsigned* active)
{
    if (!s || !active) return set_error(XD_ERR_INVALID, "scene_active: null argument");
    *active = s->active;
    return XD_OK;
}

int xd_scene_set_particle_grid(xd_scene* s, const unsigned grid[3], double cell_size, const double origin[3])
{
    if (!s || !grid || !origin) return set_error(XD_ERR_INVALID, "scene_set_particle_grid: null argument");
    if (s->mixed) return set_error(XD_ERR_STATE, "scene_set_particle_grid: FP64 scenes only");
    for (int a = 0; a < 3; ++a)
        if (grid[a] < 2 || grid[a] > 4096 || (grid[a] & (grid[a] - 1u)))
            return set_error(XD_ERR_INVALID, "scene_set_particle_grid: dimension %u not a power of two in [2, 4096]",
                             grid[a]);
    const unsigned long long nc = (unsigned long long)grid[0] * grid[1] * grid[2];
    if (nc > (1ull << 28)) return set_error(XD_ERR_INVALID, "scene_set_particle_grid: %llu cells", nc);
    if (!(cell_size > 0.0)) return set_error(XD_ERR_INVALID, "scene_set_particle_grid: cell size %g", cell_size);
    cudaDeviceSynchronize();   // the step graphs hold the grid arrays: replaced after what is queued
    free_fp64_graphs(s);
    s->graphs_np = ~0u;
    if (nc > s->ncell_p) {
        unsigned *a = nullptr, *b = nullptr;
        int st = dalloc(s, &a, nc);
        if (st == XD_OK) st = dalloc(s, &b, nc);
        if (st != XD_OK) return st;
        s->pcstart = a;
        s->pcend = b;
    }
    s->ncell_p = (unsigned)nc;
    s->Pp = s->P;
    s->Pp.gx = grid[0];
    s->Pp.gy = grid[1];
    s->Pp.gz = grid[2];
    s->Pp.ncell = (unsigned)nc;
    s->Pp.cs = cell_size;
    for (int a = 0; a < 3; ++a) s->Pp.wo[a] = origin[a];
    s->split = true;
    return XD_OK;
}

int xd_scene_set_tangential_history(xd_scene* s, unsigned slots)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_set_tangential_history: null scene");
    if (slots > kHistMaxSlots)
        return set_error(XD_ERR_INVALID, "scene_set_tangential_history: at most %u contacts per particle",
                         kHistMaxSlots);
    if (s->mixed) return mixed_set_history(s->mixed, slots);
    cudaDeviceSynchronize();   // the step graphs hold the tables: replaced after what is queued
    free_fp64_graphs(s);
    free_history(s);
    if (slots == 0 || s->np == 0) return XD_OK;
    const size_t e = (size_t)slots * s->np;
    int st = cuda_status(cudaMalloc(&s->hist_key, sizeof(unsigned) * e), "tangential history");
    if (st == XD_OK) st = cuda_status(cudaMalloc(&s->hist_delta, sizeof(double) * 3 * e), "tangential history");
    if (st == XD_OK) st = cuda_status(cudaMalloc(&s->hist_overflow, sizeof(unsigned long long)), "tangential history");
    if (st == XD_OK) st = cuda_status(cudaMemset(s->hist_key, 0xff, sizeof(unsigned) * e), "tangential history");
    if (st == XD_OK) st = cuda_status(cudaMemset(s->hist_delta, 0, sizeof(double) * 3 * e), "tangential history");
    if (st == XD_OK) st = cuda_status(cudaMemset(s->hist_overflow, 0, sizeof(unsigned long long)), "tangential history");
    if (st != XD_OK) {
        free_history(s);
        return st;
    }
    s->hist_slots = slots;
    return XD_OK;
}

int xd_scene_download_history(xd_scene* s, unsigned* keys, double* delta, unsigned long long* overflow,
                              void* stream)
{
    if (!s) return set_error(XD_ERR_INVALID, "scene_download_history: null scene");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    if (s->mixed) return mixed_download_history(s->mixed, keys, delta, overflow, q);
    if (!s->hist_slots) return set_error(XD_ERR_STATE, "scene_download_history: history is off");
    const size_t e = (size_t)s->hist_slots * s->np;
    int st = XD_OK;
    if (keys) st = d2h(keys, s->hist_key, sizeof(unsigned) * e, q);
    if (st == XD_OK && delta) st = d2h(delta, s->hist_delta, sizeof(double) * 3 * e, q);
    if (st == XD_OK && overflow) st = d2h(overflow, s->hist_overflow, sizeof(unsigned long long), q);
    if (st == XD_OK) st = cuda_status(cudaStreamSynchronize(q), "scene_download_history");
    return st;
}

int xd_scene_step_many(xd_scene* const* scenes, const unsigned* nsteps, unsigned count, int check, void* stream)
{
    NvtxRange range("xd_scene_step_many");
    if (count == 0) return XD_OK;
    if (!scenes || !nsteps) return set_error(XD_ERR_INVALID, "scene_step_many: null array");
    for (unsigned i = 0; i < count; ++i)
        if (!scenes[i]) return set_error(XD_ERR_INVALID, "scene_step_many: null scene");
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    StreamPool* p = nullptr;
    int st = pool_of_current_device(&p);
    if (st != XD_OK) return st;
    // the pool streams start after the work already queued on `stream`
    st = cuda_status(cudaEventRecord(p->start, q), "scene_step_many");
    const unsigned used = count < (unsigned)kPoolStreams ? count : (unsigned)kPoolStreams;
    for (unsigned k = 0; k < used && st == XD_OK; ++k)
        st = cuda_status(cudaStreamWaitEvent(p->s[k], p->start, 0), "scene_step_many");
    for (unsigned i = 0; i < count && st == XD_OK; ++i)
        st = xd_scene_step(scenes[i], nsteps[i], 0, p->s[i % kPoolStreams]);
    // `stream` continues after every scene, also when a launch failed
    for (unsigned k = 0; k < used; ++k) {
        int e = cuda_status(cudaEventRecord(p->done[k], p->s[k]), "scene_step_many");
        if (e == XD_OK) e = cuda_status(cudaStreamWaitEvent(q, p->done[k], 0), "scene_step_many");
        if (st == XD_OK) st = e;
    }
    if (st == XD_OK && check) st = cuda_status(cudaStreamSynchronize(q), "scene_step_many");
    return st;
}

struct xd_batch {
    MixedBatch* mixed = nullptr;
    std::vector<xd_scene*> scenes;
};

int xd_batch_create(xd_scene* const* scenes, unsigned count, xd_batch** out)
{
    if (!scenes || !out) return set_error(XD_ERR_INVALID, "batch_create: null argument");
    *out = nullptr;
    std::vector<MixedScene*> ms(count);
    for (unsigned k = 0; k < count; ++k) {
        xd_scene* s = scenes[k];
        if (!s) return set_error(XD_ERR_INVALID, "batch_create: null scene %u", k);
        if (!s->mixed) return set_error(XD_ERR_STATE, "batch_create: scene %u is not in the mixed form", k);
        if (s->emit_period || s->active != s->np)
            return set_error(XD_ERR_STATE, "batch_create: scene %u has an emitter", k);
        ms[k] = s->mixed;
    }
    MixedBatch* b = nullptr;
    int st = mixed_batch_create(ms.data(), count, &b);
    if (st != XD_OK) return st;
    xd_batch* h = new (std::nothrow) xd_batch();
    if (!h) {
        mixed_batch_destroy(b);
        return set_error(XD_ERR_NOMEM, "batch_create: host allocation");
    }
    h->mixed = b;
    h->scenes.assign(scenes, scenes + count);
    *out = h;
    return XD_OK;
}

int xd_batch_step(xd_batch* b, unsigned nsteps, int check, void* stream)
{
    NvtxRange range("xd_batch_step");
    if (!b) return set_error(XD_ERR_INVALID, "batch_step: null batch");
    for (size_t k = 0; k < b->scenes.size(); ++k)
        if (b->scenes[k]->emit_period || b->scenes[k]->active != b->scenes[k]->np)
            return set_error(XD_ERR_STATE, "batch_step: scene %u has an emitter", (unsigned)k);
    cudaStream_t q = static_cast<cudaStream_t>(stream);
    int st = mixed_batch_step(b->mixed, nsteps, q);
    if (st == XD_OK && check) st = cuda_status(cudaStreamSynchronize(q), "batch_step");
    return st;
}

int xd_batch_set_timing(xd_batch* b, int enable)
{
    if (!b) return set_error(XD_ERR_INVALID, "batch_set_timing: null batch");
    return mixed_batch_set_timing(b->mixed, enable != 0);
}

int xd_batch_kernel_times(xd_batch* b, double ms[3], unsigned long long launches[3])
{
    if (!b || !ms || !launches) return set_error(XD_ERR_INVALID, "batch_kernel_times: null argument");
    mixed_batch_kernel_times(b->mixed, ms, launches);
    return XD_OK;
}

int xd_batch_destroy(xd_batch* b)
{
    if (!b) return XD_OK;
    mixed_batch_destroy(b->mixed);
    delete b;
    return XD_OK;
}

int xd_scene_device_bytes(xd_scene* s, unsigned long long* bytes)
{
    if (!s || !bytes) return set_error(XD_ERR_INVALID, "scene_device_bytes: null argument");
    *bytes = s->bytes + (s->mixed ? mixed_device_bytes(s->mixed) : 0ull);
    return XD_OK;
}

}  // extern "C"
