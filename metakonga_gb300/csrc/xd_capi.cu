// libxdem C ABI: argument checks, status codes, the shared workspace of the
// stateless calls, and the launch of each kernel (include/xdem.h).
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "xd_grid.cuh"
#include "xd_internal.cuh"

static_assert(sizeof(xd_device_parameters) == 112, "device_parameters layout");
static_assert(sizeof(xd_contact_property) == 88, "device_contact_property layout");
static_assert(sizeof(xd_plane_info) == 232, "device_plane_info layout");
static_assert(sizeof(xd_polygon_info) == 152, "device_polygon_info layout");
static_assert(sizeof(xd_polygon_mass_info) == 160, "device_polygon_mass_info layout");
static_assert(offsetof(xd_polygon_mass_info, ep) == 32, "device_polygon_mass_info.ep offset");
static_assert(sizeof(xd_device_parameters_f) == 64, "device_parameters_f layout");
static_assert(sizeof(xd_contact_property_f) == 44, "device_contact_property_f layout");
static_assert(sizeof(xd_plane_info_f) == 116, "device_plane_info_f layout");
static_assert(sizeof(xd_polygon_info_f) == 76, "device_polygon_info_f layout");
static_assert(sizeof(xd_polygon_mass_info_f) == 80, "device_polygon_mass_info_f layout");
static_assert(offsetof(xd_polygon_mass_info_f, ep) == 16, "device_polygon_mass_info_f.ep offset");

namespace xd {

namespace {
std::mutex g_err_mu;
int g_err_status = XD_OK;
char g_err_msg[512] = "";

std::mutex g_ws_mu;
void* g_ws = nullptr;
size_t g_ws_bytes = 0;

bool g_have_params = false;
Params g_params;
}  // namespace

int set_error(int status, const char* fmt, ...)
{
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (g_err_status == XD_OK) {
        g_err_status = status;
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(g_err_msg, sizeof(g_err_msg), fmt, ap);
        va_end(ap);
    }
    return status;
}

int cuda_status(cudaError_t e, const char* where)
{
    if (e == cudaSuccess) return XD_OK;
    if (e == cudaErrorMemoryAllocation)
        return set_error(XD_ERR_NOMEM, "%s: %s", where, cudaGetErrorString(e));
    return set_error(XD_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

int launch_status(const char* where) { return cuda_status(cudaGetLastError(), where); }

void* workspace(size_t bytes, int* status)
{
    std::lock_guard<std::mutex> lk(g_ws_mu);
    *status = XD_OK;
    if (bytes <= g_ws_bytes && g_ws) return g_ws;
    if (g_ws) {
        cudaDeviceSynchronize();
        cudaFree(g_ws);
        g_ws = nullptr;
        g_ws_bytes = 0;
    }
    size_t want = bytes + bytes / 4 + 4096;
    cudaError_t e = cudaMalloc(&g_ws, want);
    if (e != cudaSuccess) {
        g_ws = nullptr;
        *status = cuda_status(e, "workspace allocation");
        return nullptr;
    }
    g_ws_bytes = want;
    return g_ws;
}

int release_workspace()
{
    std::lock_guard<std::mutex> lk(g_ws_mu);
    if (g_ws) {
        cudaError_t e = cudaDeviceSynchronize();
        cudaFree(g_ws);
        g_ws = nullptr;
        g_ws_bytes = 0;
        return cuda_status(e, "release_workspace");
    }
    return XD_OK;
}

const Params* params() { return g_have_params ? &g_params : nullptr; }
void set_params(const Params& p)
{
    g_params = p;
    g_have_params = true;
}

}  // namespace xd

using namespace xd;

#define XD_REQUIRE(cond, ...)                                     \
    do {                                                          \
        if (!(cond)) return set_error(XD_ERR_INVALID, __VA_ARGS__); \
    } while (0)

static inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
static inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

#define XD_NEED_PARAMS(name)                                                                 \
    const Params* PP = params();                                                             \
    if (!PP) return set_error(XD_ERR_STATE, "%s: xd_set_symbolic_parameter was not called", name)

extern "C" {

const char* xd_version(void) { return XDEM_VERSION; }

const char* xd_status_string(int status)
{
    switch (status) {
    case XD_OK: return "ok";
    case XD_ERR_INVALID: return "invalid argument";
    case XD_ERR_CUDA: return "CUDA error";
    case XD_ERR_NOMEM: return "out of device memory";
    case XD_ERR_CAPACITY: return "capacity exceeded";
    case XD_ERR_TIMEOUT: return "device wait timed out";
    case XD_ERR_STATE: return "call out of order";
    default: return "unknown status";
    }
}

int xd_last_error(char* msg, size_t msg_len)
{
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (msg && msg_len) {
        strncpy(msg, g_err_msg, msg_len - 1);
        msg[msg_len - 1] = '\0';
    }
    return g_err_status;
}

void xd_clear_error(void)
{
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err_status = XD_OK;
    g_err_msg[0] = '\0';
}

size_t xd_sizeof(const char* n)
{
    if (!n) return 0;
    if (!strcmp(n, "device_parameters")) return sizeof(xd_device_parameters);
    if (!strcmp(n, "device_contact_property")) return sizeof(xd_contact_property);
    if (!strcmp(n, "device_plane_info")) return sizeof(xd_plane_info);
    if (!strcmp(n, "device_polygon_info")) return sizeof(xd_polygon_info);
    if (!strcmp(n, "device_polygon_mass_info")) return sizeof(xd_polygon_mass_info);
    if (!strcmp(n, "device_parameters_f")) return sizeof(xd_device_parameters_f);
    if (!strcmp(n, "device_contact_property_f")) return sizeof(xd_contact_property_f);
    if (!strcmp(n, "device_plane_info_f")) return sizeof(xd_plane_info_f);
    if (!strcmp(n, "device_polygon_info_f")) return sizeof(xd_polygon_info_f);
    if (!strcmp(n, "device_polygon_mass_info_f")) return sizeof(xd_polygon_mass_info_f);
    if (!strcmp(n, "xd_scene_desc")) return sizeof(xd_scene_desc);
    return 0;
}

int xd_release_workspace(void) { return release_workspace(); }

int xd_report_unsupported(const char* what)
{
    return set_error(XD_ERR_INVALID, "%s: not provided", what ? what : "entry point");
}

int xd_set_symbolic_parameter(const xd_device_parameters* h)
{
    XD_REQUIRE(h, "set_symbolic_parameter: null parameters");
    unsigned gx = h->grid_size[0], gy = h->grid_size[1], gz = h->grid_size[2];
    XD_REQUIRE(gx && gy && gz && !(gx & (gx - 1)) && !(gy & (gy - 1)) && !(gz & (gz - 1)),
               "set_symbolic_parameter: grid sizes must be powers of two (the hash wraps with &)");
    XD_REQUIRE(h->cell_size > 0.0, "set_symbolic_parameter: cell_size must be > 0");
    set_params(to_params(*h));
    return XD_OK;
}

int xd_vv_update_position(double* pos, const double* vel, const double* acc, unsigned np, void* s)
{
    XD_NEED_PARAMS("vv_update_position");
    if (np == 0) return XD_OK;
    XD_REQUIRE(pos && vel && acc, "vv_update_position: null pointer");
    return launch_vv_position(*PP, pos, vel, acc, np, S(s));
}

int xd_vv_update_velocity(double* vel, double* acc, double* omega, double* alpha, double* force,
                          double* moment, const double* mass, const double* inertia, unsigned np,
                          void* s)
{
    XD_NEED_PARAMS("vv_update_velocity");
    if (np == 0) return XD_OK;
    XD_REQUIRE(vel && acc && omega && alpha && force && moment && mass && inertia,
               "vv_update_velocity: null pointer");
    return launch_vv_velocity(*PP, vel, acc, omega, alpha, force, moment, mass, inertia, np, S(s));
}

int xd_vv_update_velocity_position(double* pos, double* vel, double* acc, double* omega,
                                   double* alpha, double* force, double* moment,
                                   const double* mass, const double* inertia, unsigned np,
                                   void* s)
{
    XD_NEED_PARAMS("vv_update_velocity_position");
    if (np == 0) return XD_OK;
    XD_REQUIRE(pos && vel && acc && omega && alpha && force && moment && mass && inertia,
               "vv_update_velocity_position: null pointer");
    return launch_vv_velocity_position(*PP, pos, vel, acc, omega, alpha, force, moment, mass,
                                       inertia, np, S(s));
}

int xd_calculate_hash_and_index(unsigned* hash, unsigned* index, const double* pos, unsigned np,
                                void* s)
{
    XD_NEED_PARAMS("calculate_hash_and_index");
    if (np == 0) return XD_OK;
    XD_REQUIRE(hash && index && pos, "calculate_hash_and_index: null pointer");
    XD_REQUIRE(aligned16(pos), "calculate_hash_and_index: pos must be 16-byte aligned (double4 rows)");
    return launch_hash(*PP, hash, index, pos, np, 0, S(s));
}

int xd_calculate_hash_and_index_polysphere(unsigned* hash, unsigned* index, unsigned sid,
                                           unsigned nsphere, const double* sphere, void* s)
{
    XD_NEED_PARAMS("calculate_hash_and_index_polysphere");
    if (nsphere == 0) return XD_OK;
    XD_REQUIRE(hash && index && sphere, "calculate_hash_and_index_polysphere: null pointer");
    XD_REQUIRE(aligned16(sphere), "calculate_hash_and_index_polysphere: sphere must be 16-byte aligned");
    return launch_hash(*PP, hash, index, sphere, nsphere, sid, S(s));
}

int xd_reorder_and_find_cell_start(unsigned* hash, unsigned* index, unsigned* cstart,
                                   unsigned* cend, unsigned* sorted_index, unsigned n,
                                   unsigned ncell, void* s)
{
    XD_REQUIRE(cstart && cend, "reorder_and_find_cell_start: null cell arrays");
    XD_REQUIRE(ncell > 0, "reorder_and_find_cell_start: ncell must be > 0");
    if (n > 0) XD_REQUIRE(hash && index && sorted_index, "reorder_and_find_cell_start: null pointer");
    int st;
    void* ws = workspace(reorder_scratch_bytes(n), &st);
    if (!ws) return st;
    return reorder_and_find_cell_start(hash, index, cstart, cend, sorted_index, n, ncell, ws, S(s),
                                       true);
}

int xd_radix_sort_pairs(unsigned* keys, unsigned* values, unsigned n, unsigned key_bits, void* s)
{
    if (n <= 1) return XD_OK;
    XD_REQUIRE(keys && values, "radix_sort_pairs: null pointer");
    XD_REQUIRE(key_bits <= 32, "radix_sort_pairs: key_bits must be <= 32");
    int st;
    void* ws = workspace(radix_sort_scratch_bytes(n), &st);
    if (!ws) return st;
    unsigned *ok = nullptr, *ov = nullptr;
    st = radix_sort_pairs(keys, values, n, key_bits, ws, S(s), &ok, &ov);
    if (st != XD_OK) return st;
    if (ok != keys) {
        cudaError_t e = cudaMemcpyAsync(keys, ok, sizeof(unsigned) * (size_t)n, cudaMemcpyDeviceToDevice, S(s));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(values, ov, sizeof(unsigned) * (size_t)n, cudaMemcpyDeviceToDevice, S(s));
        return cuda_status(e, "radix_sort_pairs copy-back");
    }
    return XD_OK;
}

int xd_calculate_p2p(int tcm, const double* pos, const double* vel, const double* omega,
                     double* force, double* moment, const double* mass,
                     const unsigned* sorted_index, const unsigned* cstart, const unsigned* cend,
                     const xd_contact_property* cp, unsigned np, void* s)
{
    XD_NEED_PARAMS("calculate_p2p");
    XD_REQUIRE(tcm == 1, "calculate_p2p: only tcm = 1 (DHS) is provided");
    if (np == 0) return XD_OK;
    XD_REQUIRE(pos && vel && omega && force && moment && mass && sorted_index && cstart && cend && cp,
               "calculate_p2p: null pointer");
    XD_REQUIRE(aligned16(pos), "calculate_p2p: pos must be 16-byte aligned");
    return launch_p2p(*PP, pos, vel, omega, force, moment, mass, sorted_index, cstart, cend, cp, np,
                      S(s));
}

int xd_plane_contact_force(int tcm, const xd_plane_info* plane, const double* pos,
                           const double* vel, const double* omega, double* force, double* moment,
                           const double* mass, unsigned np, const xd_contact_property* cp, void* s)
{
    XD_NEED_PARAMS("plane_contact_force");
    XD_REQUIRE(tcm == 1, "plane_contact_force: only tcm = 1 (DHS) is provided");
    if (np == 0) return XD_OK;
    XD_REQUIRE(plane && pos && vel && omega && force && moment && mass && cp,
               "plane_contact_force: null pointer");
    XD_REQUIRE(aligned16(pos), "plane_contact_force: pos must be 16-byte aligned");
    return launch_planes(*PP, plane, cp, 0, 1, pos, vel, omega, force, moment, mass, np, S(s));
}

int xd_cylinder_contact_force(int tcm, const xd_cylinder_info* cyl, const double* pos,
                              const double* vel, const double* omega, double* force, double* moment,
                              const double* mass, unsigned np, const xd_contact_property* cp,
                              const double* mpos, double* mf, double* mm, void* s)
{
    XD_NEED_PARAMS("cylinder_contact_force");
    XD_REQUIRE(tcm == 1, "cylinder_contact_force: only tcm = 1 (DHS) is provided");
    if (np == 0) return XD_OK;
    XD_REQUIRE(cyl && pos && vel && omega && force && moment && mass && cp && mpos && mf && mm,
               "cylinder_contact_force: null pointer");
    XD_REQUIRE(aligned16(pos), "cylinder_contact_force: pos must be 16-byte aligned");
    return launch_cylinder(*PP, cyl, cp, pos, vel, omega, force, moment, mass, np, mpos, mf, mm, S(s));
}

int xd_cube_contact_force(int tcm, const xd_plane_info* planes6, const double* pos,
                          const double* vel, const double* omega, double* force, double* moment,
                          const double* mass, unsigned np, const xd_contact_property* cp, void* s)
{
    XD_NEED_PARAMS("cube_contact_force");
    XD_REQUIRE(tcm == 1, "cube_contact_force: only tcm = 1 (DHS) is provided");
    if (np == 0) return XD_OK;
    XD_REQUIRE(planes6 && pos && vel && omega && force && moment && mass && cp,
               "cube_contact_force: null pointer");
    XD_REQUIRE(aligned16(pos), "cube_contact_force: pos must be 16-byte aligned");
    return launch_planes(*PP, planes6, cp, 0, 6, pos, vel, omega, force, moment, mass, np, S(s));
}

int xd_planes_contact_force(int tcm, const xd_plane_info* planes, const xd_contact_property* cps,
                            unsigned nplanes, const double* pos, const double* vel,
                            const double* omega, double* force, double* moment,
                            const double* mass, unsigned np, void* s)
{
    XD_NEED_PARAMS("planes_contact_force");
    XD_REQUIRE(tcm == 1, "planes_contact_force: only tcm = 1 (DHS) is provided");
    if (np == 0 || nplanes == 0) return XD_OK;
    XD_REQUIRE(planes && cps && pos && vel && omega && force && moment && mass,
               "planes_contact_force: null pointer");
    XD_REQUIRE(aligned16(pos), "planes_contact_force: pos must be 16-byte aligned");
    return launch_planes(*PP, planes, cps, 1, nplanes, pos, vel, omega, force, moment, mass, np,
                         S(s));
}

int xd_particle_polygon_collision(int tcm, const xd_polygon_info* dpi, const double* dsph,
                                  xd_polygon_mass_info* dpmi, const double* pos,
                                  const double* vel, const double* omega, double* force,
                                  double* moment, const double* mass, const unsigned* sidx,
                                  const unsigned* cstart, const unsigned* cend,
                                  const xd_contact_property* cp, unsigned np, unsigned nbodies,
                                  void* s)
{
    (void)dsph;
    (void)np;   // like the reference kernel (impl:932), the particle count is the parameter block's np
    XD_NEED_PARAMS("particle_polygon_collision");
    XD_REQUIRE(tcm == 1, "particle_polygon_collision: only tcm = 1 (DHS) is provided");
    if (PP->np == 0) return XD_OK;
    XD_REQUIRE(dpi && dpmi && pos && vel && omega && force && moment && mass && sidx && cstart && cend && cp,
               "particle_polygon_collision: null pointer");
    XD_REQUIRE(aligned16(pos), "particle_polygon_collision: pos must be 16-byte aligned");
    int st = XD_OK;
    void* ws = nullptr;
    size_t need = polygon_scratch_bytes(PP->np, nbodies);
    if (need) {
        ws = workspace(need, &st);
        if (!ws) return st;
    }
    return launch_polygon(*PP, dpi, dpmi, pos, vel, omega, force, moment, mass, sidx, cstart, cend,
                          cp, nbodies, ws, S(s));
}

int xd_update_polygon_object_data(const xd_polygon_mass_info* dpmi, const double* vList,
                                  double* sphere, xd_polygon_info* dpi, unsigned ntriangle, void* s)
{
    if (ntriangle == 0) return XD_OK;
    XD_REQUIRE(dpmi && vList && sphere && dpi, "update_polygon_object_data: null pointer");
    return launch_update_polygon(dpmi, vList, sphere, dpi, ntriangle, S(s));
}

int xd_reduction_d3(const double* in, unsigned n, double out[3], void* s)
{
    XD_REQUIRE(out, "reduction_d3: null output");
    out[0] = out[1] = out[2] = 0.0;
    if (n == 0) return XD_OK;
    XD_REQUIRE(in, "reduction_d3: null input");
    int st;
    void* ws = workspace(reduction_scratch_bytes(n), &st);
    if (!ws) return st;
    return reduction_d3(in, n, out, ws, S(s));
}

int xd_pair_list(const double* pos, const unsigned* sorted_index, const unsigned* cstart,
                 const unsigned* cend, unsigned np, unsigned* counts, unsigned* pairs,
                 unsigned long long cap, unsigned long long* total, void* s)
{
    XD_NEED_PARAMS("pair_list");
    XD_REQUIRE(total, "pair_list: null total");
    *total = 0;
    if (np == 0) return XD_OK;
    XD_REQUIRE(pos && sorted_index && cstart && cend && counts && (pairs || cap == 0),
               "pair_list: null pointer");
    int st;
    void* ws = workspace(pair_list_scratch_bytes(np), &st);
    if (!ws) return st;
    return pair_list(*PP, pos, sorted_index, cstart, cend, np, counts, pairs, cap, total, ws, S(s));
}

}  // extern "C"
