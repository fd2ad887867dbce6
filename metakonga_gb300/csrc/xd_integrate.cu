// Velocity-Verlet update (the reference's vv_update_position /
// vv_update_velocity, include/mphysics_cuda_impl.cuh:85-134), FP64.
// Compiled with --fmad=false: the results equal the reference's expressions
// evaluated in IEEE double.
#include <cuda_runtime.h>

#include "xd_grid.cuh"
#include "xd_internal.cuh"

namespace xd {

// impl:85-96: _p = dt*v + half2dt*a; pos.xyz += _p
__global__ void __launch_bounds__(256) k_vv_position(Params P, double* __restrict__ pos,
                                                     const double* __restrict__ vel,
                                                     const double* __restrict__ acc, unsigned np)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    d3 p = P.dt * ld3(vel, id) + P.half2dt * ld3(acc, id);
    double* q = pos + 4 * (size_t)id;
    q[0] += p.x;
    q[1] += p.y;
    q[2] += p.z;
}

struct VelOut {
    d3 v, a;
};

// impl:98-134, one particle: returns the new velocity and acceleration and
// writes omega, alpha, force = m g, moment = 0.
__device__ __forceinline__ VelOut vv_velocity_one(const Params& P, unsigned id, double* vel,
                                                  double* acc, double* omega, double* alpha,
                                                  double* force, double* moment,
                                                  const double* mass, const double* inertia)
{
    double m = __ldg(mass + id);
    d3 v = ld3rw(vel, id);
    d3 av = ld3rw(omega, id);
    d3 a = (1.0 / m) * ld3rw(force, id);
    d3 in = (1.0 / __ldg(inertia + id)) * ld3rw(moment, id);
    double h = 0.5 * P.dt;
    v += h * (ld3rw(acc, id) + a);
    av += h * (ld3rw(alpha, id) + in);
    st3(force, id, m * mk(P.g[0], P.g[1], P.g[2]));
    st3(moment, id, mk(0.0, 0.0, 0.0));
    st3(vel, id, v);
    st3(omega, id, av);
    st3(acc, id, a);
    st3(alpha, id, in);
    return VelOut{ v, a };
}

__global__ void __launch_bounds__(256) k_vv_velocity(Params P, double* __restrict__ vel,
                                                     double* __restrict__ acc,
                                                     double* __restrict__ omega,
                                                     double* __restrict__ alpha,
                                                     double* __restrict__ force,
                                                     double* __restrict__ moment,
                                                     const double* __restrict__ mass,
                                                     const double* __restrict__ inertia, unsigned np)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    vv_velocity_one(P, id, vel, acc, omega, alpha, force, moment, mass, inertia);
}

// velocity update of step t, then the position update of step t+1 with the
// values just computed (same expressions as the two kernels above).
__global__ void __launch_bounds__(256) k_vv_velocity_position(
    Params P, double* __restrict__ pos, double* __restrict__ vel, double* __restrict__ acc,
    double* __restrict__ omega, double* __restrict__ alpha, double* __restrict__ force,
    double* __restrict__ moment, const double* __restrict__ mass,
    const double* __restrict__ inertia, unsigned np)
{
    unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    VelOut o = vv_velocity_one(P, id, vel, acc, omega, alpha, force, moment, mass, inertia);
    d3 p = P.dt * o.v + P.half2dt * o.a;
    double* q = pos + 4 * (size_t)id;
    q[0] += p.x;
    q[1] += p.y;
    q[2] += p.z;
}

int launch_vv_position(const Params& P, double* pos, const double* vel, const double* acc,
                       unsigned np, cudaStream_t s)
{
    if (np == 0) return XD_OK;
    k_vv_position<<<div_up(np, 256), 256, 0, s>>>(P, pos, vel, acc, np);
    return launch_status("vv_update_position");
}

int launch_vv_velocity(const Params& P, double* vel, double* acc, double* omega, double* alpha,
                       double* force, double* moment, const double* mass, const double* inertia,
                       unsigned np, cudaStream_t s)
{
    if (np == 0) return XD_OK;
    k_vv_velocity<<<div_up(np, 256), 256, 0, s>>>(P, vel, acc, omega, alpha, force, moment, mass,
                                                  inertia, np);
    return launch_status("vv_update_velocity");
}

int launch_vv_velocity_position(const Params& P, double* pos, double* vel, double* acc,
                                double* omega, double* alpha, double* force, double* moment,
                                const double* mass, const double* inertia, unsigned np,
                                cudaStream_t s)
{
    if (np == 0) return XD_OK;
    k_vv_velocity_position<<<div_up(np, 256), 256, 0, s>>>(P, pos, vel, acc, omega, alpha, force,
                                                           moment, mass, inertia, np);
    return launch_status("vv_update_velocity_position");
}

}  // namespace xd
