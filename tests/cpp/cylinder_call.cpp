// Drop-in check of cu_cylinder_hertzian_contact_force: the reference's C++
// name and signature (mphysics_cuda_dec.cuh), linked with
// libxdem_mphysics.so, on a particle cloud read from a file.
//
//   cylinder_call <in.bin> <out.bin>
// in:  u32 np, device_parameters, device_cylinder_info, device_contact_property,
//      double3 mpos, pos[np][4], vel, omega, force, moment [np][3], mass[np]
// out: force, moment, mf, mm [np][3]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "mphysics_cuda_dec.cuh"

template <typename T>
static void rd(FILE* f, T* p, size_t n)
{
    if (fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}

template <typename T>
static T* up(const std::vector<T>& h)
{
    T* d = nullptr;
    if (cudaMalloc(&d, sizeof(T) * h.size()) != cudaSuccess) exit(3);
    cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
    return d;
}

int main(int argc, char** argv)
{
    if (argc != 3) { fprintf(stderr, "usage: %s in out\n", argv[0]); return 2; }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    unsigned np;
    rd(f, &np, 1);
    device_parameters dp;
    device_cylinder_info cyl;
    device_contact_property cp;
    double3 mpos;
    rd(f, &dp, 1);
    rd(f, &cyl, 1);
    rd(f, &cp, 1);
    rd(f, &mpos, 1);
    std::vector<double> pos(4 * (size_t)np), vel(3 * (size_t)np), omega(3 * (size_t)np), force(3 * (size_t)np),
        moment(3 * (size_t)np), mass(np), zero(3 * (size_t)np, 0.0);
    rd(f, pos.data(), pos.size());
    rd(f, vel.data(), vel.size());
    rd(f, omega.data(), omega.size());
    rd(f, force.data(), force.size());
    rd(f, moment.data(), moment.size());
    rd(f, mass.data(), mass.size());
    fclose(f);
    setSymbolicParameter(&dp);
    double *dpos = up(pos), *dvel = up(vel), *dom = up(omega), *df = up(force), *dm = up(moment), *dmass = up(mass);
    double *dmf = up(zero), *dmm = up(zero);
    device_cylinder_info* dcyl = up(std::vector<device_cylinder_info>{ cyl });
    device_contact_property* dcp = up(std::vector<device_contact_property>{ cp });
    double3* dmpos = up(std::vector<double3>{ mpos });
    double3 hmf, hmm;
    cu_cylinder_hertzian_contact_force(1, dcyl, dpos, dvel, dom, df, dm, dmass, np, dcp, dmpos,
                                       reinterpret_cast<double3*>(dmf), reinterpret_cast<double3*>(dmm), hmf, hmm);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 2;
    for (double* d : { df, dm, dmf, dmm }) {
        cudaMemcpy(zero.data(), d, sizeof(double) * zero.size(), cudaMemcpyDeviceToHost);
        fwrite(zero.data(), sizeof(double), zero.size(), o);
    }
    fclose(o);
    return 0;
}
