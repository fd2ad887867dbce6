// Drop-in check of the legacy interface: steps written against the
// reference's own legacy names (cu_dem_dec.cuh) only -- the calls a parSIM
// time loop makes (Verlet_integrator, cell_grid::detection, dem_force and the
// cube geometry) -- linked with libxdem_legacy.so.  Reads a scene file, runs
// nsteps, writes the state.
//
//   legacy_step <in.bin> <out.bin>
// in:  u32 np, u32 nsteps, device_parameters, device_plane_info[6], double kn, vn, ks, vs, mu (cube),
//      pos, vel, acc, omega, alpha [np][4]
// out: pos, vel, acc, omega, alpha [np][4], sorted_id[np]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cu_dem_dec.cuh"

template <typename T>
static void rd(FILE* f, T* p, size_t n)
{
    if (fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}

int main(int argc, char** argv)
{
    if (argc != 3) { fprintf(stderr, "usage: %s in out\n", argv[0]); return 2; }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    unsigned hdr[2];
    rd(f, hdr, 2);
    const unsigned np = hdr[0], nsteps = hdr[1];
    device_parameters dp;
    device_plane_info planes[6];
    double wall[5];
    rd(f, &dp, 1);
    rd(f, planes, 6);
    rd(f, wall, 5);
    const char* names[5] = { "pos", "vel", "acc", "omega", "alpha" };
    std::vector<double> h[5];
    double* d[5];
    for (int k = 0; k < 5; ++k) {
        h[k].resize(4 * (size_t)np);
        rd(f, h[k].data(), h[k].size());
        cudaMalloc(&d[k], sizeof(double) * h[k].size());
        cudaMemcpy(d[k], h[k].data(), sizeof(double) * h[k].size(), cudaMemcpyHostToDevice);
    }
    fclose(f);
    (void)names;
    double *force, *moment;
    unsigned *hash, *index, *cstart, *cend, *sorted;
    device_plane_info* dplanes;
    bool* line;
    const unsigned nc = dp.ncell;
    cudaMalloc(&force, sizeof(double) * 3 * np);
    cudaMalloc(&moment, sizeof(double) * 3 * np);
    cudaMalloc(&hash, sizeof(unsigned) * np);
    cudaMalloc(&index, sizeof(unsigned) * np);
    cudaMalloc(&sorted, sizeof(unsigned) * np);
    cudaMalloc(&cstart, sizeof(unsigned) * nc);
    cudaMalloc(&cend, sizeof(unsigned) * nc);
    cudaMemset(cend, 0, sizeof(unsigned) * nc);
    cudaMalloc(&dplanes, sizeof(planes));
    cudaMemcpy(dplanes, planes, sizeof(planes), cudaMemcpyHostToDevice);
    cudaMalloc(&line, np);
    setSymbolicParameter(&dp);
    for (unsigned t = 0; t < nsteps; ++t) {
        vv_update_position(d[0], d[1], d[2], np);
        cu_calculateHashAndIndex(hash, index, d[0], np);
        cu_reorderDataAndFindCellStart(hash, index, cstart, cend, sorted, np, nc);
        cudaMemset(force, 0, sizeof(double) * 3 * np);
        cudaMemset(moment, 0, sizeof(double) * 3 * np);
        cu_calculate_p2p(d[0], d[1], d[2], d[3], d[4], force, moment, sorted, cstart, cend, np);
        cu_cube_hertzian_contact_force(dplanes, wall[0], wall[1], wall[2], wall[3], wall[4], line, d[0], d[1], d[3],
                                       force, moment, np);
        vv_update_velocity(d[1], d[2], d[3], d[4], force, moment, np);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) { fprintf(stderr, "CUDA error\n"); return 1; }
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 2;
    for (int k = 0; k < 5; ++k) {
        cudaMemcpy(h[k].data(), d[k], sizeof(double) * h[k].size(), cudaMemcpyDeviceToHost);
        fwrite(h[k].data(), sizeof(double), h[k].size(), o);
    }
    std::vector<unsigned> s(np);
    cudaMemcpy(s.data(), sorted, sizeof(unsigned) * np, cudaMemcpyDeviceToHost);
    fwrite(s.data(), sizeof(unsigned), np, o);
    fclose(o);
    return 0;
}
