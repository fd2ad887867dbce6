// Drop-in check: the reference's dem_simulation::oneStepAnalysis
// (source/simulation/dem_simulation.cpp:447-469) and
// contactManager::deviceCollision (source/contactManager.cpp:156-185),
// written against the reference's own API names (mphysics_cuda_dec.cuh,
// grid_base / neighborhood_cell, velocity_verlet) and linked with
// libxdem_mphysics.so.  Reads a scene file, runs nsteps, writes the state.
//
//   reference_step <in.bin> <out.bin>
// in:  u32 np, u32 nplanes, u32 nsteps, device_parameters, device_contact_property,
//      nplanes x (device_plane_info, device_contact_property),
//      pos[np][4], vel, acc, omega, alpha, force, moment [np][3], mass[np], inertia[np]
// out: i32 status, pos[np][4], vel, acc, omega, alpha [np][3], sorted_id[np]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mphysics_cuda_dec.cuh"
#include "xdem.h"
#include "xdem_host.h"

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
    unsigned hdr[3];
    rd(f, hdr, 3);
    unsigned np = hdr[0], npl = hdr[1], nsteps = hdr[2];
    device_parameters dp;
    device_contact_property cpp;
    rd(f, &dp, 1);
    rd(f, &cpp, 1);
    std::vector<device_plane_info> planes(npl);
    std::vector<device_contact_property> cpl(npl);
    for (unsigned i = 0; i < npl; ++i) { rd(f, &planes[i], 1); rd(f, &cpl[i], 1); }
    std::vector<double> pos(4 * np), vel(3 * np), acc(3 * np), om(3 * np), al(3 * np), fo(3 * np),
        mo(3 * np), mass(np), iner(np);
    rd(f, pos.data(), pos.size()); rd(f, vel.data(), vel.size()); rd(f, acc.data(), acc.size());
    rd(f, om.data(), om.size()); rd(f, al.data(), al.size()); rd(f, fo.data(), fo.size());
    rd(f, mo.data(), mo.size()); rd(f, mass.data(), np); rd(f, iner.data(), np);
    fclose(f);

    // dem_simulation::allocationMemory / initialize (dem_simulation.cpp:174-199, 259-307)
    double *dpos, *dvel, *dacc, *davel, *daacc, *dforce, *dmoment, *dmass, *diner;
    cudaMalloc((void**)&dpos, 8 * pos.size());
    cudaMalloc((void**)&dvel, 8 * vel.size());
    cudaMalloc((void**)&dacc, 8 * acc.size());
    cudaMalloc((void**)&davel, 8 * om.size());
    cudaMalloc((void**)&daacc, 8 * al.size());
    cudaMalloc((void**)&dforce, 8 * fo.size());
    cudaMalloc((void**)&dmoment, 8 * mo.size());
    cudaMalloc((void**)&dmass, 8 * np);
    cudaMalloc((void**)&diner, 8 * np);
    cudaMemcpy(dpos, pos.data(), 8 * pos.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dvel, vel.data(), 8 * vel.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dacc, acc.data(), 8 * acc.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(davel, om.data(), 8 * om.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(daacc, al.data(), 8 * al.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dforce, fo.data(), 8 * fo.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dmoment, mo.data(), 8 * mo.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dmass, mass.data(), 8 * np, cudaMemcpyHostToDevice);
    cudaMemcpy(diner, iner.data(), 8 * np, cudaMemcpyHostToDevice);
    device_contact_property* dcp;   // contact::cudaMemoryAlloc (contact.cpp:107-116)
    cudaMalloc((void**)&dcp, sizeof(device_contact_property));
    cudaMemcpy(dcp, &cpp, sizeof(cpp), cudaMemcpyHostToDevice);
    std::vector<device_plane_info*> dpi(npl);
    std::vector<device_contact_property*> dcpl(npl);
    for (unsigned i = 0; i < npl; ++i) {
        cudaMalloc((void**)&dpi[i], sizeof(device_plane_info));
        cudaMemcpy(dpi[i], &planes[i], sizeof(device_plane_info), cudaMemcpyHostToDevice);
        cudaMalloc((void**)&dcpl[i], sizeof(device_contact_property));
        cudaMemcpy(dcpl[i], &cpl[i], sizeof(device_contact_property), cudaMemcpyHostToDevice);
    }
    grid_base* dtor = new neighborhood_cell;
    dtor->setWorldOrigin(VEC3D(dp.world_origin.x, dp.world_origin.y, dp.world_origin.z));
    dtor->setGridSize(VEC3UI(dp.grid_size.x, dp.grid_size.y, dp.grid_size.z));
    dtor->setCellSize(dp.cell_size);
    dtor->initialize(np);
    dem_integrator* itor = new velocity_verlet;
    dp.np = np;
    dp.ncell = dtor->nCell();
    setSymbolicParameter(&dp);

    for (unsigned s = 0; s < nsteps; ++s) {
        // dem_simulation::oneStepAnalysis
        itor->updatePosition(dpos, dvel, dacc, np);
        dtor->detection(dpos, NULL, np, 0);
        // contactManager::deviceCollision: particles, then plane contacts in name order
        cu_calculate_p2p(1, dpos, dvel, davel, dforce, dmoment, dmass, dtor->sortedID(),
                         dtor->cellStart(), dtor->cellEnd(), dcp, np);
        for (unsigned i = 0; i < npl; ++i)
            cu_plane_contact_force(1, dpi[i], dpos, dvel, davel, dforce, dmoment, dmass, np, dcpl[i]);
        itor->updateVelocity(dvel, dacc, davel, daacc, dforce, dmoment, dmass, diner, np);
    }
    cudaDeviceSynchronize();
    char msg[256];
    int status = xd_last_error(msg, sizeof(msg));
    if (status) fprintf(stderr, "libxdem error %d: %s\n", status, msg);
    std::vector<unsigned> sorted(np);
    cudaMemcpy(pos.data(), dpos, 8 * pos.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(vel.data(), dvel, 8 * vel.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(acc.data(), dacc, 8 * acc.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(om.data(), davel, 8 * om.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(al.data(), daacc, 8 * al.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(sorted.data(), dtor->sortedID(), 4 * np, cudaMemcpyDeviceToHost);
    FILE* o = fopen(argv[2], "wb");
    fwrite(&status, 4, 1, o);
    fwrite(pos.data(), 8, pos.size(), o);
    fwrite(vel.data(), 8, vel.size(), o);
    fwrite(acc.data(), 8, acc.size(), o);
    fwrite(om.data(), 8, om.size(), o);
    fwrite(al.data(), 8, al.size(), o);
    fwrite(sorted.data(), 4, np, o);
    fclose(o);
    delete dtor;
    delete itor;
    return status ? 1 : 0;
}
