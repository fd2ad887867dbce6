/*
 * xdem_host.h -- the reference's host-side grid and integrator classes,
 * GPU branch, implemented on libxdem (linked from libxdem_mphysics.so).
 *
 *   grid_base / neighborhood_cell   include/grid_base.h:7-64,
 *                                   include/neighborhood_cell.h:6-24,
 *                                   source/grid_base.cpp, source/neighborhood_cell.cpp
 *   dem_integrator / velocity_verlet include/dem_integrator.h:6-32,
 *                                   include/velocity_verlet.h:6-27,
 *                                   source/velocity_verlet.cpp
 *
 * Same class names, members and virtual methods; the Qt includes are gone
 * and only the GPU branch exists (the reference's CPU branch is its own
 * single-threaded code path).  VEC3D, VEC3I and VEC3UI are the reference's
 * algebra types: an includer that already has them (vectorTypes.h) defines
 * XD_HAVE_VECTOR_TYPES first; otherwise minimal equivalents are declared.
 */
#ifndef XDEM_HOST_H
#define XDEM_HOST_H

#include <cstddef>

#ifndef XD_HAVE_VECTOR_TYPES
struct VEC3D {
    double x = 0, y = 0, z = 0;
    VEC3D() = default;
    VEC3D(double a, double b, double c) : x(a), y(b), z(c) {}
};
struct VEC3I {
    int x = 0, y = 0, z = 0;
    VEC3I() = default;
    VEC3I(int a, int b, int c) : x(a), y(b), z(c) {}
};
struct VEC3UI {
    unsigned int x = 0, y = 0, z = 0;
    VEC3UI() = default;
    VEC3UI(unsigned a, unsigned b, unsigned c) : x(a), y(b), z(c) {}
};
#endif

class grid_base
{
public:
    enum Type { NEIGHBORHOOD };
    grid_base();
    grid_base(Type t);
    virtual ~grid_base();

    void clear();
    void initialize(unsigned int np);
    virtual void detection(double* pos = NULL, double* spos = NULL, unsigned int np = 0, unsigned int snp = 0) = 0;
    virtual void detection_f(float* pos = NULL, float* spos = NULL, unsigned int np = 0, unsigned int snp = 0) = 0;

    void setWorldOrigin(VEC3D _wo) { wo = _wo; }
    void setCellSize(double _cs) { cs = _cs; }
    void setGridSize(VEC3UI _gs) { gs = _gs; }
    unsigned int nCell() { return ng; }
    void allocMemory(unsigned int n);
    void cuAllocMemory(unsigned int n);

    static VEC3I getCellNumber(double x, double y, double z);
    static unsigned int getHash(VEC3I& c3);
    unsigned int* sortedID() { return d_sorted_id; }
    unsigned int* cellStart() { return d_cell_start; }
    unsigned int* cellEnd() { return d_cell_end; }

    static VEC3D wo;    // world origin
    static double cs;   // cell size
    static VEC3UI gs;   // grid size

protected:
    Type type;
    unsigned int* d_sorted_id;
    unsigned int* d_cell_id;
    unsigned int* d_body_id;
    unsigned int* d_cell_start;
    unsigned int* d_cell_end;
    unsigned int nse;   // number of sorting elements
    unsigned int ng;    // number of cells
};

class neighborhood_cell : public grid_base
{
public:
    neighborhood_cell();
    virtual ~neighborhood_cell();
    virtual void detection(double* pos = NULL, double* spos = NULL, unsigned int np = 0, unsigned int snp = 0);
    virtual void detection_f(float* pos = NULL, float* spos = NULL, unsigned int np = 0, unsigned int snp = 0);
};

class dem_integrator
{
public:
    enum Type { VELOCITY_VERLET };
    dem_integrator() : type(VELOCITY_VERLET) {}
    dem_integrator(Type t) : type(t) {}
    virtual ~dem_integrator() {}
    Type integrationType() { return type; }
    virtual void updatePosition(double* dpos, double* dvel, double* dacc, unsigned int np) = 0;
    virtual void updateVelocity(double* dvel, double* dacc, double* domega, double* dalpha,
                                double* dforce, double* dmoment, double* dmass, double* dinertia,
                                unsigned int np) = 0;
    virtual void updatePosition(float* dpos, float* dvel, float* dacc, unsigned int np) = 0;
    virtual void updateVelocity(float* dvel, float* dacc, float* domega, float* dalpha,
                                float* dforce, float* dmoment, float* dmass, float* dinertia,
                                unsigned int np) = 0;

protected:
    Type type;
};

class velocity_verlet : public dem_integrator
{
public:
    velocity_verlet() : dem_integrator(VELOCITY_VERLET) {}
    ~velocity_verlet() {}
    virtual void updatePosition(double* dpos, double* dvel, double* dacc, unsigned int np);
    virtual void updateVelocity(double* dvel, double* dacc, double* domega, double* dalpha,
                                double* dforce, double* dmoment, double* dmass, double* dinertia,
                                unsigned int np);
    virtual void updatePosition(float* dpos, float* dvel, float* dacc, unsigned int np);
    virtual void updateVelocity(float* dvel, float* dacc, float* domega, float* dalpha,
                                float* dforce, float* dmoment, float* dmass, float* dinertia,
                                unsigned int np);
};

#endif
