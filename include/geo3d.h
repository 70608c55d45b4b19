/*
 * ibm3d-gb300 geometry C ABI: drop-in for the reference's src/geo3d.h:1-46.
 * Vector helpers and the Polyhedron (binary STL body) API.  Polyhedron_cpt
 * is the host entry point of the closest-point transform; the solver itself
 * computes the level set on the GPU during IBMSolver_assemble.
 */
#ifndef GEO3D_H
#define GEO3D_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCALE_INCH_TO_MM 25.4
#define SCALE_MM_TO_INCH (1 / 25.4)

/* 3-dimensional vector.  (src/geo3d.h:10-12) */
typedef struct _vector {
    double x, y, z;
} Vector;

/* Polyhedron (opaque).  (src/geo3d.h:15) */
typedef struct _polyhedron Polyhedron;

Vector Vector_add(const Vector, const Vector);
Vector Vector_sub(const Vector, const Vector);
double Vector_dot(const Vector, const Vector);
Vector Vector_crs(const Vector, const Vector);

double Vector_norm(const Vector);
double Vector_dist(const Vector, const Vector);
double Vector_angle(const Vector, const Vector);

Vector Vector_normalize(const Vector);
Vector Vector_lincom(const double, const Vector, const double, const Vector);
Vector Vector_rot(const Vector, const Vector, const double);

/* src/geo3d.h:31-35 */
Polyhedron *Polyhedron_new(void);
void Polyhedron_destroy(Polyhedron *);
void Polyhedron_read_stl(Polyhedron *, FILE *);
void Polyhedron_print_stats(Polyhedron *);
void Polyhedron_scale(Polyhedron *, double);

/* Signed distance of the polyhedron at the nx*ny*nz grid points (x[i],
   y[j], z[k]) into f[i][j][k] (row-major, k fastest), clipped to maxd.
   Replaces src/geo3d.c:436-704; computed on the GPU. */
void Polyhedron_cpt(
    const Polyhedron *const poly,
    const int nx, const int ny, const int nz,
    const double *x, const double *y, const double *z,
    double *f,
    const double maxd
);

/* No counterpart in the reference.  Same contract as Polyhedron_cpt (host
   arrays in and out) for callers that must not allocate device memory at
   this point - hosts whose framework allocator already owns the GPU memory,
   loops that cannot pay for an allocation.  It calls no cudaMalloc/cudaFree:
   all device buffers come from one static 32 MiB device array that every
   GPU loading the library holds until exit.  Returns 0, or -1 (with a
   message) when the grid, output and extrusion list need more than 32 MiB
   or on a CUDA error.  The array keeps the previous call's contents; the
   one value that must start at zero, the count of points left to the
   fallback scan, is cleared by every call.  The first call on a device
   looks up the array's address (setup), so make that first call before any
   stream capture.  Calls share the array: calls that overlap on the GPU
   (other threads, other streams) race. */
int Polyhedron_cpt_noalloc(
    const Polyhedron *const poly,
    const int nx, const int ny, const int nz,
    const double *x, const double *y, const double *z,
    double *f,
    const double maxd
);

#ifdef __cplusplus
}
#endif

#endif
