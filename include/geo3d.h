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

#ifdef __cplusplus
}
#endif

#endif
