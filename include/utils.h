/*
 * ibm3d-gb300: the helper header the reference's case drivers include
 * (src/utils.h of thecasterian/2020ResearchProject; src/main.c:4,
 * cavity.c:6, channel.c:5, jet.c:4, building.c:6), so that those drivers
 * compile against this library unchanged.
 *
 * The access macros address the padded host arrays of the reference's
 * layout (src/utils.h:7-16); Nx, Ny, Nz are whatever the including code
 * has in scope.  The functions are exported by libibm3d_gb300.so with the
 * reference's semantics (src/utils.c).
 */
#ifndef UTILS_H
#define UTILS_H

#include <stdio.h>

#include "ibm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* 1-D array with two padding entries on each side. */
#define c1e(a, i) ((a)[(i) + 2])
/* Padded cell array (Nx+4)(Ny+4)(Nz+4), k fastest. */
#define c3e(a, i, j, k) ((a)[(Ny + 4) * (Nz + 4) * ((i) + 2) + (Nz + 4) * ((j) + 2) + (k) + 2])
/* x-, y-, z-staggered face arrays. */
#define xse(a, i, j, k) ((a)[(Ny + 4) * (Nz + 4) * (i) + (Nz + 4) * ((j) + 2) + (k) + 2])
#define yse(a, i, j, k) ((a)[(Ny + 1) * (Nz + 4) * ((i) + 2) + (Nz + 4) * (j) + (k) + 2])
#define zse(a, i, j, k) ((a)[(Ny + 4) * (Nz + 1) * ((i) + 2) + (Nz + 1) * ((j) + 2) + (k)])

#define FOR_INNER_CELL(i, j, k) \
    for (int i = 0; i < Nx; i++)    \
        for (int j = 0; j < Ny; j++)    \
            for (int k = 0; k < Nz; k++)
#define FOR_ALL_XSTAG(i, j, k) \
    for (int i = 0; i <= Nx; i++)  \
        for (int j = 0; j < Ny; j++)   \
            for (int k = 0; k < Nz; k++)
#define FOR_ALL_YSTAG(i, j, k) \
    for (int i = 0; i < Nx; i++)   \
        for (int j = 0; j <= Ny; j++)  \
            for (int k = 0; k < Nz; k++)
#define FOR_ALL_ZSTAG(i, j, k) \
    for (int i = 0; i < Nx; i++)   \
        for (int j = 0; j < Ny; j++)   \
            for (int k = 0; k <= Nz; k++)

#define UNUSED __attribute__((unused))

#ifndef __cplusplus
/* GNU statement expressions, as the reference's drivers expect. */
#define max(a, b) ({ __typeof__(a) ibm3d_a_ = (a); __typeof__(b) ibm3d_b_ = (b); ibm3d_a_ > ibm3d_b_ ? ibm3d_a_ : ibm3d_b_; })
#define min(a, b) ({ __typeof__(a) ibm3d_a_ = (a); __typeof__(b) ibm3d_b_ = (b); ibm3d_a_ < ibm3d_b_ ? ibm3d_a_ : ibm3d_b_; })
#define SWAP(a, b) do { __typeof__(a) ibm3d_t_ = (a); (a) = (b); (b) = ibm3d_t_; } while (0)
#endif

/* fopen, or print "error: cannot open file" and exit with status 255
   (the reference aborts the MPI job, src/utils.c:13-20). */
FILE *fopen_check(const char *filename, const char *modes);
/* x * x */
double sq(const double x);
/* First index in the sorted arr[0..len) with arr[i] >= val (len if none). */
int lower_bound(const int len, const double arr[], const double val);
/* First index in the sorted arr[0..len) with arr[i] > val (len if none). */
int upper_bound(const int len, const double arr[], const double val);
/* Position of a DIR_* bit: north 0, east 1, south 2, west 3, down 4, up 5. */
int dir_to_idx(IBMSolverDirection dir);
/* ceil(a / b) for positive integers. */
int divceil(int a, int b);

#ifdef __cplusplus
}
#endif

#endif
