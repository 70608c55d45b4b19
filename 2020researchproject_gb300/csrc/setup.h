// Set-up kernels (level set, flags, ghost stencils): host interface.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "geo3d.h"

namespace ibm {

struct GhostStencil {
    int ok;             // mirror-point box inside the padded grid
    int im, jm, km;     // lower corner of the trilinear box
    double raw[8];      // trilinear weights as IBMSolver_ghost_interp returns them
    double w[8];        // solid entries dropped, renormalised, self removed
    int cell[8];        // padded index of each kept entry, -1 if dropped
    double wself;       // normalised weight of the ghost cell itself
};

// Signed distance on an nx*ny*nz grid (k fastest).  x, y, z, f are device
// pointers.  Returns 0 on success; *nfallback = points settled by full scan.
int gpu_cpt(cudaStream_t s, const CptModel &m, int nx, int ny, int nz, const double *x, const double *y,
            const double *z, double *f, double maxd, int *nfallback);
void gpu_flags(cudaStream_t s, const Grid &g, const double *lvset, uint8_t *flag);
int gpu_ghost_stencils(cudaStream_t s, const Grid &g, const double *xc, const double *yc, const double *zc,
                       const double *lvset, const uint8_t *flag, const int *gcell_dev, int ng, GhostStencil *out_dev);

}  // namespace ibm
