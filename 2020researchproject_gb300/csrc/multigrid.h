// Geometric multigrid V-cycle used as the BiCGSTAB preconditioner of the
// pressure-Poisson solve (replaces hypre's BoomerAMG, src/ibm3d_setup.c:
// 1490-1563).
//
// Level 0 is the padded fine grid and smooths the exact normalised pressure
// rows (fluid, ghost-interpolation, solid, pinned and outer boundary rows).
// Coarser levels carry a masked, symmetric cell-centred Laplacian in
// conductance form: a fine fluid-fluid face has conductance
// T = A_face dt / (2 Re dc) = Vol k_nb; a coarse face sums the fine faces it
// covers, halved when the face-normal axis was coarsened; faces touching a
// ghost, solid or pinned cell carry none (Neumann); pressure-Dirichlet
// boundaries fold into the diagonal and periodic ones wrap.  Residuals are
// restricted as Vol coeffsum r (the conductance form of a normalised row)
// and corrections are prolongated piecewise constant.  Levels small enough
// for one thread block run as a single-CTA kernel.
#pragma once

#include <vector>

#include "krylov.h"

namespace ibm {

template <typename T>
struct MGLevel {
    int nx, ny, nz;
    long long n;
    int cx, cy, cz;          // axis coarsened from the finer level
    T *Tx, *Ty, *Tz;         // conductance of the low face of each cell (wrap at 0 if periodic)
    T *diag;                 // sum of all couplings incl. Dirichlet boundaries
    T *R, *Z;
};

struct GMGConfig {
    int nu_pre = 2, nu_post = 2;
    int coarse_sweeps = 40;
    int tail_cells = 4096;   // levels at most this big run inside one CTA
};

class GMG : public Preconditioner {
  public:
    GMG() {}
    ~GMG() override;
    // ghost_cell: padded index of every ghost cell (nghost entries).
    int setup(cudaStream_t s, const OpCtx &ctx, const int *ghost_cell, int nghost, double Re, double dt,
              const GMGConfig &cfg);
    void apply(cudaStream_t s, const double *r, double *z) override;
    int nlevels() const { return (int)levels_.size() + 1; }

  private:
    OpCtx ctx_{};
    GMGConfig cfg_{};
    std::vector<MGLevel<double>> levels_;
    int tail_ = 0;                  // first coarse level handled by the single-CTA tail
    MGLevel<double> *dlevels_ = nullptr;  // device copy of the level table
    const int *ghost_cell_ = nullptr;
    int nghost_ = 0;
    double *ghost_tmp_ = nullptr;
    int *outer_ = nullptr;
    int nouter_ = 0;
    int per_[3] = {0, 0, 0};
    std::vector<void *> allocs_;
    void vcycle_level0(cudaStream_t s, const double *r, double *z);
    void smooth0(cudaStream_t s, const double *r, double *z, int sweeps);
};

}  // namespace ibm
