// Geometric multigrid V-cycle used as the BiCGSTAB preconditioner of the
// pressure-Poisson solve (replaces hypre's BoomerAMG, src/ibm3d_setup.c:
// 1490-1563), in FP64 (plain path) or FP32 (mixed path).
//
// Level 0 is the padded fine grid and smooths the exact normalised pressure
// rows (fluid, ghost-interpolation, solid, pinned and outer boundary rows).
// Coarser levels carry a masked, symmetric cell-centred Laplacian in
// conductance form: a fine fluid-fluid face has conductance
// T = A_face dt / (2 Re dc) = Vol k_nb; a coarse face sums the fine faces it
// covers, scaled by (finer centre distance) / (coarse centre distance)
// across it, so a coarse level is the rediscretised operator of its own
// cells; faces touching a ghost, solid or pinned cell carry none
// (Neumann); pressure-Dirichlet boundaries fold into the diagonal and
// periodic ones wrap.
//
// Coarsening.  A coarse cell covers one or two consecutive cells of the
// finer level along each axis (tensor-product groups).  Halving every
// axis (MG_COARSEN_HALVE) leaves the 5:1 cells of body-clustered grids
// 5:1 on every level, where point Gauss-Seidel barely smooths the weakly
// coupled direction.  By spacing (MG_COARSEN_SPACING, the default), level
// L merges a pair of neighbouring cells only while their joint width stays
// within width_ratio x 2^(L+1) x the finest width of the grid (1.5 by
// default): the small cells of
// the clustered region merge first and the large far-field cells wait
// until the others have grown to their size (semi-coarsening toward
// isotropic cells).  A level is kept at no more than half the cells of the
// one before (the threshold grows until it is), so a V-cycle costs at most
// about twice its finest level.  On a uniform grid both rules give the
// same halving.
//
// Residuals are restricted as Vol coeffsum r (the conductance form of a
// normalised row) by summation; corrections are prolongated trilinearly in cell-centre
// coordinates (renormalised over active coarse cells), which on the
// stretched benchmark grids cuts the Krylov iterations by a third against
// piecewise-constant transfer.  Smoothers are colour-ordered Gauss-Seidel
// with a fixed colour order (bitwise reproducible).  The coarsest levels
// run as one single-CTA kernel with their arrays in shared memory.
#pragma once

#include <vector>

#include "krylov.h"
#include "prof.h"

namespace ibm {

template <typename T>
struct MGLevel {
    int nx, ny, nz;
    long long n;
    int cx, cy, cz;          // axis halved uniformly from the finer level (cells 2I, 2I+1)
    T *Tx, *Ty, *Tz;         // conductance of the low face of each cell (wrap at 0 if periodic)
    T *diag;                 // sum of all couplings incl. Dirichlet boundaries; 0 = inactive
    T *idiag;                // 1 / diag (0 = inactive), for the relaxations
    T *R, *Z;
    // Trilinear prolongation to the finer level, per axis, indexed by the
    // finer level's cell index: the second coarse cell (-1: none) and the
    // weight of the cell's own parent.
    const int *po[3];
    const T *pw[3];
    // Groups, per axis: cell I covers finer cells ch[a][I] .. ch[a][I+1]-1
    // (one or two); pa[a][i] is the cell covering finer cell i.
    const int *ch[3];
    const int *pa[3];
};

// The fine rows' right-hand side r, 1/coeffsum and flags as the V-cycle's
// fine-level kernels read them.  split = 1 (the FP32 cycle on grids
// without a periodic seam): colour-split - two halves, red ((I+J+K) even)
// then black, each ordered by (I, J, K/2) over the padded box (padded
// coordinates I = i + 2, ...) - so that a colour pass reads only its
// colour's entries, contiguous along k; split = 0: the padded natural
// layout (index P).
template <typename T>
struct FineRows {
    const T *r;
    const T *dinv;
    const uint8_t *flag;
    int split;
    long long H;     // entries per colour half
    int NY, NZH;     // padded y extent; padded z extent halved, rounded up
    long long NYZH;  // NY * NZH: one padded plane of a half
    // Index of interior-relative cell (i, j, k) in the split layout, in
    // 32-bit arithmetic (the layout is used only below 2^31 entries).
    __host__ __device__ __forceinline__ int split_index(int i, int j, int k) const {
        return ((i + j + k) & 1) * (int)H + (i + 2) * (int)NYZH + (j + 2) * NZH + ((k + 2) >> 1);
    }
    __host__ __device__ __forceinline__ long long at(long long P, int i, int j, int k) const {
        return split ? split_index(i, j, k) : P;
    }
};

enum { MG_COARSEN_HALVE = 0, MG_COARSEN_SPACING = 1 };

struct GMGConfig {
    int nu_pre = 3, nu_post = 3;    // fine grid
    int nuc_pre = 2, nuc_post = 2;  // coarse levels above the coarsest
    int coarse_sweeps = 16;         // coarsest level
    double omega = 1.0;             // over-relaxation of the fine-grid fluid rows
    int coarsening = MG_COARSEN_SPACING;
    double width_ratio = 1.5;       // spacing rule: merge while the pair is within width_ratio x the target
};

// Host geometry of the fine grid: interior face coordinates per axis.
struct MGGeometry {
    std::vector<double> f[3];
};

// The coarsest levels, run inside one thread block (k_mg_tail): each
// level's place in the block's shared memory, as byte offsets into an
// image that setup builds once in global memory (conductances, diagonal,
// zeroed R and Z, transfer tables) and every launch copies with 16-byte
// loads.
constexpr int TAIL_MAXL = 16;

struct TailLevel {
    int nx, ny, nz, cx, cy, cz;
    long long n;
    int off[7];                          // Tx, Ty, Tz, diag, R, Z, idiag
    int opw[3], opo[3], opa[3], och[3];  // transfer tables toward the finer level (unused on level 0)
};

template <typename T>
struct TailDesc {
    int ntl;        // levels in the tail
    int words16;    // image size in 16-byte words
    TailLevel lv[TAIL_MAXL];
    const T *R_first;   // R and Z of the first tail level in global memory
    T *Z_first;
};

template <typename T>
class GMG : public Preconditioner<T> {
  public:
    GMG() {}
    ~GMG() override;
    // ghost_cell: padded index of every ghost cell (nghost entries).
    int setup(cudaStream_t s, const OpT<double> &A64, const OpT<T> &A, const int *ghost_cell, int nghost,
              const MGGeometry &geom, const GMGConfig &cfg);
    void apply(cudaStream_t s, const T *r, T *z, const int *gate) override;
    // FP32 cycles with colour-split fine rows round an FP64 r straight into
    // the split layout.
    bool apply_from64(cudaStream_t s, const double *r, T *z, const int *gate) override;
    bool apply_from_df(cudaStream_t s, const dfloat *r, T *z, const int *gate) override;
    int launches() const override { return launches_; }
    // Smoother sweeps (pre, post) on the fine grid and on the coarse levels,
    // and on the coarsest level; takes effect at the next apply.
    void set_omega(double w) { cfg_.omega = w; }
    void set_sweeps(int nu_pre, int nu_post, int nuc_pre, int nuc_post, int coarse) {
        cfg_.nu_pre = nu_pre;
        cfg_.nu_post = nu_post;
        cfg_.nuc_pre = nuc_pre;
        cfg_.nuc_post = nuc_post;
        cfg_.coarse_sweeps = coarse;
    }
    int nlevels() const { return (int)levels_.size() + 1; }
    // Stage timers for the phases of a V-cycle (used only while p->on,
    // i.e. host-sequenced steps with profiling on).
    void set_prof(Prof *p) { prof_ = p; }
    // Average device time (ms) of one fine-grid colour pass over r, z
    // (reps launches between CUDA events on s); bytes: its algorithmic
    // bytes (z read once, r, 1/coeffsum, flag read and z written for the
    // updated half of the interior cells).
    // timed = false: launches only (the caller times them).
    float time_color(cudaStream_t s, const T *r, T *z, int reps, double *bytes, bool timed = true);
    // Whether the fine rows are colour-split (FineRows).
    bool split() const { return split_; }

  private:
    OpT<T> A_{};
    GMGConfig cfg_{};
    std::vector<MGLevel<T>> levels_;
    int tail_ = 0;
    Prof *prof_ = nullptr;
    size_t tail_smem_ = 0;
    TailDesc<T> tail_desc_{};
    const uint4 *tail_img_ = nullptr;
    const int *ghost_cell_ = nullptr;
    int nghost_ = 0;
    T *ghost_tmp_ = nullptr;
    T *ghost_idiv_ = nullptr;  // per ghost id: inverse divisor of its relaxation
    bool ghost_reads_outer_ = false;
    // Layer-1 face cells of the outer layers: the only outer cells the
    // colour passes read (edges, corners and layer 2 are set after the
    // last sweep of each smoothing).
    int *outer1_ = nullptr;
    int nout1_ = 0;
    // Colour-split fine rows (FP32 cycles without a periodic seam): the
    // cycle's right-hand side (filled per application), 1/coeffsum and
    // flags; and per ghost the index of its row in the layout in use.
    bool split_ = false;
    T *rs_ = nullptr, *ds_ = nullptr;
    uint8_t *fs_ = nullptr;
    long long H_ = 0;
    int NZH_ = 0;
    long long *grow_ = nullptr;
    int per_[3] = {0, 0, 0};
    // Level 1's groups (host copy) and the restriction tiles cut from them.
    std::vector<int> ch1_[3];
    int *segj_ = nullptr, *segk_ = nullptr;
    int nsegj_ = 0, nsegk_ = 0;
    std::vector<void *> allocs_;
    int launches_ = 0;
    // sweeps of the fine-grid smoother; from_zero: z is taken as 0 on entry
    int smooth0(cudaStream_t s, const FineRows<T> &fr, T *z, int sweeps, bool from_zero, const int *gate);
    FineRows<T> rows(const T *r) const;
    void cycle(cudaStream_t s, const FineRows<T> &fr, T *z, const int *gate);
};

}  // namespace ibm
