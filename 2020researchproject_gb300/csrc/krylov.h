// Krylov solvers (host side): BiCGSTAB in FP64 or FP32, and an FP64
// iterative-refinement driver around FP32 inner solves.
//
// Divergence criterion: for a fluid cell P the projected face velocity has
// div U^{n+1}_P = -2 Re coeffsum_P r_P, with r the residual of the
// normalised pressure row (coeffsum = sum of the six Crank-Nicolson
// coefficients, src/ibm3d_setup.c:1641-1649).  A solve stops once
// ||r|| < tol ||b|| (when tol > 0) or max_P |2 Re coeffsum_P r_P| <= divtol
// (when divtol > 0), whichever enabled test passes first.
//
// Every solve exists in two forms with the same kernels and arithmetic:
// a host loop (reads the device scalars after each half iteration; used
// with per-stage profiling) and a recorded form that appends the whole
// solve to a CUDA graph being captured, the iteration loop as a
// conditional while node whose condition the last kernel of each
// iteration sets on the device (no host round trip per iteration).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "kernels.h"
#include "ops.cuh"

namespace ibm {

struct Prof;

constexpr int KTHREADS = 256;
constexpr int KBLOCKS = 1216;  // 8 blocks per SM on 152 SMs; grid-stride loops

// Blocks of the grid-stride vector kernels for a vector of n elements:
// about 8 elements per thread, at most KBLOCKS, so that small cases
// running side by side (batched steps) leave the GPU to each other.
inline int vector_blocks(long long n) {
    const long long b = (n + KTHREADS * 8 - 1) / (KTHREADS * 8);
    return (int)(b < 1 ? 1 : b > KBLOCKS ? KBLOCKS : b);
}

enum { KS_RUN = 0, KS_HALF = 1, KS_DONE = 2, KS_BREAKDOWN = 3 };

struct KScal {
    double bnorm2, rnorm2, snorm2;
    double rho, alpha, omega, beta;
    double divmax;
    double tol, divtol;  // this solve's stopping test (set by the init kernel)
    int iters;
    int state;
    int restart;   // the next p update restarts the recurrence (r0 = r, p = r)
};

// BiCGSTAB restarts its recurrence every KRESTART iterations of a solve
// that has not converged: the current residual becomes the shadow residual
// r0 and the search direction (rho = ||r||^2, beta = 0), which ends the
// stagnation that a near-breakdown ((r0, r) -> 0) or an inexact FP32
// preconditioner can cause; a converging solve (4-20 iterations) never
// reaches it.
constexpr int KRESTART = 30;

// Outer (FP64) state of an iterative-refinement solve, per component.
struct IRScal {
    double bnorm2, rnorm2, rmax, divmax, scale;
    int state;
    int outer;   // refinement cycles completed
    int inner;   // FP32 Krylov iterations summed over the cycles
};

struct SolveParams {
    double tol = 1e-6;
    double divtol = 0.0;
    int maxit = 1000;
    double inner_tol = 1e-5;  // iterative refinement: relative tolerance of each FP32 solve
    int max_outer = 12;
    Prof *prof = nullptr;     // optional stage timers around SpMV / preconditioner (host loop only)
    bool x_given = false;     // iterative refinement: x holds the initial guess (else x = 0)
};

struct SolveReport {
    int iters[3] = {0, 0, 0};   // Krylov iterations (summed over refinement cycles)
    int outer = 0;              // refinement cycles (mixed path)
    double relres[3] = {0, 0, 0};
    double divmax[3] = {0, 0, 0};
};

// Loop control of a recorded solve: the handle of the enclosing
// conditional while node; use = 0 outside graphs.
struct LoopCtl {
    cudaGraphConditionalHandle h = 0;
    int use = 0;
};

// Entry type of the preconditioned vectors p^ = M p and s^ = M s: T, or
// FP32 under double-float Krylov vectors, whose preconditioner (the FP32
// V-cycle) produces FP32 values, so p^ and s^ are stored as they come.
template <typename T>
struct PrecT {
    using type = T;
};
template <>
struct PrecT<dfloat> {
    using type = float;
};

// gate (device pointer or null): when it points to a value other than
// KS_RUN every kernel of the application returns at once, so a recorded
// loop iteration after convergence costs only empty launches.
template <typename T>
struct Preconditioner {
    virtual ~Preconditioner() {}
    virtual void apply(cudaStream_t s, const T *r, typename PrecT<T>::type *z, const int *gate) = 0;
    // The same from an FP64 r, rounded to T inside the application (one
    // pass fewer than rounding first); false: not available, nothing ran.
    virtual bool apply_from64(cudaStream_t, const double *, T *, const int *) { return false; }
    // The same from double-float r (its high words).
    virtual bool apply_from_df(cudaStream_t, const dfloat *, T *, const int *) { return false; }
    // Kernels one application launches.
    virtual int launches() const = 0;
};

// FP64 Krylov vectors with an FP32 preconditioner: r is rounded to FP32,
// the FP32 preconditioner applied, and z widened back to FP64.  The outer
// BiCGSTAB keeps FP64 accuracy and convergence; the preconditioner (the
// multigrid V-cycle, most of the solve's traffic) runs on half the bytes.
struct WidenedPreconditioner : Preconditioner<double> {
    Preconditioner<float> *m32 = nullptr;
    float *r32 = nullptr, *z32 = nullptr;
    long long n = 0;
    int nblk = KBLOCKS;
    ~WidenedPreconditioner() override { release(); }
    int allocate(long long ncell, Preconditioner<float> *m);
    void release();
    void apply(cudaStream_t s, const double *r, double *z, const int *gate) override;
    int launches() const override { return m32->launches() + (fused_narrow ? 1 : 2); }
    bool fused_narrow = false;   // the last application rounded r inside m32
};

// Double-float Krylov vectors (the pressure solve of IBM3D_MIXED32) with
// the FP32 preconditioner: its right-hand side is the vector's high words
// (r rounded to FP32), its FP32 output is the preconditioned vector.
// Shares the FP32 buffer of a WidenedPreconditioner (the two never run at
// once).
struct DFloatPreconditioner : Preconditioner<dfloat> {
    Preconditioner<float> *m32 = nullptr;
    float *r32 = nullptr;
    long long n = 0;
    int nblk = KBLOCKS;
    void attach(const WidenedPreconditioner &w) {
        m32 = w.m32;
        r32 = w.r32;
        n = w.n;
        nblk = w.nblk;
    }
    void apply(cudaStream_t s, const dfloat *r, float *z, const int *gate) override;
    int launches() const override { return m32->launches() + (fused_narrow ? 0 : 1); }
    bool fused_narrow = false;
};

template <typename T>
struct KrylovWork {
    bool owner = true;   // false for a view of another work's buffers
    long long n = 0;
    int nc = 0;
    int nblk = KBLOCKS;  // blocks of the vector kernels
    T *base = nullptr;
    using PT = typename PrecT<T>::type;
    T *r = nullptr, *r0 = nullptr, *p = nullptr, *v = nullptr, *s = nullptr, *t = nullptr;
    PT *ph = nullptr, *sh = nullptr;   // p and s themselves when allocated without a preconditioner
    // p^ and s^ of a solve with preconditioner M, or p and s themselves
    // when it has none (a double-float solve always has one).
    const PT *phat(const void *M) const {
        if constexpr (std::is_same<PT, T>::value) return M ? ph : p;
        else return ph;
    }
    const PT *shat(const void *M) const {
        if constexpr (std::is_same<PT, T>::value) return M ? sh : s;
        else return sh;
    }
    KScal *scal = nullptr, *scal_h = nullptr;
    double *partials = nullptr;
    unsigned int *counter = nullptr;
    ~KrylovWork() { release(); }
    // maxblocks: the largest grid of any reduction kernel (sweeps included).
    int allocate(long long ncell, int ncomp, bool precond, int maxblocks);
    void release();
};

// The FP64 work's vectors seen as double-float vectors (the same bytes per
// entry; p^ and s^ as FP32 in the first half of theirs), with its scalars,
// partials and counter: a non-owning view.  Double-float solves always
// take the FP32 preconditioner.
KrylovWork<dfloat> dfloat_view(const KrylovWork<double> &w);

// FP64 outer vectors of an iterative-refinement solve plus its FP32 inner work.
struct IRWork {
    long long n = 0;
    int nc = 0;
    int nblk = KBLOCKS;  // blocks of the vector kernels
    double *r = nullptr;          // FP64 residual
    float *b32 = nullptr, *e32 = nullptr;
    IRScal *scal = nullptr, *scal_h = nullptr;
    double *partials = nullptr;
    unsigned int *counter = nullptr;
    KrylovWork<float> inner;
    ~IRWork() { release(); }
    int allocate(long long ncell, int ncomp, bool precond, int maxblocks);
    void release();
};

// Restarted flexible GMRES (FP64, one component): the pressure solve of
// SOLVER_GMRES (src/ibm3d_setup.c:1471-1477, restart length 10 there) and
// of the mixed path, where the preconditioner (the FP32 V-cycle behind a
// WidenedPreconditioner) is not an exact linear operator: the flexible
// form keeps every preconditioned vector, so the solve does not depend on
// it being one.  Classical Gram-Schmidt with one re-orthogonalisation pass.
constexpr int GM_MAX = 32;  // largest restart length

struct GScal {
    double h[(GM_MAX + 1) * GM_MAX];  // Hessenberg after rotations, column j at h[j * (GM_MAX + 1) + i]
    double cs[GM_MAX], sn[GM_MAX];    // Givens rotations
    double g[GM_MAX + 1];             // rotated right-hand side beta e1
    double c0[GM_MAX + 1], c1[GM_MAX + 1];  // projections of the two Gram-Schmidt passes
    double bnorm2, rnorm2, beta0, divmax0, divmax, res, vscale, tol, divtol;
    int j, m, iters, cycles, state, maxit;
    int more;  // the Arnoldi loop continues (set by each step)
};

struct GmresWork {
    long long n = 0;
    int m = 0;
    int nblk = KBLOCKS;
    double *base = nullptr;
    double *V = nullptr, *Z = nullptr;  // m basis vectors, m preconditioned vectors
    double *w = nullptr, *vin = nullptr, *zj = nullptr;
    GScal *scal = nullptr, *scal_h = nullptr;
    double *partials = nullptr;
    unsigned int *counter = nullptr;
    ~GmresWork() { release(); }
    int allocate(long long ncell, int restart, int maxblocks);
    void release();
};

// Host loop: solves A x = b (OP_PRES) from x0 = 0 with the stopping test of
// bicgstab (checked on the true residual at the end of each cycle).
int gmres(cudaStream_t st, const OpT<double> &A, int op, GmresWork &w, const double *b, double *x,
          const SolveParams &prm, Preconditioner<double> *M, SolveReport &rep);
int record_gmres(cudaStream_t st, const cudaStream_t *aux, const OpT<double> &A, int op, GmresWork &w,
                 const double *b, double *x, const SolveParams &prm, Preconditioner<double> *M, int *fixed,
                 int *per_cycle, int *per_iter);
int report(const GmresWork &w, SolveReport &rep);

// Host loop.  Solves A x = b (nc components for OP_MOM, 1 for OP_PRES)
// from x0 = 0.  Returns 0 when every component converged, 1 on reaching
// maxit, 2 on a Krylov breakdown.
template <typename T>
int bicgstab(cudaStream_t st, const OpT<T> &A, int op, KrylovWork<T> &w, const T *b, T *x, const SolveParams &prm,
             Preconditioner<T> *M, SolveReport &rep);

// Mixed precision, host loop: FP64 residuals r = b - A64 x and updates
// x += e, with each correction e from an FP32 BiCGSTAB on A32 e = r
// (scaled to unit max-norm).  Stops on the same FP64 criterion as
// bicgstab<double>.
int solve_ir(cudaStream_t st, const OpT<double> &A64, const OpT<float> &A32, int op, IRWork &w, const double *b,
             double *x, const SolveParams &prm, Preconditioner<float> *M32, SolveReport &rep);

// Recorded forms: append the solve to the graph being captured on st
// (aux: two further streams, used to capture the loop bodies) and end
// with a copy of the device scalars into the work's scal_h.  After the
// graph has run and st is synchronised, report() gives the outcome and the
// status code of the host loop.  Launch counts: *fixed kernels outside
// loops, *per_iter per Krylov iteration, *per_outer per refinement cycle.
template <typename T>
int record_bicgstab(cudaStream_t st, const cudaStream_t *aux, const OpT<T> &A, int op, KrylovWork<T> &w, const T *b,
                    T *x, const SolveParams &prm, Preconditioner<T> *M, int *fixed, int *per_iter);

// BiCGSTAB on double-float vectors and the double-float operator, FP64 b
// and x: x (the initial guess when prm.x_given) is converted into xw at the
// start, the residual r = b - A xw formed from the FP64 b, and xw
// converted back into x at the end.  The scalars (alpha, omega, rho, the
// norms) and the combination of the dot products across threads stay
// FP64; the stopping test is bicgstab's, and an iteration that passes it
// on the recursive residual has it checked on the true residual b - A x
// (a miss restarts the recurrence from that residual).  Host loop and
// recorded form.
int bicgstab_df(cudaStream_t st, const OpT<dfloat> &A, int op, KrylovWork<dfloat> &w, dfloat *xw, const double *b,
                double *x, const SolveParams &prm, Preconditioner<dfloat> *M, SolveReport &rep);
int record_bicgstab_df(cudaStream_t st, const cudaStream_t *aux, const OpT<dfloat> &A, int op, KrylovWork<dfloat> &w,
                       dfloat *xw, const double *b, double *x, const SolveParams &prm, Preconditioner<dfloat> *M,
                       int *fixed, int *per_iter);
int record_ir(cudaStream_t st, const cudaStream_t *aux, const OpT<double> &A64, const OpT<float> &A32, int op,
              IRWork &w, const double *b, double *x, const SolveParams &prm, Preconditioner<float> *M32, int *fixed,
              int *per_outer, int *per_iter);
template <typename T>
int report(const KrylovWork<T> &w, SolveReport &rep);
int report(const IRWork &w, SolveReport &rep);

// Increment solve (IBM3D_MIXED32 momentum): A32 e = c in FP32 from e = 0,
// with c in w.b32 and ||b||^2, ||c||^2 per component already in w.scal
// (written by the kernel that formed c).  Each component stops once
// ||c - A e|| < max(inner_tol ||c||, tol ||b|| / 2), i.e. on the
// reference's relative test ||b - A u*|| < tol ||b|| with a factor-2
// margin for FP32 rounding.  The host loop and the recorded form; report
// returns 0 when every component met tol, 1 otherwise, 2 on breakdown.
int solve_inc(cudaStream_t st, const OpT<float> &A32, int op, IRWork &w, const SolveParams &prm, SolveReport &rep);
int record_inc(cudaStream_t st, const cudaStream_t *aux, const OpT<float> &A32, int op, IRWork &w,
               const SolveParams &prm, int *fixed, int *per_iter);
int report_inc(const IRWork &w, double tol, SolveReport &rep);

template <typename T>
void apply_operator(cudaStream_t st, const OpT<T> &A, int op, int comp, const T *x, T *y);

}  // namespace ibm
