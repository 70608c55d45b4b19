// Krylov solver interface (host side).
//
// Divergence criterion: for a fluid cell P the projected face velocity has
// div U^{n+1}_P = -2 Re coeffsum_P r_P, with r the residual of the
// normalised pressure row (coeffsum = sum of the six Crank-Nicolson
// coefficients, src/ibm3d_setup.c:1641-1649).  With divtol > 0 the pressure
// solve stops once max_P |2 Re coeffsum_P r_P| <= divtol instead of on the
// relative residual.
#pragma once

#include <cuda_runtime.h>

#include "kernels.h"

namespace ibm {

struct Prof;

constexpr int KTHREADS = 256;
constexpr int KBLOCKS = 1216;  // 8 blocks per SM on 152 SMs; grid-stride loops

enum { OP_MOM = 0, OP_PRES = 1 };
enum { KS_RUN = 0, KS_HALF = 1, KS_DONE = 2, KS_BREAKDOWN = 3 };

struct KScal {
    double bnorm2, rnorm2, snorm2;
    double rho, alpha, omega, beta;
    double divmax;
    int iters;
    int state;
};

struct SolveParams {
    double tol = 1e-6;
    double divtol = 0.0;
    double Re = 1.0;
    int maxit = 1000;
    bool sync_half = true;
    Prof *prof = nullptr;   // optional stage timers around SpMV / preconditioner
};

struct SolveReport {
    int iters[3] = {0, 0, 0};
    double relres[3] = {0, 0, 0};
    double divmax[3] = {0, 0, 0};
};

struct Preconditioner {
    virtual ~Preconditioner() {}
    virtual void apply(cudaStream_t s, const double *r, double *z) = 0;
};

struct KrylovWork {
    long long n = 0;
    int nc = 0;
    double *base = nullptr;
    double *r = nullptr, *r0 = nullptr, *p = nullptr, *v = nullptr, *s = nullptr, *t = nullptr;
    double *ph = nullptr, *sh = nullptr;
    KScal *scal = nullptr, *scal_h = nullptr;
    double *partials = nullptr;
    unsigned int *counter = nullptr;
    ~KrylovWork();
    int allocate(long long ncell, int ncomp, bool precond);
    void release();
};

// Solves A x = b (nc components for OP_MOM, 1 for OP_PRES) from x0 = 0.
// Returns 0 when every component converged, 1 on reaching maxit, 2 on a
// Krylov breakdown.
int bicgstab(cudaStream_t st, const OpCtx &ctx, int op, KrylovWork &w, const double *b, double *x,
             const SolveParams &prm, Preconditioner *M, SolveReport &rep);

void apply_operator(cudaStream_t st, const OpCtx &ctx, int op, int comp, const double *x, double *y);

double residual_norm(cudaStream_t st, const OpCtx &ctx, int op, int comp, const double *b, const double *x,
                     double *r, double two_re, KrylovWork &w, double *divmax);

}  // namespace ibm
