// Matrix-free momentum / pressure operators and the BiCGSTAB solver.
//
// Rows restate the matrices the reference assembles for hypre
// (create_matrix, src/ibm3d_setup.c:1566-2908): Crank-Nicolson Helmholtz
// rows (type 1..3) and diagonal-normalised Poisson rows (type 4) on fluid
// cells, interpolation rows on ghost cells, identity on solid cells,
// boundary rows on the two outer layers, and the pinned p'(0,0,0) row when
// no face fixes the pressure.  The solver follows hypre's BiCGSTAB as the
// reference drives it (src/ibm3d_fracstep.c:354-379, 649-703): x0 = 0,
// stop when ||b - Ax||_2 / ||b||_2 < tol.  The three momentum components
// are solved together, one Krylov recurrence per component, so each kernel
// sweeps the grid once for all three.
#include <cmath>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "krylov.h"
#include "prof.h"

namespace ibm {

enum { ROW_DIR = 0, ROW_NEU = 1, ROW_PER = 2, ROW_EXT = 3 };

__device__ __forceinline__ int outer_row_kind(int op, int type, int comp, int axis) {
    if (op == OP_MOM) {
        switch (type) {
        case BCT_VELOCITY: return ROW_DIR;
        case BCT_PRESSURE: return ROW_EXT;
        case BCT_SLIP: return comp == axis ? ROW_DIR : ROW_NEU;
        default: return ROW_PER;  // ALL_PERIODIC, VELOCITY_PERIODIC
        }
    }
    switch (type) {
    case BCT_VELOCITY:
    case BCT_SLIP: return ROW_NEU;
    case BCT_PRESSURE:
    case BCT_VELPERIODIC: return ROW_DIR;
    default: return ROW_PER;
    }
}

// One row of A (op OP_MOM with component comp, or OP_PRES) applied to x.
__device__ __forceinline__ double op_row(const OpCtx &c, int op, int comp, const double *__restrict__ x,
                                         long long P) {
    int i, j, k;
    cijk(c.g, P, i, j, k);
    int L;
    const int f = owner_face(c.g, i, j, k, L);
    if (f >= 0) {
        const BCFace &F = c.bc.f[f];
        const int axis = face_axis(f);
        const long long s = axis == 0 ? c.g.sx : axis == 1 ? c.g.sy : 1;
        const long long in = face_low(f) ? s : -s;
        switch (outer_row_kind(op, F.type, comp, axis)) {
        case ROW_DIR: return F.dir_o[L - 1] * x[P] + F.dir_m[L - 1] * x[P + (2 * L - 1) * in];
        case ROW_NEU: return x[P] - x[P + (2 * L - 1) * in];
        case ROW_PER: return x[P] - x[periodic_image(c.g, i, j, k)];
        default: return F.ext_o[L - 1] * x[P] - x[P + in] + F.ext_2[L - 1] * x[P + 2 * in];
        }
    }
    if (op == OP_PRES && c.bc.p_singular && i == 0 && j == 0 && k == 0) return x[P];
    const uint8_t fl = c.flag[P];
    if (fl == FLUID) {
        const int I = i + 2, J = j + 2, K = k + 2;
        const double kW = c.ax.km[I], kE = c.ax.kp[I], kS = c.ay.km[J], kN = c.ay.kp[J];
        const double kD = c.az.km[K], kU = c.az.kp[K];
        const long long sx = c.g.sx, sy = c.g.sy;
        const double nb = kW * x[P - sx] + kE * x[P + sx] + kS * x[P - sy] + kN * x[P + sy] + kD * x[P - 1] +
                          kU * x[P + 1];
        if (op == OP_MOM) {
            const double diag = 1 + kN + kE + kS + kW + kD + kU;
            return diag * x[P] - nb;
        }
        return x[P] - c.dinv[P] * nb;
    }
    if (fl == GHOST) {
        const int g = c.gid[P];
        double sum = 0;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int q = c.gidx[8 * g + e];
            if (q >= 0) sum += c.gw[8 * g + e] * x[q];
        }
        const double ws = c.gwself[g];
        return op == OP_MOM ? (1 + ws) * x[P] + sum : (1 - ws) * x[P] - sum;
    }
    return x[P];
}

// Weight turning a fluid-row pressure residual into the divergence of the
// projected face velocity: div U^{n+1} = -2 Re coeffsum r (see krylov.h).
__device__ __forceinline__ double div_weight(const OpCtx &c, long long P, double two_re) {
    int i, j, k;
    cijk(c.g, P, i, j, k);
    if (i < 0 || j < 0 || k < 0 || i >= c.g.nx || j >= c.g.ny || k >= c.g.nz) return 0.0;
    if (c.flag[P] != FLUID) return 0.0;
    if (c.bc.p_singular && i == 0 && j == 0 && k == 0) return 0.0;
    const int I = i + 2, J = j + 2, K = k + 2;
    return two_re * (c.ay.kp[J] + c.ax.kp[I] + c.ay.km[J] + c.ax.km[I] + c.az.km[K] + c.az.kp[K]);
}

#define GRID_STRIDE(P, n)                                                              \
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < (n); \
         P += (long long)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- init --
__global__ void __launch_bounds__(KTHREADS)
k_bicg_init(const long long n, const int nc, const double *__restrict__ b, double *x, double *r, double *r0,
            double *p, double *v, KScal *sc, double *partials, unsigned int *counter) {
    __shared__ double smem[32 * 3];
    double acc[3] = {0, 0, 0};
    for (int c = 0; c < nc; c++) {
        const long long o = c * n;
        GRID_STRIDE(P, n) {
            const double bv = b[o + P];
            x[o + P] = 0.0;
            r[o + P] = bv;
            r0[o + P] = bv;
            p[o + P] = 0.0;
            v[o + P] = 0.0;
            acc[c] += bv * bv;
        }
    }
    block_sum<3>(acc, smem);
    if (publish_partials<3>(acc, partials, counter)) {
        double tot[3];
        sum_partials<3>(partials, gridDim.x, tot);
        for (int c = 0; c < nc; c++) {
            KScal &s = sc[c];
            s.bnorm2 = tot[c];
            s.rnorm2 = tot[c];
            s.rho = tot[c];
            s.alpha = 1.0;
            s.omega = 1.0;
            s.beta = 0.0;
            s.iters = 0;
            s.state = tot[c] == 0.0 ? KS_DONE : KS_RUN;
            s.divmax = 0.0;
        }
        *counter = 0;
    }
}

// ------------------------------------------------- p = r + beta (p - w v) --
__global__ void __launch_bounds__(KTHREADS)
k_bicg_p(const long long n, const int nc, const double *__restrict__ r, double *p, const double *__restrict__ v,
         const KScal *sc) {
    for (int c = 0; c < nc; c++) {
        if (sc[c].state != KS_RUN) continue;
        const double beta = sc[c].beta, om = sc[c].omega;
        const long long o = c * n;
        GRID_STRIDE(P, n) { p[o + P] = r[o + P] + beta * (p[o + P] - om * v[o + P]); }
    }
}

// ------------------------------------------- v = A ph, alpha = rho/(r0,v) --
__global__ void __launch_bounds__(KTHREADS)
k_bicg_spmv_v(const OpCtx ctx, const int op, const long long n, const int nc, const double *__restrict__ ph,
              double *v, const double *__restrict__ r0, KScal *sc, double *partials, unsigned int *counter) {
    __shared__ double smem[32 * 3];
    double acc[3] = {0, 0, 0};
    for (int c = 0; c < nc; c++) {
        if (sc[c].state != KS_RUN) continue;
        const long long o = c * n;
        GRID_STRIDE(P, n) {
            const double y = op_row(ctx, op, c, ph + o, P);
            v[o + P] = y;
            acc[c] += r0[o + P] * y;
        }
    }
    block_sum<3>(acc, smem);
    if (publish_partials<3>(acc, partials, counter)) {
        double tot[3];
        sum_partials<3>(partials, gridDim.x, tot);
        for (int c = 0; c < nc; c++) {
            KScal &s = sc[c];
            if (s.state != KS_RUN) continue;
            if (tot[c] == 0.0) {
                s.state = KS_BREAKDOWN;
                continue;
            }
            s.alpha = s.rho / tot[c];
        }
        *counter = 0;
    }
}

// ------------------------------------------------------- s = r - alpha v --
__global__ void __launch_bounds__(KTHREADS)
k_bicg_s(const OpCtx ctx, const long long n, const int nc, const double *__restrict__ r,
         const double *__restrict__ v, double *s, KScal *sc, const double tol, const double divtol,
         const double two_re, double *partials, unsigned int *counter) {
    __shared__ double smem[32 * 4];
    double acc[4] = {0, 0, 0, 0};
    for (int c = 0; c < nc; c++) {
        if (sc[c].state != KS_RUN) continue;
        const double al = sc[c].alpha;
        const long long o = c * n;
        GRID_STRIDE(P, n) {
            const double y = r[o + P] - al * v[o + P];
            s[o + P] = y;
            acc[c] += y * y;
            if (divtol > 0) acc[3] = fmax(acc[3], fabs(y) * div_weight(ctx, P, two_re));
        }
    }
    double dm[1] = {acc[3]};
    double sm[3] = {acc[0], acc[1], acc[2]};
    block_sum<3>(sm, smem);
    __syncthreads();
    block_max<1>(dm, smem + 96);
    double out[4] = {sm[0], sm[1], sm[2], dm[0]};
    if (publish_partials<4>(out, partials, counter)) {
        double tot[4] = {0, 0, 0, 0};
        for (unsigned b = 0; b < gridDim.x; b++) {
            for (int q = 0; q < 3; q++) tot[q] += ((volatile double *)partials)[b * 4 + q];
            tot[3] = fmax(tot[3], ((volatile double *)partials)[b * 4 + 3]);
        }
        for (int c = 0; c < nc; c++) {
            KScal &st = sc[c];
            if (st.state != KS_RUN) continue;
            st.snorm2 = tot[c];
            const bool ok = divtol > 0 ? tot[3] <= divtol : sqrt(tot[c]) < tol * sqrt(st.bnorm2);
            if (ok) {
                st.state = KS_HALF;
                st.divmax = tot[3];
            }
        }
        *counter = 0;
    }
}

// --------------------------------------- t = A sh, omega = (t,s)/(t,t) --
__global__ void __launch_bounds__(KTHREADS)
k_bicg_spmv_t(const OpCtx ctx, const int op, const long long n, const int nc, const double *__restrict__ sh,
              double *t, const double *__restrict__ s, KScal *sc, double *partials, unsigned int *counter) {
    __shared__ double smem[32 * 6];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < nc; c++) {
        if (sc[c].state != KS_RUN) continue;
        const long long o = c * n;
        GRID_STRIDE(P, n) {
            const double y = op_row(ctx, op, c, sh + o, P);
            t[o + P] = y;
            acc[2 * c] += y * s[o + P];
            acc[2 * c + 1] += y * y;
        }
    }
    block_sum<6>(acc, smem);
    if (publish_partials<6>(acc, partials, counter)) {
        double tot[6];
        sum_partials<6>(partials, gridDim.x, tot);
        for (int c = 0; c < nc; c++) {
            KScal &st = sc[c];
            if (st.state != KS_RUN) continue;
            if (tot[2 * c + 1] == 0.0) {
                st.omega = 0.0;
                st.state = KS_BREAKDOWN;
                continue;
            }
            st.omega = tot[2 * c] / tot[2 * c + 1];
        }
        *counter = 0;
    }
}

// ------------------- x += alpha ph + omega sh, r = s - omega t, new rho --
__global__ void __launch_bounds__(KTHREADS)
k_bicg_xr(const OpCtx ctx, const long long n, const int nc, double *x, double *r, const double *__restrict__ r0,
          const double *__restrict__ ph, const double *__restrict__ sh, const double *__restrict__ s,
          const double *__restrict__ t, KScal *sc, const double tol, const double divtol, const double two_re,
          double *partials, unsigned int *counter) {
    __shared__ double smem[32 * 7];
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < nc; c++) {
        const int state = sc[c].state;
        const long long o = c * n;
        if (state == KS_HALF) {
            // Converged on s: x += alpha ph, r = s.
            const double al = sc[c].alpha;
            GRID_STRIDE(P, n) {
                x[o + P] += al * ph[o + P];
                r[o + P] = s[o + P];
            }
            continue;
        }
        if (state != KS_RUN) continue;
        const double al = sc[c].alpha, om = sc[c].omega;
        GRID_STRIDE(P, n) {
            x[o + P] += al * ph[o + P] + om * sh[o + P];
            const double y = s[o + P] - om * t[o + P];
            r[o + P] = y;
            acc[2 * c] += y * y;
            acc[2 * c + 1] += r0[o + P] * y;
            if (divtol > 0) acc[6] = fmax(acc[6], fabs(y) * div_weight(ctx, P, two_re));
        }
    }
    double sm[6] = {acc[0], acc[1], acc[2], acc[3], acc[4], acc[5]};
    double dm[1] = {acc[6]};
    block_sum<6>(sm, smem);
    __syncthreads();
    block_max<1>(dm, smem + 192);
    double out[7] = {sm[0], sm[1], sm[2], sm[3], sm[4], sm[5], dm[0]};
    if (publish_partials<7>(out, partials, counter)) {
        double tot[7] = {0, 0, 0, 0, 0, 0, 0};
        for (unsigned b = 0; b < gridDim.x; b++) {
            for (int q = 0; q < 6; q++) tot[q] += ((volatile double *)partials)[b * 7 + q];
            tot[6] = fmax(tot[6], ((volatile double *)partials)[b * 7 + 6]);
        }
        for (int c = 0; c < nc; c++) {
            KScal &st = sc[c];
            if (st.state == KS_HALF) {
                st.rnorm2 = st.snorm2;
                st.iters += 1;
                st.state = KS_DONE;
                continue;
            }
            if (st.state != KS_RUN) continue;
            st.iters += 1;
            st.rnorm2 = tot[2 * c];
            const double rho1 = tot[2 * c + 1];
            st.beta = (rho1 / st.rho) * (st.alpha / st.omega);
            st.rho = rho1;
            const bool ok = divtol > 0 ? tot[6] <= divtol : sqrt(tot[2 * c]) < tol * sqrt(st.bnorm2);
            if (ok) {
                st.state = KS_DONE;
                st.divmax = tot[6];
            } else if (rho1 == 0.0) {
                st.state = KS_BREAKDOWN;
            }
        }
        *counter = 0;
    }
}

// ---------------------------------------------------------- copy (M = I) --
__global__ void k_copy(const long long n, const double *__restrict__ a, double *b) {
    GRID_STRIDE(P, n) b[P] = a[P];
}

// ------------------------------------------------------------ residual --
// r = b - A x for one component; returns ||r||^2 and max weighted |r|.
__global__ void __launch_bounds__(KTHREADS)
k_residual(const OpCtx ctx, const int op, const int comp, const long long n, const double *__restrict__ b,
           const double *__restrict__ x, double *r, const double two_re, double *partials, unsigned int *counter,
           double *out) {
    __shared__ double smem[64];
    double sm[1] = {0}, dm[1] = {0};
    GRID_STRIDE(P, n) {
        const double y = b[P] - op_row(ctx, op, comp, x, P);
        if (r) r[P] = y;
        sm[0] += y * y;
        dm[0] = fmax(dm[0], fabs(y) * div_weight(ctx, P, two_re));
    }
    block_sum<1>(sm, smem);
    __syncthreads();
    block_max<1>(dm, smem + 32);
    double o2[2] = {sm[0], dm[0]};
    if (publish_partials<2>(o2, partials, counter)) {
        double s = 0, m = 0;
        for (unsigned b2 = 0; b2 < gridDim.x; b2++) {
            s += ((volatile double *)partials)[b2 * 2];
            m = fmax(m, ((volatile double *)partials)[b2 * 2 + 1]);
        }
        out[0] = s;
        out[1] = m;
        *counter = 0;
    }
}

__global__ void __launch_bounds__(KTHREADS)
k_apply(const OpCtx ctx, const int op, const int comp, const long long n, const double *__restrict__ x,
        double *y) {
    GRID_STRIDE(P, n) y[P] = op_row(ctx, op, comp, x, P);
}

void apply_operator(cudaStream_t st, const OpCtx &ctx, int op, int comp, const double *x, double *y) {
    k_apply<<<KBLOCKS, KTHREADS, 0, st>>>(ctx, op, comp, ctx.g.ncell, x, y);
    note_launches(1);
}

// -------------------------------------------------------------- driver --
KrylovWork::~KrylovWork() { release(); }

void KrylovWork::release() {
    if (base) cudaFree(base);
    if (scal) cudaFree(scal);
    if (scal_h) cudaFreeHost(scal_h);
    if (partials) cudaFree(partials);
    if (counter) cudaFree(counter);
    base = nullptr;
    scal = nullptr;
    scal_h = nullptr;
    partials = nullptr;
    counter = nullptr;
}

int KrylovWork::allocate(long long ncell, int ncomp, bool precond) {
    release();
    n = ncell;
    nc = ncomp;
    const int nvec = precond ? 8 : 6;
    size_t bytes = sizeof(double) * (size_t)n * nc * nvec;
    if (cudaMalloc(&base, bytes) != cudaSuccess) return -1;
    cudaMemset(base, 0, bytes);
    double *q = base;
    const long long m = n * nc;
    r = q; q += m;
    r0 = q; q += m;
    p = q; q += m;
    v = q; q += m;
    s = q; q += m;
    t = q; q += m;
    if (precond) {
        ph = q; q += m;
        sh = q; q += m;
    } else {
        ph = p;
        sh = s;
    }
    if (cudaMalloc(&scal, sizeof(KScal) * 3) != cudaSuccess) return -1;
    if (cudaMallocHost(&scal_h, sizeof(KScal) * 3) != cudaSuccess) return -1;
    if (cudaMalloc(&partials, sizeof(double) * KBLOCKS * 8) != cudaSuccess) return -1;
    if (cudaMalloc(&counter, sizeof(unsigned int)) != cudaSuccess) return -1;
    cudaMemset(counter, 0, sizeof(unsigned int));
    return 0;
}

static int prof_begin(Prof *p, const char *name) { return p ? p->begin(name) : -1; }
static void prof_end(Prof *p, int t) {
    if (p) p->end(t);
}

static bool all_in(const KScal *s, int nc, int a, int b, int c2) {
    for (int q = 0; q < nc; q++)
        if (s[q].state != a && s[q].state != b && s[q].state != c2) return false;
    return true;
}

int bicgstab(cudaStream_t st, const OpCtx &ctx, int op, KrylovWork &w, const double *b, double *x,
             const SolveParams &prm, Preconditioner *M, SolveReport &rep) {
    const long long n = w.n;
    const int nc = w.nc;
    k_bicg_init<<<KBLOCKS, KTHREADS, 0, st>>>(n, nc, b, x, w.r, w.r0, w.p, w.v, w.scal, w.partials, w.counter);
    note_launches(1);
    const double two_re = 2 * prm.Re;
    int it = 0;
    auto fetch = [&]() {
        cudaMemcpyAsync(w.scal_h, w.scal, sizeof(KScal) * nc, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
    };
    fetch();
    while (!all_in(w.scal_h, nc, KS_DONE, KS_BREAKDOWN, KS_DONE) && it < prm.maxit) {
        it++;
        k_bicg_p<<<KBLOCKS, KTHREADS, 0, st>>>(n, nc, w.r, w.p, w.v, w.scal);
        note_launches(1);
        int tm = -1;
        if (M) {
            tm = prof_begin(prm.prof, "mg_vcycle");
            M->apply(st, w.p, w.ph);
            prof_end(prm.prof, tm);
        }
        tm = prof_begin(prm.prof, op == OP_MOM ? "spmv_mom" : "spmv_p");
        k_bicg_spmv_v<<<KBLOCKS, KTHREADS, 0, st>>>(ctx, op, n, nc, w.ph, w.v, w.r0, w.scal, w.partials, w.counter);
        note_launches(1);
        prof_end(prm.prof, tm);
        k_bicg_s<<<KBLOCKS, KTHREADS, 0, st>>>(ctx, n, nc, w.r, w.v, w.s, w.scal, prm.tol, prm.divtol, two_re,
                                             w.partials, w.counter);
        note_launches(1);
        if (prm.sync_half) {
            fetch();
            if (all_in(w.scal_h, nc, KS_HALF, KS_DONE, KS_BREAKDOWN)) {
                k_bicg_xr<<<KBLOCKS, KTHREADS, 0, st>>>(ctx, n, nc, x, w.r, w.r0, w.ph, w.sh, w.s, w.t, w.scal,
                                                      prm.tol, prm.divtol, two_re, w.partials, w.counter);
                note_launches(1);
                fetch();
                break;
            }
        }
        if (M) {
            tm = prof_begin(prm.prof, "mg_vcycle");
            M->apply(st, w.s, w.sh);
            prof_end(prm.prof, tm);
        }
        tm = prof_begin(prm.prof, op == OP_MOM ? "spmv_mom" : "spmv_p");
        k_bicg_spmv_t<<<KBLOCKS, KTHREADS, 0, st>>>(ctx, op, n, nc, w.sh, w.t, w.s, w.scal, w.partials, w.counter);
        note_launches(1);
        prof_end(prm.prof, tm);
        k_bicg_xr<<<KBLOCKS, KTHREADS, 0, st>>>(ctx, n, nc, x, w.r, w.r0, w.ph, w.sh, w.s, w.t, w.scal, prm.tol,
                                              prm.divtol, two_re, w.partials, w.counter);
        note_launches(1);
        fetch();
    }
    int status = 0;
    for (int c = 0; c < nc; c++) {
        const KScal &s = w.scal_h[c];
        rep.iters[c] = s.iters;
        rep.relres[c] = s.bnorm2 > 0 ? std::sqrt(s.rnorm2 / s.bnorm2) : 0.0;
        rep.divmax[c] = s.divmax;
        if (s.state == KS_BREAKDOWN) status = 2;
        else if (s.state != KS_DONE && status == 0) status = 1;
    }
    return status;
}

double residual_norm(cudaStream_t st, const OpCtx &ctx, int op, int comp, const double *b, const double *x,
                     double *r, double two_re, KrylovWork &w, double *divmax) {
    double *out;
    cudaMalloc(&out, 2 * sizeof(double));
    k_residual<<<KBLOCKS, KTHREADS, 0, st>>>(ctx, op, comp, ctx.g.ncell, b, x, r, two_re, w.partials, w.counter,
                                           out);
    double h[2];
    cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFree(out);
    if (divmax) *divmax = h[1];
    return std::sqrt(h[0]);
}

}  // namespace ibm
