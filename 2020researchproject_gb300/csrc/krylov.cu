// BiCGSTAB on the matrix-free rows of ops.cuh, in FP64 or FP32, and the
// FP64 iterative-refinement driver of the mixed-precision path.
//
// The solver follows hypre's BiCGSTAB as the reference drives it
// (src/ibm3d_fracstep.c:354-379, 649-703): x0 = 0, stop when
// ||b - Ax||_2 / ||b||_2 < tol.  The three momentum components are solved
// together, one Krylov recurrence per component, so each kernel sweeps the
// grid once for all three.  Scalar recurrences (alpha, omega, beta) are
// computed on the device by the last block of each reduction, in FP64;
// reductions combine per-block partials in a fixed order, so results are
// bitwise reproducible and identical between the host loop and the
// recorded (graph) form.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "krylov.h"
#include "prof.h"

namespace ibm {

#define GRID_STRIDE(P, n)                                                              \
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < (n); \
         P += (long long)gridDim.x * blockDim.x)

// Per-thread accumulator type: FP64 for FP64 vectors; FP32 for FP32 vectors
// (each thread adds a handful of products; partials are combined in FP64).
template <typename T> struct AccT;
template <> struct AccT<double> { using type = double; };
template <> struct AccT<float> { using type = float; };
template <> struct AccT<dfloat> { using type = dfloat; };

// 16-byte packs for the streaming vector kernels: with n % 4 == 0 every
// vector (and every component of a 3-component vector) starts on a 16-byte
// boundary, and a thread moves PW elements per load.
template <typename T>
struct alignas(16) Pack {
    T v[16 / sizeof(T)];
};
template <typename T>
constexpr int PW = 16 / sizeof(T);
template <typename T>
__device__ __forceinline__ Pack<T> ldp(const T *p, long long q) {
    return reinterpret_cast<const Pack<T> *>(p)[q];
}
template <typename T>
__device__ __forceinline__ void stp(T *p, long long q, const Pack<T> &x) {
    reinterpret_cast<Pack<T> *>(p)[q] = x;
}
// PW<T> entries of type E (the FP32 p^ and s^ of double-float vectors; a
// Pack<T> when E = T).
template <typename E, int N>
struct alignas(sizeof(E) * N) PackN {
    E v[N];
};
template <typename T, typename E>
__device__ __forceinline__ PackN<E, PW<T>> ldpn(const E *p, long long q) {
    return reinterpret_cast<const PackN<E, PW<T>> *>(p)[q];
}

// Weighted |r| for the divergence criterion (FP32 is ample for a stopping
// test; an FP64 y is rounded on the integer pipe, since an FP64 -> FP32
// conversion instruction runs at the FP64 rate and these kernels are
// FP64-pipe bound).
__device__ __forceinline__ float to_f32(double y) { return d2f_int(y); }
__device__ __forceinline__ float to_f32(float y) { return y; }
__device__ __forceinline__ float to_f32(dfloat y) { return y.hi; }

template <typename T>
__device__ __forceinline__ float divw(const OpT<T> &c, long long P, T y) {
    return c.wdiv[P] * fabsf(to_f32(y));
}

// Stopping test: ||r|| < tol ||b|| (tol > 0) or max weighted |r| <= divtol
// (divtol > 0); either one that is enabled suffices.
// A non-finite residual norm never passes (NaN in the vectors ends the
// solve as a breakdown instead, see the dot-product checks below).
__device__ __forceinline__ bool converged(double rn2, double bn2, double divmax, double tol, double divtol) {
    if (!isfinite(rn2)) return false;
    return (tol > 0 && sqrt(rn2) < tol * sqrt(bn2)) || (divtol > 0 && divmax <= divtol);
}

__device__ __forceinline__ void set_loop(const LoopCtl &lc, bool cont) {
    if (lc.use) cudaGraphSetConditional(lc.h, cont ? 1u : 0u);
}

// Reduction tail shared by the kernels below: block-level combine, then
// the last block reduces all partials (NS sums first, then maxima) and
// thread 0 runs `fin(tot)`.
template <int NV, int NS, typename A, typename Fin>
__device__ __forceinline__ void reduce_and_finish(const A (&v)[NV], double *smem, double *partials,
                                                  unsigned int *counter, Fin fin) {
    static_assert(NS >= 1 && NS <= NV, "at least one summed entry");
    double out[NV];
    block_reduce<NV, NS>(v, out, smem);
    if (!publish_partials<NV>(out, partials, counter)) return;
    double tot[NV];
    reduce_partials<NV, NS>(partials, gridDim.x, tot, smem);
    if (threadIdx.x == 0) {
        fin(tot);
        *counter = 0;
    }
}

// ---------------------------------------------------------------- init --
// x = 0, r = b, ||b||^2; the first p update of the loop sets p = r0 = r
// (restart flag), so nothing reads p, r0 or v before it writes them.  The
// stopping test of the solve is
// fixed here: (tol, divtol) as given, or, for the inner solve of a
// refinement cycle (outer != null), derived from the outer state: the
// relative tolerance is raised to what the outer FP64 test still needs
// (half of it, as margin) and the divergence bound is expressed in the
// scaled units of the inner right-hand side.  b may be FP64 under
// double-float vectors (B = double, T = dfloat), converted as it is read.
template <typename T, int NC, typename B = T>
__global__ void __launch_bounds__(KTHREADS)
k_bicg_init(const long long n, const B *__restrict__ b, T *x, T *r, KScal *sc, double *partials,
            unsigned int *counter, const double tol, const double divtol, const IRScal *__restrict__ outer,
            const double outer_tol, const double outer_divtol, const LoopCtl lc) {
    pdl_enter();
    __shared__ double smem[32 * NC];
    typename AccT<T>::type a[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) a[c] = 0;
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const long long o = c * n;
        GRID_STRIDE(P, n) {
            const T bv = (T)b[o + P];
            x[o + P] = 0;
            r[o + P] = bv;
            mac(a[c], bv, bv);
        }
    }
    reduce_and_finish<NC, NC>(a, smem, partials, counter, [&](const double *tot) {
        bool run = false;
        for (int c = 0; c < NC; c++) {
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
            s.restart = 1;   // the first p update sets p = r0 = r
            s.tol = tol;
            s.divtol = divtol;
            if (outer) {
                const IRScal &o = outer[c];
                if (outer_tol > 0 && o.rnorm2 > 0) s.tol = fmax(tol, 0.5 * outer_tol * sqrt(o.bnorm2 / o.rnorm2));
                s.divtol = (outer_divtol > 0 && NC == 1) ? 0.5 * outer_divtol * o.scale : 0.0;
            }
            run = run || s.state == KS_RUN;
        }
        set_loop(lc, run);
    });
}

// ------------------------------------------------- p = r + beta (p - w v) --
template <typename T, int NC, bool VEC>
__global__ void __launch_bounds__(KTHREADS)
k_bicg_p(const long long n, const T *__restrict__ r, T *__restrict__ p, const T *__restrict__ v, T *__restrict__ r0,
         const KScal *sc) {
    pdl_enter();
#pragma unroll
    for (int c = 0; c < NC; c++) {
        if (sc[c].state != KS_RUN) continue;
        const T beta = (T)sc[c].beta, om = (T)sc[c].omega;
        const long long o = c * n;
        if (sc[c].restart) {   // the recurrence restarts from the current residual
            GRID_STRIDE(P, n) {
                const T rv = r[o + P];
                p[o + P] = rv;
                r0[o + P] = rv;
            }
            continue;
        }
        if (VEC) {
            const long long np = n / PW<T>, op = o / PW<T>;
            GRID_STRIDE(q, np) {
                const Pack<T> rr = ldp(r, op + q), vv = ldp(v, op + q);
                Pack<T> pp = ldp(p, op + q);
#pragma unroll
                for (int l = 0; l < PW<T>; l++) pp.v[l] = p_update(rr.v[l], beta, pp.v[l], om, vv.v[l]);
                stp(p, op + q, pp);
            }
        } else {
            GRID_STRIDE(P, n) { p[o + P] = p_update(r[o + P], beta, p[o + P], om, v[o + P]); }
        }
    }
}

// Calls f(c, P, i, q) for every interior row of this thread's column and
// g(c, P) for its outer row, for each running component c.  Components
// one after the other (each component's rows in i order): only one
// component's loads are live at a time, which keeps the 3-component
// kernels' registers, and so their occupancy, in check.
template <typename T, int NC, typename FI, typename FO>
__device__ __forceinline__ void sweep_rows(const OpT<T> &A, const bool (&run)[NC], FI fi, FO fo) {
    int i0, i1, j, k;
    if (sweep_column(A.sw, A.g, i0, i1, j, k)) {
        if (j >= A.g.ny || k >= A.g.nz) return;
        const Column<T> q = column(A, j, k);
        const long long P0 = cidx(A.g, i0, j, k);
#pragma unroll
        for (int c = 0; c < NC; c++) {
            if (!run[c]) continue;
            long long P = P0;
#pragma unroll 2
            for (int i = i0; i < i1; i++, P += A.g.sx) fi(c, P, i, q);
        }
    } else {
        const int t = sweep_outer(A.sw);
        if (t >= A.sw.nout) return;
        const long long P = A.sw.outer[t];
#pragma unroll
        for (int c = 0; c < NC; c++)
            if (run[c]) fo(c, P);
    }
}

// The same with x holding an initial guess: r = b - A x (p = r0 = r at the
// first p update),
// ||b||^2 (the relative test stays relative to b; to the initial residual
// where b = 0, whose solution x = 0 a relative test to 0 would never
// reach), ||r||^2 and the divergence max of r; a guess that already passes
// the stopping test ends the solve before its first iteration.  b as in
// k_bicg_init.
template <typename T, int NC, typename B = T>
__global__ void __launch_bounds__(SW_THREADS, std::is_same<T, dfloat>::value ? 4 : 1)
k_bicg_init_guess(const OpT<T> A, const int op, const long long n, const B *__restrict__ b, const T *__restrict__ x,
                  T *r, KScal *sc, double *partials, unsigned int *counter, const double tol,
                  const double divtol, const LoopCtl lc) {
    pdl_enter();
    __shared__ double smem[32 * (2 * NC + 1)];
    typename AccT<T>::type a[2 * NC + 1];
    bool run[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        a[c] = a[NC + c] = 0;
        run[c] = true;
    }
    float dmax = 0.0f;
    auto put = [&](int c, long long P, T bv, T y) {
        r[c * n + P] = y;
        mac(a[c], bv, bv);
        mac(a[NC + c], y, y);
        if (divtol > 0) dmax = fmaxf(dmax, divw(A, P, y));
    };
    sweep_rows<T, NC>(
        A, run,
        [&](int c, long long P, int i, const Column<T> &q) {
            const T bv = (T)b[c * n + P];
            put(c, P, bv, bv - interior_row(A, op, x + c * n, P, i, q));
        },
        [&](int c, long long P) {
            const T bv = (T)b[c * n + P];
            put(c, P, bv, bv - op_row(A, op, c, x + c * n, P));
        });
    a[2 * NC] = dmax;
    reduce_and_finish<2 * NC + 1, 2 * NC>(a, smem, partials, counter, [&](const double *tot) {
        bool go = false;
        for (int c = 0; c < NC; c++) {
            KScal &s = sc[c];
            s.bnorm2 = tot[c] > 0.0 ? tot[c] : tot[NC + c];
            s.rnorm2 = tot[NC + c];
            s.rho = tot[NC + c];
            s.alpha = 1.0;
            s.omega = 1.0;
            s.beta = 0.0;
            s.iters = 0;
            s.tol = tol;
            s.divtol = divtol;
            s.divmax = tot[2 * NC];
            s.restart = 1;   // the first p update sets p = r0 = r
            const bool done = tot[NC + c] == 0.0 || converged(tot[NC + c], s.bnorm2, tot[2 * NC], tol, divtol);
            s.state = done ? KS_DONE : KS_RUN;
            go = go || !done;
        }
        set_loop(lc, go);
    });
}

// ------------------------------------------- v = A ph, alpha = rho/(r0,v) --
template <typename T, int NC>
__global__ void __launch_bounds__(SW_THREADS, (sizeof(T) == 4 || NC == 1) ? 4 : 2)
k_bicg_spmv_v(const OpT<T> A, const int op, const long long n, const typename PrecT<T>::type *__restrict__ ph,
              T *__restrict__ v,
              const T *__restrict__ r0, KScal *sc, double *partials, unsigned int *counter) {
    pdl_enter();
    __shared__ double smem[32 * NC];
    typename AccT<T>::type a[NC];
    bool run[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        a[c] = 0;
        run[c] = sc[c].state == KS_RUN;
    }
    sweep_rows<T, NC>(
        A, run,
        [&](int c, long long P, int i, const Column<T> &q) {
            const long long o = c * n;
            const T y = interior_row(A, op, ph + o, P, i, q);
            v[o + P] = y;
            mac(a[c], r0[o + P], y);
        },
        [&](int c, long long P) {
            const long long o = c * n;
            const T y = op_row(A, op, c, ph + o, P);
            v[o + P] = y;
            mac(a[c], r0[o + P], y);
        });
    reduce_and_finish<NC, NC>(a, smem, partials, counter, [&](const double *tot) {
        for (int c = 0; c < NC; c++) {
            KScal &s = sc[c];
            s.restart = 0;   // k_bicg_p, the only reader, has finished
            if (s.state != KS_RUN) continue;
            // A zero or non-finite (r0, v) ends the solve: NaN or Inf in
            // the operands would otherwise run it to its iteration cap.
            if (tot[c] == 0.0 || !isfinite(tot[c])) {
                s.state = KS_BREAKDOWN;
                continue;
            }
            s.alpha = s.rho / tot[c];
        }
    });
}

// ------------------------------------------------------- s = r - alpha v --
template <typename T, int NC, bool VEC>
__global__ void __launch_bounds__(KTHREADS)
k_bicg_s(const OpT<T> A, const long long n, const T *__restrict__ r, const T *__restrict__ v, T *__restrict__ s,
         KScal *sc, double *partials, unsigned int *counter) {
    pdl_enter();
    __shared__ double smem[32 * (NC + 1)];
    typename AccT<T>::type a[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) a[c] = 0;
    float dmax = 0.0f;
    const bool want_div = sc[0].divtol > 0;
#pragma unroll
    for (int c = 0; c < NC; c++) {
        if (sc[c].state != KS_RUN) continue;
        const T al = (T)sc[c].alpha;
        const long long o = c * n;
        if (VEC) {
            const long long np = n / PW<T>, op = o / PW<T>;
            GRID_STRIDE(q, np) {
                const Pack<T> rr = ldp(r, op + q), vv = ldp(v, op + q);
                Pack<T> ss;
#pragma unroll
                for (int l = 0; l < PW<T>; l++) {
                    const T y = sub_mul(rr.v[l], al, vv.v[l]);
                    ss.v[l] = y;
                    mac(a[c], y, y);
                    if (want_div) dmax = fmaxf(dmax, divw(A, q * PW<T> + l, y));
                }
                stp(s, op + q, ss);
            }
        } else {
            GRID_STRIDE(P, n) {
                const T y = sub_mul(r[o + P], al, v[o + P]);
                s[o + P] = y;
                mac(a[c], y, y);
                if (want_div) dmax = fmaxf(dmax, divw(A, P, y));
            }
        }
    }
    typename AccT<T>::type acc[NC + 1];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = a[c];
    acc[NC] = dmax;
    reduce_and_finish<NC + 1, NC>(acc, smem, partials, counter, [&](const double *tot) {
        for (int c = 0; c < NC; c++) {
            KScal &st = sc[c];
            if (st.state != KS_RUN) continue;
            st.snorm2 = tot[c];
            if (converged(tot[c], st.bnorm2, tot[NC], st.tol, st.divtol)) {
                st.state = KS_HALF;
                st.divmax = tot[NC];
            }
        }
    });
}

// --------------------------------------- t = A sh, omega = (t,s)/(t,t) --
template <typename T, int NC>
__global__ void __launch_bounds__(SW_THREADS, (sizeof(T) == 4 || NC == 1) ? 4 : 2)
k_bicg_spmv_t(const OpT<T> A, const int op, const long long n, const typename PrecT<T>::type *__restrict__ sh,
              T *__restrict__ t,
              const T *__restrict__ s, KScal *sc, double *partials, unsigned int *counter) {
    pdl_enter();
    __shared__ double smem[32 * 2 * NC];
    typename AccT<T>::type a[2 * NC];
    bool run[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        a[2 * c] = a[2 * c + 1] = 0;
        run[c] = sc[c].state == KS_RUN;
    }
    sweep_rows<T, NC>(
        A, run,
        [&](int c, long long P, int i, const Column<T> &q) {
            const long long o = c * n;
            const T y = interior_row(A, op, sh + o, P, i, q);
            t[o + P] = y;
            mac(a[2 * c], y, s[o + P]);
            mac(a[2 * c + 1], y, y);
        },
        [&](int c, long long P) {
            const long long o = c * n;
            const T y = op_row(A, op, c, sh + o, P);
            t[o + P] = y;
            mac(a[2 * c], y, s[o + P]);
            mac(a[2 * c + 1], y, y);
        });
    reduce_and_finish<2 * NC, 2 * NC>(a, smem, partials, counter, [&](const double *tot) {
        for (int c = 0; c < NC; c++) {
            KScal &st = sc[c];
            if (st.state != KS_RUN) continue;
            if (tot[2 * c + 1] == 0.0 || !isfinite(tot[2 * c + 1]) || !isfinite(tot[2 * c])) {
                st.omega = 0.0;
                st.state = KS_BREAKDOWN;
                continue;
            }
            st.omega = tot[2 * c] / tot[2 * c + 1];
        }
    });
}

// ------------------- x += alpha ph + omega sh, r = s - omega t, new rho --
// Ends the iteration: sets the loop condition (some component still
// running and below maxit).
template <typename T, int NC, bool VEC>
__global__ void __launch_bounds__(KTHREADS)
k_bicg_xr(const OpT<T> A, const long long n, T *__restrict__ x, T *__restrict__ r, const T *__restrict__ r0,
          const typename PrecT<T>::type *__restrict__ ph, const typename PrecT<T>::type *__restrict__ sh,
          const T *__restrict__ s, const T *__restrict__ t,
          KScal *sc, double *partials, unsigned int *counter, const int maxit, const LoopCtl lc) {
    pdl_enter();
    __shared__ double smem[32 * (2 * NC + 1)];
    typename AccT<T>::type a[2 * NC];
#pragma unroll
    for (int q = 0; q < 2 * NC; q++) a[q] = 0;
    float dmax = 0.0f;
    const bool want_div = sc[0].divtol > 0;
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const int state = sc[c].state;
        const long long o = c * n;
        if (state == KS_HALF) {
            // Converged on s: x += alpha ph, r = s.
            const T al = (T)sc[c].alpha;
            GRID_STRIDE(P, n) {
                x[o + P] += al * T(ph[o + P]);
                r[o + P] = s[o + P];
            }
            continue;
        }
        if (state != KS_RUN) continue;
        const T al = (T)sc[c].alpha, om = (T)sc[c].omega;
        if (VEC) {
            const long long np = n / PW<T>, op = o / PW<T>;
            GRID_STRIDE(q, np) {
                Pack<T> xx = ldp(x, op + q);
                const auto pp = ldpn<T>(ph, op + q), ss = ldpn<T>(sh, op + q);
                const Pack<T> s0 = ldp(s, op + q), tt = ldp(t, op + q), rr0 = ldp(r0, op + q);
                Pack<T> rr;
#pragma unroll
                for (int l = 0; l < PW<T>; l++) {
                    xx.v[l] = add_mul2(xx.v[l], al, T(pp.v[l]), om, T(ss.v[l]));
                    const T y = sub_mul(s0.v[l], om, tt.v[l]);
                    rr.v[l] = y;
                    mac(a[2 * c], y, y);
                    mac(a[2 * c + 1], rr0.v[l], y);
                    if (want_div) dmax = fmaxf(dmax, divw(A, q * PW<T> + l, y));
                }
                stp(x, op + q, xx);
                stp(r, op + q, rr);
            }
        } else {
            GRID_STRIDE(P, n) {
                x[o + P] = add_mul2(x[o + P], al, T(ph[o + P]), om, T(sh[o + P]));
                const T y = sub_mul(s[o + P], om, t[o + P]);
                r[o + P] = y;
                mac(a[2 * c], y, y);
                mac(a[2 * c + 1], r0[o + P], y);
                if (want_div) dmax = fmaxf(dmax, divw(A, P, y));
            }
        }
    }
    typename AccT<T>::type acc[2 * NC + 1];
#pragma unroll
    for (int q = 0; q < 2 * NC; q++) acc[q] = a[q];
    acc[2 * NC] = dmax;
    reduce_and_finish<2 * NC + 1, 2 * NC>(acc, smem, partials, counter, [&](const double *tot) {
        bool run = false;
        for (int c = 0; c < NC; c++) {
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
            if (converged(tot[2 * c], st.bnorm2, tot[2 * NC], st.tol, st.divtol)) {
                st.state = KS_DONE;
                st.divmax = tot[2 * NC];
            } else if (!isfinite(rho1) || !isfinite(tot[2 * c])) {
                st.state = KS_BREAKDOWN;
            } else if (st.iters % KRESTART == 0 || rho1 == 0.0) {
                st.restart = 1;
                st.rho = tot[2 * c];
                st.beta = 0.0;
            }
            run = run || (st.state == KS_RUN && st.iters < maxit);
        }
        set_loop(lc, run);
    });
}

template <typename T>
__global__ void __launch_bounds__(SW_THREADS)
k_apply(const OpT<T> A, const int op, const int comp, const T *__restrict__ x, T *y) {
    pdl_enter();
    const bool run[1] = {true};
    sweep_rows<T, 1>(
        A, run, [&](int, long long P, int i, const Column<T> &q) { y[P] = interior_row(A, op, x, P, i, q); },
        [&](int, long long P) { y[P] = op_row(A, op, comp, x, P); });
}

// ------------------------------------------------- true-residual check --
// Runs after k_bicg_xr of a one-component solve and acts only when that
// iteration ended the solve (KS_DONE): r = b - A x from the solution
// itself, and the stopping test on it.  A pass keeps the solve done (the
// reported norms become the true residual's); a miss restarts the
// recurrence from the true residual (r0 = p = r at the next p update) and
// keeps the loop going below maxit.  Used by the double-float solve, whose
// recursive residual can drift from the true one by more than the
// divergence bound's margin over a long solve.
template <typename T, typename B>
__global__ void __launch_bounds__(SW_THREADS, std::is_same<T, dfloat>::value ? 4 : 1)
k_bicg_verify(const OpT<T> A, const int op, const long long n, const B *__restrict__ b, const T *__restrict__ x,
              T *r, KScal *sc, double *partials, unsigned int *counter, const int maxit, const LoopCtl lc) {
    pdl_enter();
    if (sc[0].state != KS_DONE) return;   // the same value in every block: written only by the last one below
    __shared__ double smem[32 * 2];
    typename AccT<T>::type a[1] = {0};
    float dmax = 0.0f;
    const bool run[1] = {true};
    const bool want_div = sc[0].divtol > 0;
    auto put = [&](long long P, T y) {
        r[P] = y;
        mac(a[0], y, y);
        if (want_div) dmax = fmaxf(dmax, divw(A, P, y));
    };
    sweep_rows<T, 1>(
        A, run, [&](int, long long P, int i, const Column<T> &q) { put(P, (T)b[P] - interior_row(A, op, x, P, i, q)); },
        [&](int, long long P) { put(P, (T)b[P] - op_row(A, op, 0, x, P)); });
    typename AccT<T>::type acc[2] = {a[0], dmax};
    reduce_and_finish<2, 1>(acc, smem, partials, counter, [&](const double *tot) {
        KScal &st = sc[0];
        st.rnorm2 = tot[0];
        if (!isfinite(tot[0])) {
            st.state = KS_BREAKDOWN;
            set_loop(lc, false);
            return;
        }
        if (converged(tot[0], st.bnorm2, tot[1], st.tol, st.divtol)) {
            st.divmax = tot[1];
            set_loop(lc, false);
            return;
        }
        st.state = KS_RUN;
        st.restart = 1;
        st.rho = tot[0];
        st.beta = 0.0;
        set_loop(lc, st.iters < maxit);
    });
}

// --------------------------------------------- iterative refinement (FP64) --
// r = b - A x (or r = b while x is still zero), with per-component ||r||^2,
// max|r| and the divergence max; the last block derives each component's
// state, the FP32 scale 1/max|r| (0 for converged components), counts the
// cycle and sets the outer loop condition.  mode: IR_NEXT (a later cycle),
// IR_ZERO (the first, x = 0), IR_GUESS (the first, x an initial guess);
// the first also records ||b||^2 for the relative test.
enum { IR_NEXT = 0, IR_ZERO = 1, IR_GUESS = 2 };

template <int NC>
__global__ void __launch_bounds__(SW_THREADS)
k_ir_residual(const OpT<double> A, const int op, const long long n, const double *__restrict__ b,
              const double *__restrict__ x, double *r, const int mode, IRScal *sc, const double tol,
              const double divtol, const int max_outer, double *partials, unsigned int *counter, const LoopCtl lc) {
    pdl_enter();
    constexpr int NV = 3 * NC + 1;
    __shared__ double smem[32 * NV];
    const bool x_zero = mode == IR_ZERO, first = mode != IR_NEXT;
    double sm[2 * NC], mx[NC + 1];  // ||r||^2, ||b||^2 (first cycle only); max|r|, divergence max
    bool run[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        sm[c] = sm[NC + c] = 0;
        mx[c] = 0;
        run[c] = true;
    }
    mx[NC] = 0;
    auto acc = [&](int c, long long P, double y) {
        const double bv = b[c * n + P];
        r[c * n + P] = y;
        sm[c] += y * y;
        if (first) sm[NC + c] += bv * bv;
        mx[c] = fmax(mx[c], fabs(y));
        if (divtol > 0) mx[NC] = fmax(mx[NC], (double)divw(A, P, y));
    };
    sweep_rows<double, NC>(
        A, run,
        [&](int c, long long P, int i, const Column<double> &q) {
            const long long o = c * n;
            acc(c, P, x_zero ? b[o + P] : b[o + P] - interior_row(A, op, x + o, P, i, q));
        },
        [&](int c, long long P) {
            const long long o = c * n;
            acc(c, P, x_zero ? b[o + P] : b[o + P] - op_row(A, op, c, x + o, P));
        });
    double v[NV];
#pragma unroll
    for (int q = 0; q < 2 * NC; q++) v[q] = sm[q];
#pragma unroll
    for (int q = 0; q <= NC; q++) v[2 * NC + q] = mx[q];
    reduce_and_finish<NV, 2 * NC>(v, smem, partials, counter, [&](const double *tot) {
        bool go = false;
        for (int c = 0; c < NC; c++) {
            IRScal &s = sc[c];
            if (first) {
                s.bnorm2 = tot[NC + c];
                s.outer = 0;
                s.inner = 0;
            } else {
                s.outer += 1;
            }
            s.rnorm2 = tot[c];
            s.rmax = tot[2 * NC + c];
            s.divmax = tot[3 * NC];
            const bool done = s.bnorm2 == 0.0 || converged(tot[c], s.bnorm2, tot[3 * NC], tol, divtol);
            s.state = done ? KS_DONE : KS_RUN;
            s.scale = (done || s.rmax == 0.0) ? 0.0 : 1.0 / s.rmax;
            go = go || (!done && s.outer < max_outer);
        }
        set_loop(lc, go);
    });
}

template <int NC>
__global__ void __launch_bounds__(KTHREADS)
k_ir_to32(const long long n, const double *__restrict__ r, const IRScal *sc, float *b32) {
    pdl_enter();
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const double s = sc[c].scale;
        const long long o = c * n;
        GRID_STRIDE(P, n) b32[o + P] = d2f_int(r[o + P] * s);
    }
}

// x += e / scale; counts the inner iterations of the cycle.
template <int NC>
__global__ void __launch_bounds__(KTHREADS)
k_ir_update(const long long n, double *x, const float *__restrict__ e, IRScal *sc, const KScal *__restrict__ inner) {
    pdl_enter();
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const double s = sc[c].scale;
        if (s == 0.0) continue;
        const double inv = 1.0 / s;
        const long long o = c * n;
        GRID_STRIDE(P, n) x[o + P] += (double)e[o + P] * inv;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (int c = 0; c < NC; c++) sc[c].inner += inner[c].iters;
}

// ------------------------------------------------------------ workspace --
template <typename T>
void KrylovWork<T>::release() {
    if (!owner) {   // a view: the buffers belong to another work
        *this = KrylovWork<T>();
        return;
    }
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

template <typename T>
int KrylovWork<T>::allocate(long long ncell, int ncomp, bool precond, int maxblocks) {
    release();
    n = ncell;
    nc = ncomp;
    nblk = vector_blocks(ncell);
    const int nvec = precond ? 8 : 6;
    const size_t bytes = sizeof(T) * (size_t)n * nc * nvec;
    if (cudaMalloc(&base, bytes) != cudaSuccess) return -1;
    cudaMemset(base, 0, bytes);
    T *q = base;
    const long long m = n * nc;
    r = q; q += m;
    r0 = q; q += m;
    p = q; q += m;
    v = q; q += m;
    s = q; q += m;
    t = q; q += m;
    if (precond) {
        ph = reinterpret_cast<PT *>(q); q += m;
        sh = reinterpret_cast<PT *>(q); q += m;
    } else if constexpr (std::is_same<PT, T>::value) {
        ph = p;
        sh = s;
    }
    if (cudaMalloc(&scal, sizeof(KScal) * 3) != cudaSuccess) return -1;
    cudaMemset(scal, 0, sizeof(KScal) * 3);
    if (cudaMallocHost(&scal_h, sizeof(KScal) * 3) != cudaSuccess) return -1;
    if (cudaMalloc(&partials, sizeof(double) * std::max(nblk, maxblocks) * 10) != cudaSuccess) return -1;
    if (cudaMalloc(&counter, sizeof(unsigned int)) != cudaSuccess) return -1;
    cudaMemset(counter, 0, sizeof(unsigned int));
    return 0;
}

template struct KrylovWork<double>;
template struct KrylovWork<float>;
template void KrylovWork<dfloat>::release();

KrylovWork<dfloat> dfloat_view(const KrylovWork<double> &w) {
    static_assert(sizeof(dfloat) == sizeof(double), "double-float vectors take the FP64 vectors' place");
    KrylovWork<dfloat> v;
    v.owner = false;
    v.n = w.n;
    v.nc = w.nc;
    v.nblk = w.nblk;
    auto as = [](double *q) { return reinterpret_cast<dfloat *>(q); };
    v.base = as(w.base);
    v.r = as(w.r);
    v.r0 = as(w.r0);
    v.p = as(w.p);
    v.v = as(w.v);
    v.s = as(w.s);
    v.t = as(w.t);
    v.ph = reinterpret_cast<float *>(w.ph);
    v.sh = reinterpret_cast<float *>(w.sh);
    v.scal = w.scal;
    v.scal_h = w.scal_h;
    v.partials = w.partials;
    v.counter = w.counter;
    return v;
}

void IRWork::release() {
    if (r) cudaFree(r);
    if (b32) cudaFree(b32);
    if (e32) cudaFree(e32);
    if (scal) cudaFree(scal);
    if (scal_h) cudaFreeHost(scal_h);
    if (partials) cudaFree(partials);
    if (counter) cudaFree(counter);
    r = nullptr;
    b32 = e32 = nullptr;
    scal = scal_h = nullptr;
    partials = nullptr;
    counter = nullptr;
    inner.release();
}

int IRWork::allocate(long long ncell, int ncomp, bool precond, int maxblocks) {
    release();
    n = ncell;
    nc = ncomp;
    nblk = vector_blocks(ncell);
    const size_t m = (size_t)n * nc;
    if (cudaMalloc(&r, sizeof(double) * m) != cudaSuccess) return -1;
    if (cudaMalloc(&b32, sizeof(float) * m) != cudaSuccess) return -1;
    if (cudaMalloc(&e32, sizeof(float) * m) != cudaSuccess) return -1;
    if (cudaMalloc(&scal, sizeof(IRScal) * 3) != cudaSuccess) return -1;
    cudaMemset(scal, 0, sizeof(IRScal) * 3);
    if (cudaMallocHost(&scal_h, sizeof(IRScal) * 3) != cudaSuccess) return -1;
    if (cudaMalloc(&partials, sizeof(double) * std::max(nblk, maxblocks) * 10) != cudaSuccess) return -1;
    if (cudaMalloc(&counter, sizeof(unsigned int)) != cudaSuccess) return -1;
    cudaMemset(counter, 0, sizeof(unsigned int));
    return inner.allocate(ncell, ncomp, precond, maxblocks);
}

// ------------------------------------------------------------ launches --
static int prof_begin(Prof *p, const char *name) { return p ? p->begin(name) : -1; }
static void prof_end(Prof *p, int t) {
    if (p) p->end(t);
}

template <typename SC>
static bool all_in(const SC *s, int nc, int a, int b, int c2) {
    for (int q = 0; q < nc; q++)
        if (s[q].state != a && s[q].state != b && s[q].state != c2) return false;
    return true;
}

template <typename T, typename B>
static void launch_init(cudaStream_t st, KrylovWork<T> &w, const B *b, T *x, double tol, double divtol,
                        const IRScal *outer, double outer_tol, double outer_divtol, LoopCtl lc) {
    if (w.nc == 3)
        launch_pdl(k_bicg_init<T, 3, B>, w.nblk, KTHREADS, 0, st, w.n, b, x, w.r, w.scal, w.partials,
                                                       w.counter, tol, divtol, outer, outer_tol, outer_divtol, lc);
    else
        launch_pdl(k_bicg_init<T, 1, B>, w.nblk, KTHREADS, 0, st, w.n, b, x, w.r, w.scal, w.partials,
                                                       w.counter, tol, divtol, outer, outer_tol, outer_divtol, lc);
    note_launches(1);
}

template <typename T, typename B>
static void launch_init_guess(cudaStream_t st, const OpT<T> &A, int op, KrylovWork<T> &w, const B *b, const T *x,
                              double tol, double divtol, LoopCtl lc) {
    if (w.nc == 3)
        launch_pdl(k_bicg_init_guess<T, 3, B>, A.sw.nblocks, SW_THREADS, 0, st, A, op, w.n, b, x, w.r, w.scal,
                   w.partials, w.counter, tol, divtol, lc);
    else
        launch_pdl(k_bicg_init_guess<T, 1, B>, A.sw.nblocks, SW_THREADS, 0, st, A, op, w.n, b, x, w.r, w.scal,
                   w.partials, w.counter, tol, divtol, lc);
    note_launches(1);
}

// p update, preconditioner, v = A ph, s = r - alpha v.
template <typename T>
static void first_half(cudaStream_t st, const OpT<T> &A, int op, KrylovWork<T> &w, Preconditioner<T> *M, Prof *pf) {
    const long long n = w.n;
    const int nc = w.nc;
    const int *gate = nc == 1 ? &w.scal[0].state : nullptr;
    const bool vec = n % 4 == 0;
    if (nc == 3 && vec) launch_pdl(k_bicg_p<T, 3, true>, w.nblk, KTHREADS, 0, st, n, w.r, w.p, w.v, w.r0, w.scal);
    else if (nc == 3) launch_pdl(k_bicg_p<T, 3, false>, w.nblk, KTHREADS, 0, st, n, w.r, w.p, w.v, w.r0, w.scal);
    else if (vec) launch_pdl(k_bicg_p<T, 1, true>, w.nblk, KTHREADS, 0, st, n, w.r, w.p, w.v, w.r0, w.scal);
    else launch_pdl(k_bicg_p<T, 1, false>, w.nblk, KTHREADS, 0, st, n, w.r, w.p, w.v, w.r0, w.scal);
    note_launches(1);
    if (M) {
        const int tm = prof_begin(pf, "mg_vcycle");
        M->apply(st, w.p, w.ph, gate);
        prof_end(pf, tm);
    }
    const int tm = prof_begin(pf, op == OP_MOM ? "spmv_mom" : "spmv_p");
    if (nc == 3)
        launch_pdl(k_bicg_spmv_v<T, 3>, A.sw.nblocks, SW_THREADS, 0, st, A, op, n, w.phat(M), w.v, w.r0, w.scal, w.partials,
                                                                w.counter);
    else
        launch_pdl(k_bicg_spmv_v<T, 1>, A.sw.nblocks, SW_THREADS, 0, st, A, op, n, w.phat(M), w.v, w.r0, w.scal, w.partials,
                                                                w.counter);
    note_launches(1);
    prof_end(pf, tm);
    if (nc == 3 && vec) launch_pdl(k_bicg_s<T, 3, true>, w.nblk, KTHREADS, 0, st, A, n, w.r, w.v, w.s, w.scal, w.partials, w.counter);
    else if (nc == 3) launch_pdl(k_bicg_s<T, 3, false>, w.nblk, KTHREADS, 0, st, A, n, w.r, w.v, w.s, w.scal, w.partials, w.counter);
    else if (vec) launch_pdl(k_bicg_s<T, 1, true>, w.nblk, KTHREADS, 0, st, A, n, w.r, w.v, w.s, w.scal, w.partials, w.counter);
    else launch_pdl(k_bicg_s<T, 1, false>, w.nblk, KTHREADS, 0, st, A, n, w.r, w.v, w.s, w.scal, w.partials, w.counter);
    note_launches(1);
}

// Preconditioner, t = A sh (both skipped by converged components).
template <typename T>
static void second_half(cudaStream_t st, const OpT<T> &A, int op, KrylovWork<T> &w, Preconditioner<T> *M, Prof *pf) {
    const int *gate = w.nc == 1 ? &w.scal[0].state : nullptr;
    if (M) {
        const int tm = prof_begin(pf, "mg_vcycle");
        M->apply(st, w.s, w.sh, gate);
        prof_end(pf, tm);
    }
    const int tm = prof_begin(pf, op == OP_MOM ? "spmv_mom" : "spmv_p");
    if (w.nc == 3)
        launch_pdl(k_bicg_spmv_t<T, 3>, A.sw.nblocks, SW_THREADS, 0, st, A, op, w.n, w.shat(M), w.t, w.s, w.scal, w.partials,
                                                                w.counter);
    else
        launch_pdl(k_bicg_spmv_t<T, 1>, A.sw.nblocks, SW_THREADS, 0, st, A, op, w.n, w.shat(M), w.t, w.s, w.scal, w.partials,
                                                                w.counter);
    note_launches(1);
    prof_end(pf, tm);
}

template <typename T>
static void launch_xr(cudaStream_t st, const OpT<T> &A, KrylovWork<T> &w, T *x, int maxit, const void *M,
                      LoopCtl lc) {
#define XR_ARGS A, w.n, x, w.r, w.r0, w.phat(M), w.shat(M), w.s, w.t, w.scal, w.partials, w.counter, maxit, lc
    const bool vec = w.n % 4 == 0;
    if (w.nc == 3 && vec) launch_pdl(k_bicg_xr<T, 3, true>, w.nblk, KTHREADS, 0, st, XR_ARGS);
    else if (w.nc == 3) launch_pdl(k_bicg_xr<T, 3, false>, w.nblk, KTHREADS, 0, st, XR_ARGS);
    else if (vec) launch_pdl(k_bicg_xr<T, 1, true>, w.nblk, KTHREADS, 0, st, XR_ARGS);
    else launch_pdl(k_bicg_xr<T, 1, false>, w.nblk, KTHREADS, 0, st, XR_ARGS);
#undef XR_ARGS
    note_launches(1);
}

template <typename T, typename B>
static void launch_verify(cudaStream_t st, const OpT<T> &A, int op, KrylovWork<T> &w, const B *b, const T *x,
                          int maxit, LoopCtl lc) {
    launch_pdl(k_bicg_verify<T, B>, A.sw.nblocks, SW_THREADS, 0, st, A, op, w.n, b, x, w.r, w.scal, w.partials,
               w.counter, maxit, lc);
    note_launches(1);
}

static void launch_residual(cudaStream_t st, const OpT<double> &A64, int op, IRWork &w, const double *b,
                            const double *x, int mode, const SolveParams &prm, LoopCtl lc) {
    if (w.nc == 3)
        launch_pdl(k_ir_residual<3>, A64.sw.nblocks, SW_THREADS, 0, st, A64, op, w.n, b, x, w.r, mode, w.scal, prm.tol,
                                                               prm.divtol, prm.max_outer, w.partials, w.counter, lc);
    else
        launch_pdl(k_ir_residual<1>, A64.sw.nblocks, SW_THREADS, 0, st, A64, op, w.n, b, x, w.r, mode, w.scal, prm.tol,
                                                               prm.divtol, prm.max_outer, w.partials, w.counter, lc);
    note_launches(1);
}

static void launch_to32(cudaStream_t st, IRWork &w) {
    if (w.nc == 3) launch_pdl(k_ir_to32<3>, w.nblk, KTHREADS, 0, st, w.n, w.r, w.scal, w.b32);
    else launch_pdl(k_ir_to32<1>, w.nblk, KTHREADS, 0, st, w.n, w.r, w.scal, w.b32);
    note_launches(1);
}

// ------------------------------------------- widened preconditioner --
__global__ void __launch_bounds__(KTHREADS)
k_narrow(const long long n, const double *__restrict__ r, float *r32, const int *gate) {
    pdl_enter();
    if (gate && *gate != KS_RUN) return;
    GRID_STRIDE(P, n) r32[P] = d2f_int(r[P]);   // on the integer pipe: conversions run at the FP64 rate
}

__global__ void __launch_bounds__(KTHREADS)
k_widen(const long long n, const float *__restrict__ z32, double *z, const int *gate) {
    pdl_enter();
    if (gate && *gate != KS_RUN) return;
    GRID_STRIDE(P, n) z[P] = f2d_int(z32[P]);
}

int WidenedPreconditioner::allocate(long long ncell, Preconditioner<float> *m) {
    release();
    n = ncell;
    m32 = m;
    nblk = vector_blocks(n);
    if (cudaMalloc(&r32, sizeof(float) * n) != cudaSuccess || cudaMalloc(&z32, sizeof(float) * n) != cudaSuccess) {
        release();
        return -1;
    }
    cudaMemset(r32, 0, sizeof(float) * n);
    cudaMemset(z32, 0, sizeof(float) * n);
    return 0;
}

void WidenedPreconditioner::release() {
    if (r32) cudaFree(r32);
    if (z32) cudaFree(z32);
    r32 = z32 = nullptr;
}

void WidenedPreconditioner::apply(cudaStream_t s, const double *r, double *z, const int *gate) {
    fused_narrow = m32->apply_from64(s, r, z32, gate);
    if (!fused_narrow) {
        launch_pdl(k_narrow, nblk, KTHREADS, 0, s, n, r, r32, gate);
        note_launches(1);
        m32->apply(s, r32, z32, gate);
    }
    launch_pdl(k_widen, nblk, KTHREADS, 0, s, n, z32, z, gate);
    note_launches(1);
}

// Double-float vectors: the FP32 preconditioner takes the high words (r
// rounded to FP32) when it cannot read them itself.
__global__ void __launch_bounds__(KTHREADS)
k_narrow_df(const long long n, const dfloat *__restrict__ r, float *r32, const int *gate) {
    pdl_enter();
    if (gate && *gate != KS_RUN) return;
    GRID_STRIDE(P, n) r32[P] = r[P].hi;
}


// FP64 <-> double-float at the ends of a double-float solve.
__global__ void __launch_bounds__(KTHREADS)
k_to_dfloat(const long long n, const double *__restrict__ x, dfloat *y) {
    pdl_enter();
    GRID_STRIDE(P, n) y[P] = dfloat(x[P]);
}

__global__ void __launch_bounds__(KTHREADS)
k_from_dfloat(const long long n, const dfloat *__restrict__ x, double *y) {
    pdl_enter();
    GRID_STRIDE(P, n) y[P] = (double)x[P];
}

void DFloatPreconditioner::apply(cudaStream_t s, const dfloat *r, float *z, const int *gate) {
    fused_narrow = m32->apply_from_df(s, r, z, gate);
    if (!fused_narrow) {
        launch_pdl(k_narrow_df, nblk, KTHREADS, 0, s, n, r, r32, gate);
        note_launches(1);
        m32->apply(s, r32, z, gate);
    }
}

static void launch_update(cudaStream_t st, IRWork &w, double *x) {
    if (w.nc == 3) launch_pdl(k_ir_update<3>, w.nblk, KTHREADS, 0, st, w.n, x, w.e32, w.scal, w.inner.scal);
    else launch_pdl(k_ir_update<1>, w.nblk, KTHREADS, 0, st, w.n, x, w.e32, w.scal, w.inner.scal);
    note_launches(1);
}

// Relative residual of a report: NaN when either norm is not finite (the
// host turns that into a status), 0 for a zero right-hand side.
static double relres(double rn2, double bn2) {
    if (!std::isfinite(rn2) || !std::isfinite(bn2)) return NAN;
    return bn2 > 0 ? std::sqrt(rn2 / bn2) : 0.0;
}

template <typename T>
int report(const KrylovWork<T> &w, SolveReport &rep) {
    int status = 0;
    for (int c = 0; c < w.nc; c++) {
        const KScal &s = w.scal_h[c];
        rep.iters[c] = s.iters;
        rep.relres[c] = relres(s.rnorm2, s.bnorm2);
        rep.divmax[c] = s.divmax;
        if (s.state == KS_BREAKDOWN) status = 2;
        else if (s.state != KS_DONE && status == 0) status = 1;
    }
    return status;
}

template int report<double>(const KrylovWork<double> &, SolveReport &);
template int report<float>(const KrylovWork<float> &, SolveReport &);
template int report<dfloat>(const KrylovWork<dfloat> &, SolveReport &);

int report(const IRWork &w, SolveReport &rep) {
    rep = SolveReport();
    int status = 0;
    for (int c = 0; c < w.nc; c++) {
        const IRScal &s = w.scal_h[c];
        rep.iters[c] = s.inner;
        rep.outer = std::max(rep.outer, s.outer);
        rep.relres[c] = relres(s.rnorm2, s.bnorm2);
        rep.divmax[c] = s.divmax;
        if (s.state != KS_DONE) status = 1;
    }
    return status;
}

// ----------------------------------------------------------- host loops --
template <typename T>
static void fetch(cudaStream_t st, KrylovWork<T> &w) {
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(KScal) * w.nc, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
}

// vb (one-component solves): the right-hand side, to check the true
// residual after the iteration that ends the solve (k_bicg_verify).
template <typename T, typename B = T>
static void host_loop(cudaStream_t st, const OpT<T> &A, int op, KrylovWork<T> &w, T *x, int maxit,
                      Preconditioner<T> *M, Prof *pf, const B *vb = nullptr) {
    const LoopCtl none;
    fetch(st, w);
    int it = 0;
    while (!all_in(w.scal_h, w.nc, KS_DONE, KS_BREAKDOWN, KS_DONE) && it < maxit) {
        it++;
        first_half(st, A, op, w, M, pf);
        fetch(st, w);
        // Components converged on s skip the second half (its kernels would
        // return at once for them).
        if (!all_in(w.scal_h, w.nc, KS_HALF, KS_DONE, KS_BREAKDOWN)) second_half(st, A, op, w, M, pf);
        launch_xr(st, A, w, x, maxit, M, none);
        if (vb) launch_verify(st, A, op, w, vb, x, maxit, none);
        fetch(st, w);
    }
}

template <typename T>
int bicgstab(cudaStream_t st, const OpT<T> &A, int op, KrylovWork<T> &w, const T *b, T *x, const SolveParams &prm,
             Preconditioner<T> *M, SolveReport &rep) {
    if (prm.x_given) launch_init_guess(st, A, op, w, b, x, prm.tol, prm.divtol, LoopCtl());
    else launch_init(st, w, b, x, prm.tol, prm.divtol, nullptr, 0.0, 0.0, LoopCtl());
    host_loop(st, A, op, w, x, prm.maxit, M, prm.prof);
    return report(w, rep);
}

template int bicgstab<double>(cudaStream_t, const OpT<double> &, int, KrylovWork<double> &, const double *,
                              double *, const SolveParams &, Preconditioner<double> *, SolveReport &);
template int bicgstab<float>(cudaStream_t, const OpT<float> &, int, KrylovWork<float> &, const float *, float *,
                             const SolveParams &, Preconditioner<float> *, SolveReport &);

static void launch_to_dfloat(cudaStream_t st, long long n, const double *x, dfloat *y) {
    launch_pdl(k_to_dfloat, vector_blocks(n), KTHREADS, 0, st, n, x, y);
    note_launches(1);
}

static void launch_from_dfloat(cudaStream_t st, long long n, const dfloat *x, double *y) {
    launch_pdl(k_from_dfloat, vector_blocks(n), KTHREADS, 0, st, n, x, y);
    note_launches(1);
}

int bicgstab_df(cudaStream_t st, const OpT<dfloat> &A, int op, KrylovWork<dfloat> &w, dfloat *xw, const double *b,
                double *x, const SolveParams &prm, Preconditioner<dfloat> *M, SolveReport &rep) {
    if (!M) return 2;   // p^ and s^ are the preconditioner's FP32 output
    const long long m = w.n * w.nc;
    if (prm.x_given) {
        launch_to_dfloat(st, m, x, xw);
        launch_init_guess(st, A, op, w, b, xw, prm.tol, prm.divtol, LoopCtl());
    } else {
        launch_init(st, w, b, xw, prm.tol, prm.divtol, nullptr, 0.0, 0.0, LoopCtl());
    }
    host_loop(st, A, op, w, xw, prm.maxit, M, prm.prof, b);
    launch_from_dfloat(st, m, xw, x);
    return report(w, rep);
}

int solve_ir(cudaStream_t st, const OpT<double> &A64, const OpT<float> &A32, int op, IRWork &w, const double *b,
             double *x, const SolveParams &prm, Preconditioner<float> *M32, SolveReport &rep) {
    const long long n = w.n;
    const int nc = w.nc;
    auto fetch_outer = [&]() {
        cudaMemcpyAsync(w.scal_h, w.scal, sizeof(IRScal) * nc, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
    };
    if (!prm.x_given) cudaMemsetAsync(x, 0, sizeof(double) * n * nc, st);
    launch_residual(st, A64, op, w, b, x, prm.x_given ? IR_GUESS : IR_ZERO, prm, LoopCtl());
    fetch_outer();
    int outer = 0;
    while (!all_in(w.scal_h, nc, KS_DONE, KS_DONE, KS_DONE) && outer < prm.max_outer) {
        outer++;
        launch_to32(st, w);
        launch_init(st, w.inner, w.b32, w.e32, prm.inner_tol, 0.0, w.scal, prm.tol, prm.divtol, LoopCtl());
        host_loop(st, A32, op, w.inner, w.e32, prm.maxit, M32, prm.prof);
        launch_update(st, w, x);
        launch_residual(st, A64, op, w, b, x, IR_NEXT, prm, LoopCtl());
        fetch_outer();
    }
    return report(w, rep);
}

int solve_inc(cudaStream_t st, const OpT<float> &A32, int op, IRWork &w, const SolveParams &prm, SolveReport &rep) {
    launch_init(st, w.inner, w.b32, w.e32, prm.inner_tol, 0.0, w.scal, prm.tol, 0.0, LoopCtl());
    host_loop<float>(st, A32, op, w.inner, w.e32, prm.maxit, nullptr, prm.prof);
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(IRScal) * w.nc, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    return report_inc(w, prm.tol, rep);
}

int report_inc(const IRWork &w, double tol, SolveReport &rep) {
    rep = SolveReport();
    int status = 0;
    for (int c = 0; c < w.nc; c++) {
        const KScal &s = w.inner.scal_h[c];
        rep.iters[c] = s.iters;
        rep.relres[c] = relres(s.rnorm2, w.scal_h[c].bnorm2);
        rep.divmax[c] = 0.0;
        if (s.state == KS_BREAKDOWN) status = 2;
        else if (!(rep.relres[c] < tol) && rep.relres[c] != 0.0 && status == 0) status = 1;
    }
    return status;
}

// ------------------------------------------------------- recorded forms --
// Graph being captured on st.
static cudaGraph_t capture_graph(cudaStream_t st) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
        return nullptr;
    return g;
}

static int new_loop(cudaStream_t st, LoopCtl &lc) {
    cudaGraph_t g = capture_graph(st);
    if (!g) return -1;
    if (cudaGraphConditionalHandleCreate(&lc.h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return -1;
    lc.use = 1;
    return 0;
}

// Appends a while node on lc.h after st's current work and starts capturing
// its body on body_stream.
static int begin_while(cudaStream_t st, const LoopCtl &lc, cudaStream_t body_stream) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess) return -1;
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = lc.h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &p) != cudaSuccess) return -1;
    if (cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
        return -1;
    if (cudaStreamBeginCaptureToGraph(body_stream, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return -1;
    return 0;
}

static int end_while(cudaStream_t body_stream) {
    cudaGraph_t g = nullptr;
    return cudaStreamEndCapture(body_stream, &g) == cudaSuccess ? 0 : -1;
}

// Init (already recorded by the caller with lc) + while loop of iterations
// (vb as in host_loop).
template <typename T, typename B = T>
static int record_loop(cudaStream_t st, cudaStream_t body, const OpT<T> &A, int op, KrylovWork<T> &w, T *x,
                       int maxit, Preconditioner<T> *M, const LoopCtl &lc, int *per_iter, const B *vb = nullptr) {
    if (begin_while(st, lc, body) != 0) return -1;
    first_half(body, A, op, w, M, nullptr);
    second_half(body, A, op, w, M, nullptr);
    launch_xr(body, A, w, x, maxit, M, lc);
    if (vb) launch_verify(body, A, op, w, vb, x, maxit, lc);
    if (end_while(body) != 0) return -1;
    *per_iter = 5 + (vb ? 1 : 0) + (M ? 2 * M->launches() : 0);
    return 0;
}

template <typename T>
int record_bicgstab(cudaStream_t st, const cudaStream_t *aux, const OpT<T> &A, int op, KrylovWork<T> &w, const T *b,
                    T *x, const SolveParams &prm, Preconditioner<T> *M, int *fixed, int *per_iter) {
    LoopCtl lc;
    if (new_loop(st, lc) != 0) return -1;
    if (prm.x_given) launch_init_guess(st, A, op, w, b, x, prm.tol, prm.divtol, lc);
    else launch_init(st, w, b, x, prm.tol, prm.divtol, nullptr, 0.0, 0.0, lc);
    if (record_loop(st, aux[0], A, op, w, x, prm.maxit, M, lc, per_iter) != 0) return -1;
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(KScal) * w.nc, cudaMemcpyDeviceToHost, st);
    *fixed = 1;
    return 0;
}

template int record_bicgstab<double>(cudaStream_t, const cudaStream_t *, const OpT<double> &, int,
                                     KrylovWork<double> &, const double *, double *, const SolveParams &,
                                     Preconditioner<double> *, int *, int *);
template int record_bicgstab<float>(cudaStream_t, const cudaStream_t *, const OpT<float> &, int, KrylovWork<float> &,
                                    const float *, float *, const SolveParams &, Preconditioner<float> *, int *,
                                    int *);

int record_bicgstab_df(cudaStream_t st, const cudaStream_t *aux, const OpT<dfloat> &A, int op, KrylovWork<dfloat> &w,
                       dfloat *xw, const double *b, double *x, const SolveParams &prm, Preconditioner<dfloat> *M,
                       int *fixed, int *per_iter) {
    if (!M) return -1;   // p^ and s^ are the preconditioner's FP32 output
    const long long m = w.n * w.nc;
    LoopCtl lc;
    if (new_loop(st, lc) != 0) return -1;
    if (prm.x_given) {
        launch_to_dfloat(st, m, x, xw);
        launch_init_guess(st, A, op, w, b, xw, prm.tol, prm.divtol, lc);
    } else {
        launch_init(st, w, b, xw, prm.tol, prm.divtol, nullptr, 0.0, 0.0, lc);
    }
    if (record_loop(st, aux[0], A, op, w, xw, prm.maxit, M, lc, per_iter, b) != 0) return -1;
    launch_from_dfloat(st, m, xw, x);
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(KScal) * w.nc, cudaMemcpyDeviceToHost, st);
    *fixed = prm.x_given ? 3 : 2;
    return 0;
}

int record_ir(cudaStream_t st, const cudaStream_t *aux, const OpT<double> &A64, const OpT<float> &A32, int op,
              IRWork &w, const double *b, double *x, const SolveParams &prm, Preconditioner<float> *M32, int *fixed,
              int *per_outer, int *per_iter) {
    const long long n = w.n;
    const int nc = w.nc;
    LoopCtl outer;
    if (new_loop(st, outer) != 0) return -1;
    if (!prm.x_given) cudaMemsetAsync(x, 0, sizeof(double) * n * nc, st);
    launch_residual(st, A64, op, w, b, x, prm.x_given ? IR_GUESS : IR_ZERO, prm, outer);
    if (begin_while(st, outer, aux[0]) != 0) return -1;
    {
        cudaStream_t bs = aux[0];
        launch_to32(bs, w);
        LoopCtl inner;
        if (new_loop(bs, inner) != 0) return -1;
        launch_init(bs, w.inner, w.b32, w.e32, prm.inner_tol, 0.0, w.scal, prm.tol, prm.divtol, inner);
        if (record_loop(bs, aux[1], A32, op, w.inner, w.e32, prm.maxit, M32, inner, per_iter) != 0) return -1;
        launch_update(bs, w, x);
        launch_residual(bs, A64, op, w, b, x, IR_NEXT, prm, outer);
    }
    if (end_while(aux[0]) != 0) return -1;
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(IRScal) * nc, cudaMemcpyDeviceToHost, st);
    *fixed = 1;
    *per_outer = 4;
    return 0;
}

int record_inc(cudaStream_t st, const cudaStream_t *aux, const OpT<float> &A32, int op, IRWork &w,
               const SolveParams &prm, int *fixed, int *per_iter) {
    LoopCtl lc;
    if (new_loop(st, lc) != 0) return -1;
    launch_init(st, w.inner, w.b32, w.e32, prm.inner_tol, 0.0, w.scal, prm.tol, 0.0, lc);
    if (record_loop<float>(st, aux[0], A32, op, w.inner, w.e32, prm.maxit, nullptr, lc, per_iter) != 0) return -1;
    cudaMemcpyAsync(w.inner.scal_h, w.inner.scal, sizeof(KScal) * w.nc, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(IRScal) * w.nc, cudaMemcpyDeviceToHost, st);
    *fixed = 1;
    return 0;
}

template <typename T>
void apply_operator(cudaStream_t st, const OpT<T> &A, int op, int comp, const T *x, T *y) {
    launch_pdl(k_apply<T>, A.sw.nblocks, SW_THREADS, 0, st, A, op, comp, x, y);
    note_launches(1);
}

template void apply_operator<double>(cudaStream_t, const OpT<double> &, int, int, const double *, double *);
template void apply_operator<float>(cudaStream_t, const OpT<float> &, int, int, const float *, float *);

// ================================================== flexible GMRES (FP64) ==
// One restart cycle: V[0] = r / beta; for j = 0, 1, ...: z_j = M V[j]
// (kept in Z[j]), w = A z_j, two classical Gram-Schmidt passes against
// V[0..j], h[j+1][j] = ||w||, V[j+1] = w / h[j+1][j]; Givens rotations keep
// the least-squares residual |g[j+1]| current.  The cycle ends when that
// estimate passes the stopping test, at j = m, or on breakdown; then
// x += Z y (H y = g) and the true residual r = b - A x decides whether
// another cycle runs.  For the divergence rule the in-cycle estimate scales
// the cycle's starting divergence maximum by |g[j+1]| / beta.
enum { GM_RUN = 0, GM_DONE = 2, GM_MAXIT = 4 };

int GmresWork::allocate(long long ncell, int restart, int maxblocks) {
    release();
    n = ncell;
    m = std::max(1, std::min(restart, GM_MAX));
    nblk = vector_blocks(ncell);
    const size_t nvec = 2 * (size_t)m + 3;
    if (cudaMalloc(&base, sizeof(double) * n * nvec) != cudaSuccess) return -1;
    cudaMemset(base, 0, sizeof(double) * n * nvec);
    V = base;
    Z = V + (size_t)m * n;
    w = Z + (size_t)m * n;
    vin = w + n;
    zj = vin + n;
    if (cudaMalloc(&scal, sizeof(GScal)) != cudaSuccess) return -1;
    cudaMemset(scal, 0, sizeof(GScal));
    if (cudaMallocHost(&scal_h, sizeof(GScal)) != cudaSuccess) return -1;
    memset(scal_h, 0, sizeof(GScal));
    if (cudaMalloc(&partials, sizeof(double) * std::max(nblk, maxblocks) * (GM_MAX + 2)) != cudaSuccess) return -1;
    if (cudaMalloc(&counter, sizeof(unsigned int)) != cudaSuccess) return -1;
    cudaMemset(counter, 0, sizeof(unsigned int));
    return 0;
}

void GmresWork::release() {
    if (base) cudaFree(base);
    if (scal) cudaFree(scal);
    if (scal_h) cudaFreeHost(scal_h);
    if (partials) cudaFree(partials);
    if (counter) cudaFree(counter);
    base = V = Z = w = vin = zj = nullptr;
    scal = scal_h = nullptr;
    partials = nullptr;
    counter = nullptr;
}

// Residual w = b - A x (x_zero: w = b, x = 0 assumed), ||w||^2 (and ||b||^2
// when x_zero), divergence max; the last block applies the stopping test
// on this true residual and starts the next cycle (V[0] scale, g = beta e1).
__global__ void __launch_bounds__(SW_THREADS)
k_gm_residual(const OpT<double> A, const int op, const double *__restrict__ b, const double *__restrict__ x,
              double *w, const int x_zero, GScal *gs, const double tol, const double divtol, const int m,
              const int maxit, double *partials, unsigned int *counter, const LoopCtl lc) {
    pdl_enter();
    __shared__ double smem[32 * 2];
    double sm = 0.0, mx = 0.0;
    bool run[1] = {true};
    auto acc = [&](long long P, double y) {
        w[P] = y;
        sm += y * y;
        if (divtol > 0) mx = fmax(mx, (double)divw(A, P, y));
    };
    sweep_rows<double, 1>(
        A, run, [&](int, long long P, int i, const Column<double> &q) {
            acc(P, x_zero ? b[P] : b[P] - interior_row(A, op, x, P, i, q));
        },
        [&](int, long long P) { acc(P, x_zero ? b[P] : b[P] - op_row(A, op, 0, x, P)); });
    double v[2] = {sm, mx};
    reduce_and_finish<2, 1>(v, smem, partials, counter, [&](const double *tot) {
        GScal &s = *gs;
        if (x_zero) {
            s.bnorm2 = tot[0];
            s.iters = 0;
            s.cycles = 0;
            s.m = m;
            s.tol = tol;
            s.divtol = divtol;
            s.maxit = maxit;
        } else {
            s.cycles += 1;
        }
        s.rnorm2 = tot[0];
        s.divmax = tot[1];
        const double beta = sqrt(tot[0]);
        const bool done = s.bnorm2 == 0.0 || beta == 0.0 || converged(tot[0], s.bnorm2, tot[1], tol, divtol);
        s.state = done ? GM_DONE : (s.iters >= maxit ? GM_MAXIT : GM_RUN);
        s.beta0 = beta;
        s.divmax0 = tot[1];
        s.res = beta;
        s.vscale = beta > 0 ? 1.0 / beta : 0.0;
        s.j = 0;
        for (int q = 0; q <= GM_MAX; q++) s.g[q] = 0.0;
        s.g[0] = beta;
        set_loop(lc, s.state == GM_RUN);
    });
}

// Start of a cycle's Arnoldi loop: its condition.
__global__ void k_gm_cycle(const GScal *gs, const LoopCtl lc) {
    pdl_enter();
    if (threadIdx.x == 0 && blockIdx.x == 0) set_loop(lc, gs->state == GM_RUN);
}

// V[j] = vin = w * vscale.
__global__ void __launch_bounds__(KTHREADS)
k_gm_next(const long long n, const double *__restrict__ w, double *V, double *vin, const GScal *gs) {
    pdl_enter();
    const double sc = gs->vscale;
    double *vj = V + (size_t)gs->j * n;
    GRID_STRIDE(P, n) {
        const double y = w[P] * sc;
        vj[P] = y;
        vin[P] = y;
    }
}

// w = A z, Z[j] = z.
__global__ void __launch_bounds__(SW_THREADS)
k_gm_spmv(const OpT<double> A, const int op, const long long n, const double *__restrict__ z, double *w, double *Z,
          const GScal *gs) {
    pdl_enter();
    double *zj = Z + (size_t)gs->j * n;
    bool run[1] = {true};
    sweep_rows<double, 1>(
        A, run,
        [&](int, long long P, int i, const Column<double> &q) {
            w[P] = interior_row(A, op, z, P, i, q);
            zj[P] = z[P];
        },
        [&](int, long long P) {
            w[P] = op_row(A, op, 0, z, P);
            zj[P] = z[P];
        });
}

// c_i = (V[i], w) for i <= j into gs->c0 (pass 0) or gs->c1 (pass 1).
template <int MM>
__global__ void __launch_bounds__(KTHREADS)
k_gm_dots(const long long n, const double *__restrict__ V, const double *__restrict__ w, GScal *gs, const int pass,
          double *partials, unsigned int *counter) {
    pdl_enter();
    __shared__ double smem[32 * MM];
    const int j = gs->j;
    double a[MM];
#pragma unroll
    for (int i = 0; i < MM; i++) a[i] = 0.0;
    GRID_STRIDE(P, n) {
        const double wv = w[P];
#pragma unroll
        for (int i = 0; i < MM; i++)
            if (i <= j) a[i] += V[(size_t)i * n + P] * wv;
    }
    reduce_and_finish<MM, MM>(a, smem, partials, counter, [&](const double *tot) {
        double *c = pass == 0 ? gs->c0 : gs->c1;
        for (int i = 0; i < MM; i++) c[i] = i <= j ? tot[i] : 0.0;
    });
}

// w -= sum_{i<=j} c_i V[i] with c the projections of this pass; the final
// pass also sums ||w||^2 and its last block closes the Arnoldi step: column
// j of H (both passes' projections and ||w||), the rotations, the residual
// estimate, the in-cycle stopping test, j + 1 and the loop condition.
template <int MM>
__global__ void __launch_bounds__(KTHREADS)
k_gm_orth(const long long n, const double *__restrict__ V, double *w, GScal *gs, const int final_pass,
          double *partials, unsigned int *counter, const LoopCtl lc) {
    pdl_enter();
    __shared__ double smem[32];
    __shared__ double cs_[MM];
    const int j = gs->j;
    const double *c = final_pass ? gs->c1 : gs->c0;
    if (threadIdx.x < MM) cs_[threadIdx.x] = threadIdx.x <= j ? c[threadIdx.x] : 0.0;
    __syncthreads();
    double ss = 0.0;
    GRID_STRIDE(P, n) {
        double y = w[P];
        for (int i = 0; i <= j; i++) y -= cs_[i] * V[(size_t)i * n + P];
        w[P] = y;
        ss += y * y;
    }
    if (!final_pass) return;
    double v[1] = {ss};
    reduce_and_finish<1, 1>(v, smem, partials, counter, [&](const double *tot) {
        GScal &s = *gs;
        const int L = GM_MAX + 1;
        double *hc = s.h + (size_t)j * L;
        for (int i = 0; i <= j; i++) hc[i] = s.c0[i] + s.c1[i];
        const double hn = sqrt(tot[0]);
        hc[j + 1] = hn;
        for (int i = 0; i < j; i++) {
            const double t = s.cs[i] * hc[i] + s.sn[i] * hc[i + 1];
            hc[i + 1] = -s.sn[i] * hc[i] + s.cs[i] * hc[i + 1];
            hc[i] = t;
        }
        const double d = hypot(hc[j], hc[j + 1]);
        bool breakdown = d == 0.0 || !isfinite(d);
        if (!breakdown) {
            s.cs[j] = hc[j] / d;
            s.sn[j] = hc[j + 1] / d;
            hc[j] = d;
            hc[j + 1] = 0.0;
            s.g[j + 1] = -s.sn[j] * s.g[j];
            s.g[j] = s.cs[j] * s.g[j];
        }
        s.res = fabs(s.g[j + 1]);
        s.iters += 1;
        s.j = j + 1;
        s.vscale = hn > 0 ? 1.0 / hn : 0.0;
        const bool est = (s.tol > 0 && s.res < s.tol * sqrt(s.bnorm2)) ||
                         (s.divtol > 0 && s.beta0 > 0 && s.divmax0 * (s.res / s.beta0) <= 0.5 * s.divtol);
        const bool more = !breakdown && !est && hn > 0 && s.j < s.m && s.iters < s.maxit;
        s.more = more ? 1 : 0;
        set_loop(lc, more);
    });
}

// x += sum_{i<k} y_i Z[i] with H y = g solved (back substitution, k = j)
// by every block for itself.
__global__ void __launch_bounds__(KTHREADS)
k_gm_update(const long long n, const double *__restrict__ Z, double *x, const GScal *gs) {
    pdl_enter();
    __shared__ double y[GM_MAX];
    const int k = gs->j;
    if (threadIdx.x == 0) {
        const int L = GM_MAX + 1;
        for (int i = k - 1; i >= 0; i--) {
            double t = gs->g[i];
            for (int l = i + 1; l < k; l++) t -= gs->h[(size_t)l * L + i] * y[l];
            const double d = gs->h[(size_t)i * L + i];
            y[i] = d != 0.0 ? t / d : 0.0;
        }
    }
    __syncthreads();
    GRID_STRIDE(P, n) {
        double xv = x[P];
        for (int i = 0; i < k; i++) xv += y[i] * Z[(size_t)i * n + P];
        x[P] = xv;
    }
}

static void gm_residual(cudaStream_t st, const OpT<double> &A, int op, GmresWork &w, const double *b,
                        const double *x, int x_zero, const SolveParams &prm, LoopCtl lc) {
    launch_pdl(k_gm_residual, A.sw.nblocks, SW_THREADS, 0, st, A, op, b, x, w.w, x_zero, w.scal, prm.tol, prm.divtol, w.m,
                                                       prm.maxit, w.partials, w.counter, lc);
    note_launches(1);
}

// One Arnoldi step (6 launches + the preconditioner's).
static void gm_step(cudaStream_t st, const OpT<double> &A, int op, GmresWork &w, Preconditioner<double> *M,
                    Prof *pf, LoopCtl lc) {
    const long long n = w.n;
    launch_pdl(k_gm_next, w.nblk, KTHREADS, 0, st, n, w.w, w.V, w.vin, w.scal);
    note_launches(1);
    const double *z = w.vin;
    if (M) {
        const int tm = prof_begin(pf, "mg_vcycle");
        M->apply(st, w.vin, w.zj, nullptr);
        prof_end(pf, tm);
        z = w.zj;
    }
    const int tm = prof_begin(pf, "spmv_p");
    launch_pdl(k_gm_spmv, A.sw.nblocks, SW_THREADS, 0, st, A, op, n, z, w.w, w.Z, w.scal);
    note_launches(1);
    prof_end(pf, tm);
    const int to = prof_begin(pf, "gmres_orth");
    for (int pass = 0; pass < 2; pass++) {
        launch_pdl(k_gm_dots<GM_MAX>, w.nblk, KTHREADS, 0, st, n, w.V, w.w, w.scal, pass, w.partials, w.counter);
        launch_pdl(k_gm_orth<GM_MAX>, w.nblk, KTHREADS, 0, st, n, w.V, w.w, w.scal, pass, w.partials, w.counter, lc);
        note_launches(2);
    }
    prof_end(pf, to);
}

static void gm_update(cudaStream_t st, GmresWork &w, double *x) {
    launch_pdl(k_gm_update, w.nblk, KTHREADS, 0, st, w.n, w.Z, x, w.scal);
    note_launches(1);
}

static void gm_fetch(cudaStream_t st, GmresWork &w) {
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(GScal), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
}

int report(const GmresWork &w, SolveReport &rep) {
    rep = SolveReport();
    const GScal &s = *w.scal_h;
    rep.iters[0] = s.iters;
    rep.outer = s.cycles;
    rep.relres[0] = relres(s.rnorm2, s.bnorm2);
    rep.divmax[0] = s.divmax;
    return s.state == GM_DONE ? 0 : 1;
}

int gmres(cudaStream_t st, const OpT<double> &A, int op, GmresWork &w, const double *b, double *x,
          const SolveParams &prm, Preconditioner<double> *M, SolveReport &rep) {
    const LoopCtl none;
    cudaMemsetAsync(x, 0, sizeof(double) * w.n, st);
    gm_residual(st, A, op, w, b, x, 1, prm, none);
    gm_fetch(st, w);
    while (w.scal_h->state == GM_RUN) {
        do {
            gm_step(st, A, op, w, M, prm.prof, none);
            gm_fetch(st, w);
        } while (w.scal_h->more);
        gm_update(st, w, x);
        gm_residual(st, A, op, w, b, x, 0, prm, none);
        gm_fetch(st, w);
    }
    return report(w, rep);
}

int record_gmres(cudaStream_t st, const cudaStream_t *aux, const OpT<double> &A, int op, GmresWork &w,
                 const double *b, double *x, const SolveParams &prm, Preconditioner<double> *M, int *fixed,
                 int *per_cycle, int *per_iter) {
    LoopCtl outer;
    if (new_loop(st, outer) != 0) return -1;
    cudaMemsetAsync(x, 0, sizeof(double) * w.n, st);
    gm_residual(st, A, op, w, b, x, 1, prm, outer);
    if (begin_while(st, outer, aux[0]) != 0) return -1;
    {
        cudaStream_t bs = aux[0];
        LoopCtl inner;
        if (new_loop(bs, inner) != 0) return -1;
        launch_pdl(k_gm_cycle, 1, 32, 0, bs, w.scal, inner);
        note_launches(1);
        if (begin_while(bs, inner, aux[1]) != 0) return -1;
        gm_step(aux[1], A, op, w, M, nullptr, inner);
        if (end_while(aux[1]) != 0) return -1;
        gm_update(bs, w, x);
        gm_residual(bs, A, op, w, b, x, 0, prm, outer);
    }
    if (end_while(aux[0]) != 0) return -1;
    cudaMemcpyAsync(w.scal_h, w.scal, sizeof(GScal), cudaMemcpyDeviceToHost, st);
    *fixed = 1;
    *per_cycle = 3;
    *per_iter = 6 + (M ? M->launches() : 0);
    return 0;
}

}  // namespace ibm
