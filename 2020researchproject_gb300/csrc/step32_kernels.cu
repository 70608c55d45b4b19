// FP32 explicit stages of the IBM3D_MIXED32 step.
//
// The same fractional step as step_kernels.cu (src/ibm3d_fracstep.c:117-487,
// 709-805), with the explicit stencils in FP32 and the momentum solve in
// increment form:
//
//   A u* = b   becomes   A e = c,  c = b - A u^n,  u* = u^n + e.
//
// For a fluid row, with k the Crank-Nicolson coefficients,
//   b   = u_P + sum k (u_nb - u_P) + r,   r = -dt/2 (3 N - N_prev) - dt G_c p + dt f - dt div tau
//   A x = x_P - sum k (x_nb - x_P)
// so c = 2 sum k (u_nb - u_P) + r: the O(1) parts cancel analytically and
// c is O(dt).  Evaluated in FP32, its error is ~1e-7 of |c| plus ~1e-8 of
// |u| (the FP32 neighbour differences), far below the 1e-6 relative
// momentum tolerance, and the FP64 state u^{n+1} = u^n + (e - dt G_c p')
// only ever receives O(dt) increments rounded to FP32.  The solve stops on
// the reference's test ||b - A u*|| < tol ||b|| (||b|| is reduced here).
//
// U* is computed in FP32 and stored widened to FP64; the Poisson right-hand
// side is the FP64 divergence of those stored faces, so the projection
// (FP64) drives div U^{n+1} of the stored faces to the solve's tolerance
// exactly as in the FP64 step.  Every face is computed by both cells that
// share it; the FP32 arithmetic uses explicitly rounded operations so both
// get the same bits.
//
// FP64 fields are read as FP32 with d2f_int / written with f2d_int
// (integer pipe; see common.cuh).
#include "common.cuh"
#include "kernels.h"
#include "krylov.h"
#include "ops.cuh"

namespace ibm {

namespace {

constexpr int K32_THREADS = 256;
constexpr int K32_BLOCKS = 1216;  // 8 per SM on 152 SMs; grid-stride

// An FP64 field value in FP32; NaN (solid cells) becomes 0, the value the
// momentum solve gives solid rows.
__device__ __forceinline__ float ld32(const double *__restrict__ a, long long P) {
    const float v = d2f_int(__ldg(a + P));
    return v == v ? v : 0.0f;
}

__device__ __forceinline__ float ldp32(const double *__restrict__ a, long long P) { return d2f_int(__ldg(a + P)); }

// Outer row of the FP32 momentum operator applied to the current velocity
// component (the rows of ops.cuh outer_row, values loaded from FP64).
__device__ __forceinline__ float outer_row_u(const OpT<float> &c, int comp, const double *__restrict__ u, long long P,
                                             int i, int j, int k, int f, int L) {
    const BCRow<float> &F = c.bc[f];
    const int axis = face_axis(f);
    const long long s = axis == 0 ? c.g.sx : axis == 1 ? c.g.sy : 1;
    const long long in = face_low(f) ? s : -s;
    switch (outer_row_kind(OP_MOM, F.type, comp, axis)) {
    case ROW_DIR: return F.dir_o[L - 1] * ld32(u, P) + F.dir_m[L - 1] * ld32(u, P + (2 * L - 1) * in);
    case ROW_NEU: return ld32(u, P) - ld32(u, P + (2 * L - 1) * in);
    case ROW_PER: return ld32(u, P) - ld32(u, periodic_image(c.g, i, j, k));
    default: return F.ext_o[L - 1] * ld32(u, P) - ld32(u, P + in) + F.ext_2[L - 1] * ld32(u, P + 2 * in);
    }
}

}  // namespace

// ------------------------------------------------------------------------
// calc_N + momentum right-hand side (src/ibm3d_fracstep.c:117-170,
// 237-352) in FP32, written as the increment system's right-hand side c
// (3 components, w.b32 layout l*n + P) and N (FP32).  The last block
// stores ||b||^2 and ||c||^2 per component in the increment solve's
// scalars (out[l].bnorm2, .rnorm2).
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(K32_THREADS)
k_conv_rhs32(const Grid g, const AxisF ax, const AxisF ay, const AxisF az, const OpT<float> A, const BCSet bc,
             const uint8_t *__restrict__ flag, const Conv32Args a, const float dt, const float f1, const float f2,
             const float f3, const int les, double *partials, unsigned int *counter, IRScal *out) {
    __shared__ double smem[32 * 6];
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // ||b||^2 (3), ||c||^2 (3)
    const long long n = g.ncell;
    const float NaNf = __int_as_float(0x7fc00000);
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cijk_g(g, P, i, j, k);
        int layer;
        const int f = owner_face(g, i, j, k, layer);
        float bv[3], cv[3];
        if (f >= 0) {
            // Outer rows: the velocity BC value (VELOCITY faces) or 0.
            const BCFace &F = bc.f[f];
            const bool vel = F.type == BCT_VELOCITY;
            const double *sv = F.scur ? F.scur + face_line(g, f, i, j, k) : nullptr;
#pragma unroll
            for (int l = 0; l < 3; l++) {
                bv[l] = vel ? d2f_int(sv ? sv[l * F.nt] : F.val[l]) : 0.0f;
                cv[l] = bv[l] - outer_row_u(A, l, a.u[l], P, i, j, k, f, layer);
            }
        } else if (flag[P] != FLUID) {
            // Ghost rows (1 + w_self) x_g + sum w x = 0, solid rows x = 0.
#pragma unroll
            for (int l = 0; l < 3; l++) {
                a.N[l][P] = NaNf;
                bv[l] = 0.0f;
                cv[l] = 0.0f;
            }
            if (flag[P] == GHOST) {
                const int q = A.gid[P];
                const float ws = A.gwself[q];
#pragma unroll
                for (int l = 0; l < 3; l++) {
                    float sum = 0.0f;
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        const int m = A.gidx[8 * q + e];
                        if (m >= 0) sum += A.gw[8 * q + e] * ld32(a.u[l], m);
                    }
                    cv[l] = -((1.0f + ws) * ld32(a.u[l], P) + sum);
                }
            }
        } else {
            const long long sx = g.sx, sy = g.sy;
            const int I = i + 2, J = j + 2, K = k + 2;
            const float wmx0 = ax.wm[I], wpx0 = ax.wp[I], wmx1 = ax.wm[I + 1], wpx1 = ax.wp[I + 1];
            const float wmy0 = ay.wm[J], wpy0 = ay.wp[J], wmy1 = ay.wm[J + 1], wpy1 = ay.wp[J + 1];
            const float wmz0 = az.wm[K], wpz0 = az.wp[K], wmz1 = az.wm[K + 1], wpz1 = az.wp[K + 1];
            const float Uw = ldp32(a.U[0], P), Ue = ldp32(a.U[0], P + sx);
            const float Vs = ldp32(a.U[1], P), Vn = ldp32(a.U[1], P + sy);
            const float Wd = ldp32(a.U[2], P), Wu = ldp32(a.U[2], P + 1);
            const float rdx = ax.rd[I], rdy = ay.rd[J], rdz = az.rd[K];
            const float kW = ax.km[I], kE = ax.kp[I], kS = ay.km[J], kN = ay.kp[J], kD = az.km[K], kU = az.kp[K];
            const float gx = ax.rdcc[I], gy = ay.rdcc[J], gz = az.rdcc[K];
            const float ff[3] = {f1, f2, f3};
#pragma unroll
            for (int l = 0; l < 3; l++) {
                const double *u = a.u[l];
                const float uc = ld32(u, P);
                const float uW = ld32(u, P - sx), uE = ld32(u, P + sx), uS = ld32(u, P - sy), uN = ld32(u, P + sy);
                const float uD = ld32(u, P - 1), uU = ld32(u, P + 1);
                const float fw = uW * wmx0 + uc * wpx0, fe = uc * wmx1 + uE * wpx1;
                const float fs = uS * wmy0 + uc * wpy0, fn = uc * wmy1 + uN * wpy1;
                const float fd = uD * wmz0 + uc * wpz0, fu = uc * wmz1 + uU * wpz1;
                const float Nl = (Ue * fe - Uw * fw) * rdx + (Vn * fn - Vs * fs) * rdy + (Wu * fu - Wd * fd) * rdz;
                a.N[l][P] = Nl;
                float dp;
                if (l == 0) dp = (ldp32(a.p, P + sx) - ldp32(a.p, P - sx)) * gx;
                else if (l == 1) dp = (ldp32(a.p, P + sy) - ldp32(a.p, P - sy)) * gy;
                else dp = (ldp32(a.p, P + 1) - ldp32(a.p, P - 1)) * gz;
                float divtau = 0.0f;
                if (les) {
                    const int t1 = l == 0 ? 0 : l == 1 ? 1 : 2;
                    const int t2 = l == 0 ? 1 : l == 1 ? 3 : 4;
                    const int t3 = l == 0 ? 2 : l == 1 ? 4 : 5;
                    divtau = (ldp32(a.tau[t1], P + sx) - ldp32(a.tau[t1], P - sx)) * gx +
                             (ldp32(a.tau[t2], P + sy) - ldp32(a.tau[t2], P - sy)) * gy +
                             (ldp32(a.tau[t3], P + 1) - ldp32(a.tau[t3], P - 1)) * gz;
                }
                const float fl = a.force ? ldp32(a.force, l * n + P) : ff[l];
                const float lap = kW * (uW - uc) + kE * (uE - uc) + kS * (uS - uc) + kN * (uN - uc) +
                                  kD * (uD - uc) + kU * (uU - uc);
                const float rest = -dt / 2 * (3 * Nl - a.Np[l][P]) - dt * dp + dt * fl - dt * divtau;
                bv[l] = uc + lap + rest;
                cv[l] = 2 * lap + rest;
            }
        }
#pragma unroll
        for (int l = 0; l < 3; l++) {
            a.c[l * n + P] = cv[l];
            acc[l] += bv[l] * bv[l];
            acc[3 + l] += cv[l] * cv[l];
        }
    }
    double tot[6];
    block_reduce<6, 6, float>(acc, tot, smem);
    if (!publish_partials<6>(tot, partials, counter)) return;
    double all[6];
    reduce_partials<6, 6>(partials, gridDim.x, all, smem);
    if (threadIdx.x == 0) {
        for (int l = 0; l < 3; l++) {
            IRScal &s = out[l];
            s.bnorm2 = all[l];
            s.rnorm2 = all[3 + l];
            s.rmax = 0.0;
            s.divmax = 0.0;
            s.scale = 1.0;
            s.state = all[3 + l] == 0.0 ? KS_DONE : KS_RUN;
            s.outer = 0;
            s.inner = 0;
        }
        *counter = 0;
    }
}

void launch_conv_rhs32(cudaStream_t s, const Grid &g, const AxisF axf[3], const OpT<float> &A, const BCSet &bc,
                       const uint8_t *flag, const Conv32Args &a, double dt, const double f[3], int les,
                       double *partials, unsigned int *counter, IRScal *out) {
    k_conv_rhs32<<<K32_BLOCKS, K32_THREADS, 0, s>>>(g, axf[0], axf[1], axf[2], A, bc, flag, a, (float)dt, (float)f[0],
                                                    (float)f[1], (float)f[2], les, partials, counter, out);
    note_launches(1);
}

// ------------------------------------------------------------------------
// calc_u_tilde + calc_U_star (src/ibm3d_fracstep.c:388-487) in FP32 from
// u* = u^n + e, fused with the pressure-Poisson right-hand side
// (src/ibm3d_fracstep.c:530-647) in FP64 from the stored faces.
// ------------------------------------------------------------------------
namespace {

__device__ __forceinline__ float ustar_at(const double *__restrict__ u, const float *__restrict__ e, long long P) {
    return __fadd_rn(ld32(u, P), e[P]);
}

// Face between cells Pm (index ii-1) and Pp (index ii) along stride s;
// explicitly rounded so that both cells sharing the face get its bits.
__device__ __forceinline__ float face32(const double *__restrict__ u, const float *__restrict__ e,
                                        const double *__restrict__ p, const AxisF &a, int ii, long long Pm,
                                        long long Pp, long long s, bool fluid_ghost, float dt) {
    const float um = ustar_at(u, e, Pm), up = ustar_at(u, e, Pp);
    const float wm = a.wm[ii + 2], wp = a.wp[ii + 2];
    if (fluid_ghost) return __fadd_rn(__fmul_rn(um, wm), __fmul_rn(up, wp));
    const float gm = __fmul_rn(__fsub_rn(ldp32(p, Pm + s), ldp32(p, Pm - s)), a.rdcc[ii + 1]);
    const float gp = __fmul_rn(__fsub_rn(ldp32(p, Pp + s), ldp32(p, Pp - s)), a.rdcc[ii + 2]);
    const float tm = __fadd_rn(um, __fmul_rn(dt, gm));
    const float tp = __fadd_rn(up, __fmul_rn(dt, gp));
    const float gf = __fmul_rn(__fsub_rn(ldp32(p, Pp), ldp32(p, Pm)), a.rdc[ii + 2]);
    return __fsub_rn(__fadd_rn(__fmul_rn(tm, wm), __fmul_rn(tp, wp)), __fmul_rn(dt, gf));
}

__device__ __forceinline__ bool fg_pair32(uint8_t a, uint8_t b) {
    return (a == FLUID && b == GHOST) || (a == GHOST && b == FLUID);
}

}  // namespace

__global__ void __launch_bounds__(K32_THREADS)
k_ustar_prhs32(const Grid g, const AxisF ax, const AxisF ay, const AxisF az, const Axis ax64, const Axis ay64,
               const Axis az64, const BCSet bc, const uint8_t *__restrict__ flag, const Ustar32Args a, const float dt,
               const double m2re) {
    const long long n = g.ncell;
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cijk_g(g, P, i, j, k);
        int layer;
        const int face = owner_face(g, i, j, k, layer);
        if (face >= 0) {
            // Pressure-Dirichlet rows: p_bc(t + dt) - p_bc(t) (0 for constants).
            const BCFace &F = bc.f[face];
            double v = 0.0;
            if (F.scur && (F.type == BCT_PRESSURE || F.type == BCT_VELPERIODIC)) {
                const int t = 3 * F.nt + face_line(g, face, i, j, k);
                v = F.snxt[t] - F.scur[t];
            }
            a.b[P] = v;
            continue;
        }
        const long long sx = g.sx, sy = g.sy;
        const uint8_t fc = flag[P];
        const float Uw = face32(a.u[0], a.e[0], a.p, ax, i, P - sx, P, sx, fg_pair32(flag[P - sx], fc), dt);
        const float Ue = face32(a.u[0], a.e[0], a.p, ax, i + 1, P, P + sx, sx, fg_pair32(fc, flag[P + sx]), dt);
        const float Vs = face32(a.u[1], a.e[1], a.p, ay, j, P - sy, P, sy, fg_pair32(flag[P - sy], fc), dt);
        const float Vn = face32(a.u[1], a.e[1], a.p, ay, j + 1, P, P + sy, sy, fg_pair32(fc, flag[P + sy]), dt);
        const float Wd = face32(a.u[2], a.e[2], a.p, az, k, P - 1, P, 1, fg_pair32(flag[P - 1], fc), dt);
        const float Wu = face32(a.u[2], a.e[2], a.p, az, k + 1, P, P + 1, 1, fg_pair32(fc, flag[P + 1]), dt);
        const double Uw64 = f2d_int(Uw), Ue64 = f2d_int(Ue), Vs64 = f2d_int(Vs), Vn64 = f2d_int(Vn);
        const double Wd64 = f2d_int(Wd), Wu64 = f2d_int(Wu);
        a.Us[0][P] = Uw64;
        a.Us[1][P] = Vs64;
        a.Us[2][P] = Wd64;
        if (i == g.nx - 1) a.Us[0][P + sx] = Ue64;
        if (j == g.ny - 1) a.Us[1][P + sy] = Vn64;
        if (k == g.nz - 1) a.Us[2][P + 1] = Wu64;
        double rhs = 0.0;
        if (fc == FLUID && !(bc.p_singular && i == 0 && j == 0 && k == 0)) {
            const double div = (Ue64 - Uw64) * ax64.rd[i + 2] + (Vn64 - Vs64) * ay64.rd[j + 2] +
                               (Wu64 - Wd64) * az64.rd[k + 2];
            rhs = div * m2re * a.dinv[P];   // -div / (2 Re coeffsum)
        }
        a.b[P] = rhs;
    }
}

void launch_ustar_prhs32(cudaStream_t s, const Grid &g, const AxisF axf[3], const Axis ax64[3], const BCSet &bc,
                         const uint8_t *flag, const Ustar32Args &a, double dt, double Re) {
    k_ustar_prhs32<<<K32_BLOCKS, K32_THREADS, 0, s>>>(g, axf[0], axf[1], axf[2], ax64[0], ax64[1], ax64[2], bc, flag,
                                                      a, (float)dt, -1.0 / (2.0 * Re));
    note_launches(1);
}

// ------------------------------------------------------------------------
// update_next (src/ibm3d_fracstep.c:709-805) for the increment form: the
// cell velocity u^{n+1} = u^n + (e - dt G_c p') with the increment in
// FP32; faces U^{n+1} = U* - dt G_f p', p^{n+1} = p + p' and the
// divergence check max|div U^{n+1}| in FP64, as the FP64 step.
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_update_next32(const Grid g, const Axis ax, const Axis ay, const Axis az, const AxisF axf, const AxisF ayf,
                const AxisF azf, const BCSet bc, const uint8_t *__restrict__ flag, const Next32Args a, const double dt,
                double *partials, unsigned int *counter, double *maxdiv_out) {
    __shared__ double smem[32];
    const long long n = (long long)g.nx * g.ny * g.nz;
    double mdiv[1] = {0.0};
    const double NaN = __longlong_as_double(0x7ff8000000000000LL);
    const float dtf = (float)dt;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        ijk_interior(g, q, i, j, k);
        const long long P = cidx(g, i, j, k);
        const long long sx = g.sx, sy = g.sy;
        const int I = i + 2, J = j + 2, K = k + 2;
        const uint8_t fc = flag[P];
        const double pp = a.pp[P];
        a.pn[P] = (fc == FLUID || fc == GHOST) ? a.p[P] + pp : NaN;
        if (fc == FLUID) {
            const float gx = (ldp32(a.pp, P + sx) - ldp32(a.pp, P - sx)) * axf.rdcc[I];
            const float gy = (ldp32(a.pp, P + sy) - ldp32(a.pp, P - sy)) * ayf.rdcc[J];
            const float gz = (ldp32(a.pp, P + 1) - ldp32(a.pp, P - 1)) * azf.rdcc[K];
            a.un[0][P] = a.u[0][P] + f2d_int(a.e[0][P] - dtf * gx);
            a.un[1][P] = a.u[1][P] + f2d_int(a.e[1][P] - dtf * gy);
            a.un[2][P] = a.u[2][P] + f2d_int(a.e[2][P] - dtf * gz);
        } else if (fc == SOLID) {
            a.un[0][P] = a.un[1][P] = a.un[2][P] = NaN;
        }
        const uint8_t fw = flag[P - sx], fe = flag[P + sx], fs = flag[P - sy], fn = flag[P + sy];
        const uint8_t fd = flag[P - 1], fu = flag[P + 1];
        const double Uw = (fw != SOLID && fc != SOLID) ? a.Us[0][P] - dt * (pp - a.pp[P - sx]) * ax.rdc[I] : NaN;
        const double Ue = (fc != SOLID && fe != SOLID) ? a.Us[0][P + sx] - dt * (a.pp[P + sx] - pp) * ax.rdc[I + 1] : NaN;
        const double Vs = (fs != SOLID && fc != SOLID) ? a.Us[1][P] - dt * (pp - a.pp[P - sy]) * ay.rdc[J] : NaN;
        const double Vn = (fc != SOLID && fn != SOLID) ? a.Us[1][P + sy] - dt * (a.pp[P + sy] - pp) * ay.rdc[J + 1] : NaN;
        const double Wd = (fd != SOLID && fc != SOLID) ? a.Us[2][P] - dt * (pp - a.pp[P - 1]) * az.rdc[K] : NaN;
        const double Wu = (fc != SOLID && fu != SOLID) ? a.Us[2][P + 1] - dt * (a.pp[P + 1] - pp) * az.rdc[K + 1] : NaN;
        a.Un[0][P] = Uw;
        a.Un[1][P] = Vs;
        a.Un[2][P] = Wd;
        if (i == g.nx - 1) a.Un[0][P + sx] = Ue;
        if (j == g.ny - 1) a.Un[1][P + sy] = Vn;
        if (k == g.nz - 1) a.Un[2][P + 1] = Wu;
        if (fc == FLUID && !(bc.p_singular && i == 0 && j == 0 && k == 0)) {
            const double div = (Ue - Uw) * ax.rd[I] + (Vn - Vs) * ay.rd[J] + (Wu - Wd) * az.rd[K];
            mdiv[0] = nanmax(mdiv[0], fabs(div));
        }
    }
    block_max<1>(mdiv, smem);
    if (!publish_partials<1>(mdiv, partials, counter)) return;
    double m[1];
    reduce_partials<1, 0>(partials, gridDim.x, m, smem);
    if (threadIdx.x == 0) {
        *maxdiv_out = m[0];
        *counter = 0;
    }
}

void launch_update_next32(cudaStream_t s, const Grid &g, const Axis ax64[3], const AxisF axf[3], const BCSet &bc,
                          const uint8_t *flag, const Next32Args &a, double dt, double *partials,
                          unsigned int *counter, double *maxdiv_out, int nblocks) {
    k_update_next32<<<nblocks, 256, 0, s>>>(g, ax64[0], ax64[1], ax64[2], axf[0], axf[1], axf[2], bc, flag, a, dt,
                                            partials, counter, maxdiv_out);
    note_launches(1);
}

// ------------------------------------------------------------------------
// FP32 N read back as FP64 (field export of the mixed FP32 step).
// ------------------------------------------------------------------------
__global__ void k_widen_f32(const long long n, const float *__restrict__ x, double *__restrict__ y) {
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x)
        y[P] = (double)x[P];
}

void launch_widen_f32(cudaStream_t s, long long n, const float *x, double *y) {
    k_widen_f32<<<K32_BLOCKS, 256, 0, s>>>(n, x, y);
    note_launches(1);
}

// u* = u^n + e (NaN in u^n, solid cells, counts as 0), for read-back.
__global__ void k_ustar_from_increment(const long long n, const double *__restrict__ u, const float *__restrict__ e,
                                       double *__restrict__ y) {
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        const double v = u[P];
        y[P] = (v == v ? v : 0.0) + (double)e[P];
    }
}

void launch_ustar_from_increment(cudaStream_t s, long long n, const double *u, const float *e, double *y) {
    k_ustar_from_increment<<<K32_BLOCKS, 256, 0, s>>>(n, u, e, y);
    note_launches(1);
}

// ------------------------------------------------------------------------
// Self-test of the integer-pipe conversions against the hardware ones:
// x[q] for q < n is converted both ways; mismatches are counted (ties of
// the rounding, where d2f_int rounds away from zero and the hardware to
// even, and float subnormals are excluded by the caller's values).
// ------------------------------------------------------------------------
__global__ void k_conversion_check(const long long n, const double *__restrict__ x, unsigned long long *bad) {
    unsigned long long nb = 0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const double v = x[q];
        const float a = d2f_int(v), b = __double2float_rn(v);
        const bool same_f = __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
        const double c = f2d_int(b), d = (double)b;
        const bool same_d = __double_as_longlong(c) == __double_as_longlong(d) || (c != c && d != d);
        nb += (!same_f) + (!same_d);
    }
    atomicAdd(bad, nb);
}

int conversion_check(long long n, const double *x_host, unsigned long long *mismatches) {
    double *x = nullptr;
    unsigned long long *bad = nullptr;
    int rc = -1;
    if (cudaMalloc(&x, sizeof(double) * n) == cudaSuccess && cudaMalloc(&bad, sizeof *bad) == cudaSuccess &&
        cudaMemcpy(x, x_host, sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemset(bad, 0, sizeof *bad) == cudaSuccess) {
        k_conversion_check<<<K32_BLOCKS, 256>>>(n, x, bad);
        if (cudaGetLastError() == cudaSuccess &&
            cudaMemcpy(mismatches, bad, sizeof *bad, cudaMemcpyDeviceToHost) == cudaSuccess)
            rc = 0;
    }
    cudaFree(x);
    cudaFree(bad);
    return rc;
}

}  // namespace ibm
