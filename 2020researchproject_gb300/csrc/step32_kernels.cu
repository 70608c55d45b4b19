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
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "krylov.h"
#include "ops.cuh"

namespace ibm {

namespace {

constexpr int K32_THREADS = 256;
constexpr int K32_BLOCKS = 1216;  // 8 per SM on 152 SMs; grid-stride
// Tiles of the marching kernels: 32 (k) x 8 (j) columns, UN_PLANES planes of i.
constexpr int UN_TK = 32, UN_TJ = 8, UN_PLANES = 8;

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
    const int lane = threadIdx.x & 31;
    // Block-uniform loop: the lanes of a warp hold consecutive padded cells,
    // so the k neighbours (P -/+ 1) of the values every lane converts for
    // its own cell come by shuffle; lanes 0 and 31 load theirs.
    for (long long base = blockIdx.x * (long long)blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
        const long long P = base + threadIdx.x;
        const bool act = P < n;
        float own[5] = {0.f, 0.f, 0.f, 0.f, 0.f};   // u1, u2, u3, p, W (low z face)
        if (act) {
            own[0] = ld32(a.u[0], P);
            own[1] = ld32(a.u[1], P);
            own[2] = ld32(a.u[2], P);
            own[3] = ldp32(a.p, P);
            own[4] = ldp32(a.U[2], P);
        }
        float dn[4], up[5];
#pragma unroll
        for (int q = 0; q < 4; q++) dn[q] = __shfl_up_sync(0xffffffffu, own[q], 1);
#pragma unroll
        for (int q = 0; q < 5; q++) up[q] = __shfl_down_sync(0xffffffffu, own[q], 1);
        if (!act) continue;
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
            // A fluid cell is interior, so P -/+ 1 are cells of the grid:
            // the warp's edge lanes load them here.
            if (lane == 0) {
                for (int q = 0; q < 3; q++) dn[q] = ld32(a.u[q], P - 1);
                dn[3] = ldp32(a.p, P - 1);
            }
            if (lane == 31) {
                for (int q = 0; q < 3; q++) up[q] = ld32(a.u[q], P + 1);
                up[3] = ldp32(a.p, P + 1);
                up[4] = ldp32(a.U[2], P + 1);
            }
            const float wmx0 = ax.wm[I], wpx0 = ax.wp[I], wmx1 = ax.wm[I + 1], wpx1 = ax.wp[I + 1];
            const float wmy0 = ay.wm[J], wpy0 = ay.wp[J], wmy1 = ay.wm[J + 1], wpy1 = ay.wp[J + 1];
            const float wmz0 = az.wm[K], wpz0 = az.wp[K], wmz1 = az.wm[K + 1], wpz1 = az.wp[K + 1];
            const float Uw = ldp32(a.U[0], P), Ue = ldp32(a.U[0], P + sx);
            const float Vs = ldp32(a.U[1], P), Vn = ldp32(a.U[1], P + sy);
            const float Wd = own[4], Wu = up[4];
            const float rdx = ax.rd[I], rdy = ay.rd[J], rdz = az.rd[K];
            const float kW = ax.km[I], kE = ax.kp[I], kS = ay.km[J], kN = ay.kp[J], kD = az.km[K], kU = az.kp[K];
            const float gx = ax.rdcc[I], gy = ay.rdcc[J], gz = az.rdcc[K];
            const float ff[3] = {f1, f2, f3};
#pragma unroll
            for (int l = 0; l < 3; l++) {
                const double *u = a.u[l];
                const float uc = own[l];
                const float uW = ld32(u, P - sx), uE = ld32(u, P + sx), uS = ld32(u, P - sy), uN = ld32(u, P + sy);
                const float uD = dn[l], uU = up[l];
                const float fw = uW * wmx0 + uc * wpx0, fe = uc * wmx1 + uE * wpx1;
                const float fs = uS * wmy0 + uc * wpy0, fn = uc * wmy1 + uN * wpy1;
                const float fd = uD * wmz0 + uc * wpz0, fu = uc * wmz1 + uU * wpz1;
                const float Nl = (Ue * fe - Uw * fw) * rdx + (Vn * fn - Vs * fs) * rdy + (Wu * fu - Wd * fd) * rdz;
                a.N[l][P] = Nl;
                float dp;
                if (l == 0) dp = (ldp32(a.p, P + sx) - ldp32(a.p, P - sx)) * gx;
                else if (l == 1) dp = (ldp32(a.p, P + sy) - ldp32(a.p, P - sy)) * gy;
                else dp = (up[3] - dn[3]) * gz;
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
// u* = u^n + e, with the pressure-Poisson right-hand side
// (src/ibm3d_fracstep.c:530-647) in FP64 from the stored faces, in two
// passes: u~ = u* + dt G_c p in FP32 on every cell the faces read (i, j, k
// in [-1, N]), then the faces and the right-hand side over tiles of 32 (k)
// x 8 (j) columns marching over planes of i, each face computed once (x
// faces carried along i, y faces in shared memory, z faces by warp
// shuffle).  Tile-edge threads compute their high faces as well; face32t is
// explicitly rounded, so both computations of such a face give its bits.
// ------------------------------------------------------------------------
namespace {

__device__ __forceinline__ float ustar_at(const double *__restrict__ u, const float *__restrict__ e, long long P) {
    return __fadd_rn(ld32(u, P), e[P]);
}

__device__ __forceinline__ bool fg_pair32(uint8_t a, uint8_t b) {
    return (a == FLUID && b == GHOST) || (a == GHOST && b == FLUID);
}

// U* on the face between Pm (index ii-1) and Pp (index ii) from u~ (ut)
// or, across a fluid-ghost pair, from u*.
__device__ __forceinline__ float face32t(const double *__restrict__ u, const float *__restrict__ e,
                                         const float *__restrict__ ut, const double *__restrict__ p, const AxisF &a,
                                         int ii, long long Pm, long long Pp, bool fluid_ghost, float dt) {
    const float wm = a.wm[ii + 2], wp = a.wp[ii + 2];
    if (fluid_ghost) return __fadd_rn(__fmul_rn(ustar_at(u, e, Pm), wm), __fmul_rn(ustar_at(u, e, Pp), wp));
    const float gf = __fmul_rn(__fsub_rn(ldp32(p, Pp), ldp32(p, Pm)), a.rdc[ii + 2]);
    return __fsub_rn(__fadd_rn(__fmul_rn(ut[Pm], wm), __fmul_rn(ut[Pp], wp)), __fmul_rn(dt, gf));
}

}  // namespace

__global__ void __launch_bounds__(256)
k_utilde32(const Grid g, const AxisF ax, const AxisF ay, const AxisF az, const Ustar32Args a, float *__restrict__ ut,
           const float dt) {
    const long long nx2 = g.nx + 2, ny2 = g.ny + 2, nz2 = g.nz + 2, n = nx2 * ny2 * nz2;
    const long long sx = g.sx, sy = g.sy;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q % nz2) - 1;
        const long long r = q / nz2;
        const int j = (int)(r % ny2) - 1, i = (int)(r / ny2) - 1;
        const long long P = cidx(g, i, j, k);
        const float gx = (ldp32(a.p, P + sx) - ldp32(a.p, P - sx)) * ax.rdcc[i + 2];
        const float gy = (ldp32(a.p, P + sy) - ldp32(a.p, P - sy)) * ay.rdcc[j + 2];
        const float gz = (ldp32(a.p, P + 1) - ldp32(a.p, P - 1)) * az.rdcc[k + 2];
        ut[P] = ustar_at(a.u[0], a.e[0], P) + dt * gx;
        ut[g.ncell + P] = ustar_at(a.u[1], a.e[1], P) + dt * gy;
        ut[2 * g.ncell + P] = ustar_at(a.u[2], a.e[2], P) + dt * gz;
    }
}

__global__ void __launch_bounds__(UN_TK * UN_TJ)
k_ustar_faces32(const Grid g, const AxisF ax, const AxisF ay, const AxisF az, const Axis ax64, const Axis ay64,
                const Axis az64, const BCSet bc, const uint8_t *__restrict__ flag, const Ustar32Args a,
                const float *__restrict__ ut, const float dt, const double m2re, const int tk, const int tj,
                const int planes) {
    __shared__ float sVs[2][UN_TJ][UN_TK];
    int b = blockIdx.x;
    const int bk = b % tk;
    b /= tk;
    const int bj = b % tj, bi = b / tj;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int k = bk * UN_TK + tx, j = bj * UN_TJ + ty;
    const int i0 = bi * planes, i1 = min(i0 + planes, g.nx);
    const bool live = j < g.ny && k < g.nz;
    const bool own_vn = ty == UN_TJ - 1 || j == g.ny - 1;
    const bool own_wu = tx == UN_TK - 1 || k == g.nz - 1;
    const long long sx = g.sx, sy = g.sy, n = g.ncell;
    const float *ut0 = ut, *ut1 = ut + n, *ut2 = ut + 2 * n;
    long long P = live ? cidx(g, i0, j, k) : 0;
    uint8_t fc = live ? flag[P] : (uint8_t)SOLID;
    float Uw = 0.0f;
    if (live) Uw = face32t(a.u[0], a.e[0], ut0, a.p, ax, i0, P - sx, P, fg_pair32(flag[P - sx], fc), dt);
    int buf = 0;
    for (int i = i0; i < i1; i++, P += sx) {
        float Ue = 0.f, Vs = 0.f, Wd = 0.f, Vn = 0.f, Wu = 0.f;
        uint8_t fe = SOLID;
        if (live) {
            fe = flag[P + sx];
            Ue = face32t(a.u[0], a.e[0], ut0, a.p, ax, i + 1, P, P + sx, fg_pair32(fc, fe), dt);
            Vs = face32t(a.u[1], a.e[1], ut1, a.p, ay, j, P - sy, P, fg_pair32(flag[P - sy], fc), dt);
            Wd = face32t(a.u[2], a.e[2], ut2, a.p, az, k, P - 1, P, fg_pair32(flag[P - 1], fc), dt);
            if (own_vn) Vn = face32t(a.u[1], a.e[1], ut1, a.p, ay, j + 1, P, P + sy, fg_pair32(fc, flag[P + sy]), dt);
            if (own_wu) Wu = face32t(a.u[2], a.e[2], ut2, a.p, az, k + 1, P, P + 1, fg_pair32(fc, flag[P + 1]), dt);
        }
        sVs[buf][ty][tx] = Vs;
        const float wnext = __shfl_down_sync(0xffffffffu, Wd, 1);
        __syncthreads();
        if (!own_vn) Vn = sVs[buf][ty + 1][tx];
        if (!own_wu) Wu = wnext;
        buf ^= 1;
        if (live) {
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
        Uw = Ue;
        fc = fe;
    }
}

// Outer rows of the Poisson right-hand side: the pressure-BC increments
// p_bc(t + dt) - p_bc(t) (0 for constant values), over the outer-cell list.
__global__ void __launch_bounds__(256)
k_prhs_outer(const Grid g, const BCSet bc, const int *__restrict__ outer, const int nout, double *b) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nout) return;
    const long long P = outer[t];
    int i, j, k;
    cijk_g(g, P, i, j, k);
    int layer;
    const int face = owner_face(g, i, j, k, layer);
    const BCFace &F = bc.f[face];
    double v = 0.0;
    if (F.scur && (F.type == BCT_PRESSURE || F.type == BCT_VELPERIODIC)) {
        const int q = 3 * F.nt + face_line(g, face, i, j, k);
        v = F.snxt[q] - F.scur[q];
    }
    b[P] = v;
}

void launch_ustar_prhs32_tiled(cudaStream_t s, const Grid &g, const AxisF axf[3], const Axis ax64[3],
                               const BCSet &bc, const uint8_t *flag, const Ustar32Args &a, float *ut, double dt,
                               double Re, const int *outer, int nout) {
    const long long nt = (long long)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
    k_utilde32<<<(unsigned)std::min<long long>((nt + 255) / 256, 8 * K32_BLOCKS), 256, 0, s>>>(
        g, axf[0], axf[1], axf[2], a, ut, (float)dt);
    const int tk = (g.nz + UN_TK - 1) / UN_TK, tj = (g.ny + UN_TJ - 1) / UN_TJ, planes = UN_PLANES;
    const int nb = tk * tj * ((g.nx + planes - 1) / planes);
    k_ustar_faces32<<<nb, dim3(UN_TK, UN_TJ), 0, s>>>(g, axf[0], axf[1], axf[2], ax64[0], ax64[1], ax64[2], bc, flag, a,
                                                      ut, (float)dt, -1.0 / (2.0 * Re), tk, tj, planes);
    if (nout > 0) k_prhs_outer<<<(nout + 255) / 256, 256, 0, s>>>(g, bc, outer, nout, a.b);
    note_launches(nout > 0 ? 3 : 2);
}

// ------------------------------------------------------------------------
// update_next (src/ibm3d_fracstep.c:709-805) on tiles: each thread owns a
// (j, k) column of a 32 x 8 tile and marches over the planes of i of its
// tile.  The x face between cells i and i+1 is computed once and carried
// to the next plane as its low face; the high y face of a cell is the low
// y face of the thread at j+1 (shared memory, one barrier per plane); the
// high z face is the low z face of the next lane (warp shuffle).  Tile-edge
// threads compute their high faces themselves.  Per fluid cell that is 3
// face updates on the FP64 pipe instead of 6.  F32: the increment form of
// the FP32-stage step (the cell velocity takes the FP32 increment
// e - dt G_c p'); otherwise the FP64 step.
// ------------------------------------------------------------------------
template <bool F32>
__global__ void __launch_bounds__(UN_TK * UN_TJ)
k_update_next_tiled(const Grid g, const Axis ax, const Axis ay, const Axis az, const DtAxis dx, const DtAxis dy,
                    const DtAxis dz, const AxisF axf, const AxisF ayf, const AxisF azf, const BCSet bc,
                    const uint8_t *__restrict__ flag, const NextArgs a64, const Next32Args a32, const double dt,
                    const int tk, const int tj, const int planes, double *partials, unsigned int *counter,
                    double *maxdiv_out) {
    __shared__ double smem[32];
    __shared__ double sVs[2][UN_TJ][UN_TK];
    const double NaN = __longlong_as_double(0x7ff8000000000000LL);
    int b = blockIdx.x;
    const int bk = b % tk;
    b /= tk;
    const int bj = b % tj, bi = b / tj;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int k = bk * UN_TK + tx, j = bj * UN_TJ + ty;
    const int i0 = bi * planes, i1 = min(i0 + planes, g.nx);
    const bool live = j < g.ny && k < g.nz;
    const bool own_vn = ty == UN_TJ - 1 || j == g.ny - 1;
    const bool own_wu = tx == UN_TK - 1 || k == g.nz - 1;
    const long long sx = g.sx, sy = g.sy;
    const double *Us0 = F32 ? a32.Us[0] : a64.Us[0], *Us1 = F32 ? a32.Us[1] : a64.Us[1],
                 *Us2 = F32 ? a32.Us[2] : a64.Us[2];
    const double *pp = F32 ? a32.pp : a64.pp, *p = F32 ? a32.p : a64.p;
    double *const *Un = F32 ? a32.Un : a64.Un;
    double *const *un = F32 ? a32.un : a64.un;
    double *pn = F32 ? a32.pn : a64.pn;
    const int J = j + 2, K = k + 2;
    double mdiv = 0.0;
    long long P = live ? cidx(g, i0, j, k) : 0;
    uint8_t fc = live ? flag[P] : (uint8_t)SOLID;
    double ppc = live ? pp[P] : 0.0;
    double Uw = NaN;
    if (live && flag[P - sx] != SOLID && fc != SOLID) Uw = Us0[P] - dx.dtrdc[i0 + 2] * (ppc - pp[P - sx]);
    int buf = 0;
    for (int i = i0; i < i1; i++, P += sx) {
        const int I = i + 2;
        double Ue = NaN, Vs = NaN, Wd = NaN, Vn = NaN, Wu = NaN;
        uint8_t fe = SOLID;
        double ppe = 0.0;
        if (live) {
            fe = flag[P + sx];
            ppe = pp[P + sx];
            if (fc != SOLID && fe != SOLID) Ue = Us0[P + sx] - dx.dtrdc[I + 1] * (ppe - ppc);
            if (fc != SOLID && flag[P - sy] != SOLID) Vs = Us1[P] - dy.dtrdc[J] * (ppc - pp[P - sy]);
            if (fc != SOLID && flag[P - 1] != SOLID) Wd = Us2[P] - dz.dtrdc[K] * (ppc - pp[P - 1]);
            if (own_vn && fc != SOLID && flag[P + sy] != SOLID) Vn = Us1[P + sy] - dy.dtrdc[J + 1] * (pp[P + sy] - ppc);
            if (own_wu && fc != SOLID && flag[P + 1] != SOLID) Wu = Us2[P + 1] - dz.dtrdc[K + 1] * (pp[P + 1] - ppc);
        }
        sVs[buf][ty][tx] = Vs;
        const double wnext = __shfl_down_sync(0xffffffffu, Wd, 1);
        __syncthreads();
        if (!own_vn) Vn = sVs[buf][ty + 1][tx];
        if (!own_wu) Wu = wnext;
        buf ^= 1;
        if (live) {
            Un[0][P] = Uw;
            Un[1][P] = Vs;
            Un[2][P] = Wd;
            if (i == g.nx - 1) Un[0][P + sx] = Ue;
            if (j == g.ny - 1) Un[1][P + sy] = Vn;
            if (k == g.nz - 1) Un[2][P + 1] = Wu;
            pn[P] = (fc == FLUID || fc == GHOST) ? p[P] + ppc : NaN;
            if (fc == FLUID) {
                const double ppw = pp[P - sx], pps = pp[P - sy], ppn = pp[P + sy], ppd = pp[P - 1], ppu = pp[P + 1];
                if (F32) {
                    const float gx = (d2f_int(ppe) - d2f_int(ppw)) * axf.rdcc[I];
                    const float gy = (d2f_int(ppn) - d2f_int(pps)) * ayf.rdcc[J];
                    const float gz = (d2f_int(ppu) - d2f_int(ppd)) * azf.rdcc[K];
                    const float dtf = (float)dt;
                    un[0][P] = a32.u[0][P] + f2d_int(a32.e[0][P] - dtf * gx);
                    un[1][P] = a32.u[1][P] + f2d_int(a32.e[1][P] - dtf * gy);
                    un[2][P] = a32.u[2][P] + f2d_int(a32.e[2][P] - dtf * gz);
                } else {
                    un[0][P] = a64.us[0][P] - dx.dtrdcc[I] * (ppe - ppw);
                    un[1][P] = a64.us[1][P] - dy.dtrdcc[J] * (ppn - pps);
                    un[2][P] = a64.us[2][P] - dz.dtrdcc[K] * (ppu - ppd);
                }
                if (!(bc.p_singular && i == 0 && j == 0 && k == 0)) {
                    const double div = (Ue - Uw) * ax.rd[I] + (Vn - Vs) * ay.rd[J] + (Wu - Wd) * az.rd[K];
                    mdiv = nanmax(mdiv, fabs(div));
                }
            } else if (fc == SOLID) {
                un[0][P] = un[1][P] = un[2][P] = NaN;
            }
        }
        Uw = Ue;
        fc = fe;
        ppc = ppe;
    }
    // Maximum over the block, then over the blocks (the last block to
    // finish reduces every block's value in a fixed order).
    const int t = ty * UN_TK + tx, lane = t & 31, warp = t >> 5;
    double x = mdiv;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = nanmax(x, __shfl_down_sync(0xffffffffu, x, o));
    if (lane == 0) smem[warp] = x;
    __syncthreads();
    __shared__ bool last;
    if (t == 0) {
        double m = 0.0;
        for (int w = 0; w < (UN_TK * UN_TJ) / 32; w++) m = nanmax(m, smem[w]);
        partials[blockIdx.x] = m;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double m = 0.0;
    for (int q = t; q < (int)gridDim.x; q += UN_TK * UN_TJ) m = nanmax(m, __ldcg(partials + q));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = nanmax(m, __shfl_down_sync(0xffffffffu, m, o));
    __syncthreads();
    if (lane == 0) smem[warp] = m;
    __syncthreads();
    if (t == 0) {
        double r = 0.0;
        for (int w = 0; w < (UN_TK * UN_TJ) / 32; w++) r = nanmax(r, smem[w]);
        *maxdiv_out = r;
        *counter = 0;
    }
}

void launch_update_next_tiled(cudaStream_t s, const Grid &g, const Axis ax64[3], const DtAxis dta[3],
                              const AxisF axf[3], const BCSet &bc, const uint8_t *flag, const NextArgs *a64,
                              const Next32Args *a32, double dt, double *partials, unsigned int *counter,
                              double *maxdiv_out) {
    const int tk = (g.nz + UN_TK - 1) / UN_TK, tj = (g.ny + UN_TJ - 1) / UN_TJ;
    // UN_PLANES planes per tile, more on grids whose tiles would outnumber
    // the reduction's partials (8 x 4096).
    int planes = UN_PLANES;
    while ((long long)tk * tj * ((g.nx + planes - 1) / planes) > 8 * 4096) planes *= 2;
    const int nb = tk * tj * ((g.nx + planes - 1) / planes);
    const dim3 blk(UN_TK, UN_TJ);
    if (a32)
        k_update_next_tiled<true><<<nb, blk, 0, s>>>(g, ax64[0], ax64[1], ax64[2], dta[0], dta[1], dta[2], axf[0],
                                                    axf[1], axf[2], bc, flag, NextArgs{}, *a32, dt, tk, tj, planes,
                                                    partials, counter, maxdiv_out);
    else
        k_update_next_tiled<false><<<nb, blk, 0, s>>>(g, ax64[0], ax64[1], ax64[2], dta[0], dta[1], dta[2], axf[0],
                                                     axf[1], axf[2], bc, flag, *a64, Next32Args{}, dt, tk, tj,
                                                     planes, partials, counter, maxdiv_out);
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
