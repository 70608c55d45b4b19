// Explicit kernels of one fractional step (FP64).
//
// Each kernel restates one routine of src/ibm3d_fracstep.c (cited per
// kernel) over the padded grid.  Divisions by metric terms are replaced by
// products with 1-D reciprocal tables built once at assembly: FP64
// arithmetic, not HBM, is the scarce resource on GB300, and the tables cost
// a few KB of L1-resident loads.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace ibm {

static inline unsigned grid_for(long long n, int block) {
    long long b = (n + block - 1) / block;
    return (unsigned)(b > 0 ? b : 1);
}

// ------------------------------------------------------------------------
// calc_N (src/ibm3d_fracstep.c:117-170) fused with the momentum right-hand
// side of calc_u_star (src/ibm3d_fracstep.c:237-352): AB2 convection,
// Crank-Nicolson explicit half, cell-centred pressure gradient, body force
// and subgrid-stress divergence.  Outer rows carry the velocity BC value
// (VELOCITY faces) or 0; interior non-fluid rows are 0 and N is NaN there.
// ------------------------------------------------------------------------
// Two blocks per SM: 128 registers, no spills (218 unbounded, one block
// per SM); the kernel is bound by the FP64 pipe, which more resident warps
// keep busier.
__global__ void __launch_bounds__(256, 2)
k_conv_rhs(const Grid g, const Axis ax, const Axis ay, const Axis az, const BCSet bc,
           const uint8_t *__restrict__ flag, ConvArgs a, const double dt, const double f1,
           const double f2, const double f3, const int les) {
    const long long n = g.ncell;
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cijk_g(g, P, i, j, k);
        int layer;
        const int f = owner_face(g, i, j, k, layer);
        if (f >= 0) {
            const BCFace &F = bc.f[f];
            const bool vel = F.type == BCT_VELOCITY;
            const double *sv = F.scur ? F.scur + face_line(g, f, i, j, k) : nullptr;
#pragma unroll
            for (int l = 0; l < 3; l++) a.b[l][P] = vel ? (sv ? sv[l * F.nt] : F.val[l]) : 0.0;
            continue;
        }
        if (flag[P] != FLUID) {
            a.N[0][P] = a.N[1][P] = a.N[2][P] = __longlong_as_double(0x7ff8000000000000LL);
            a.b[0][P] = a.b[1][P] = a.b[2][P] = 0.0;
            continue;
        }
        const long long sx = g.sx, sy = g.sy;
        const int I = i + 2, J = j + 2, K = k + 2;
        const double wmx0 = ax.wm[I], wpx0 = ax.wp[I], wmx1 = ax.wm[I + 1], wpx1 = ax.wp[I + 1];
        const double wmy0 = ay.wm[J], wpy0 = ay.wp[J], wmy1 = ay.wm[J + 1], wpy1 = ay.wp[J + 1];
        const double wmz0 = az.wm[K], wpz0 = az.wp[K], wmz1 = az.wm[K + 1], wpz1 = az.wp[K + 1];
        const double Uw = a.U[0][P], Ue = a.U[0][P + sx];
        const double Vs = a.U[1][P], Vn = a.U[1][P + sy];
        const double Wd = a.U[2][P], Wu = a.U[2][P + 1];
        const double rdx = ax.rd[I], rdy = ay.rd[J], rdz = az.rd[K];
        const double kW = ax.km[I], kE = ax.kp[I], kS = ay.km[J], kN = ay.kp[J], kD = az.km[K], kU = az.kp[K];
        const double cdiag = 1 - kW - kE - kS - kN - kD - kU;
        const double gx = ax.rdcc[I], gy = ay.rdcc[J], gz = az.rdcc[K];
        const double ff[3] = {f1, f2, f3};
#pragma unroll
        for (int l = 0; l < 3; l++) {
            const double *u = a.u[l];
            const double uc = u[P];
            const double uW = u[P - sx], uE = u[P + sx], uS = u[P - sy], uN = u[P + sy];
            const double uD = u[P - 1], uU = u[P + 1];
            const double fw = uW * wmx0 + uc * wpx0, fe = uc * wmx1 + uE * wpx1;
            const double fs = uS * wmy0 + uc * wpy0, fn = uc * wmy1 + uN * wpy1;
            const double fd = uD * wmz0 + uc * wpz0, fu = uc * wmz1 + uU * wpz1;
            const double Nl = (Ue * fe - Uw * fw) * rdx + (Vn * fn - Vs * fs) * rdy + (Wu * fu - Wd * fd) * rdz;
            a.N[l][P] = Nl;
            double dp;
            if (l == 0) dp = (a.p[P + sx] - a.p[P - sx]) * gx;
            else if (l == 1) dp = (a.p[P + sy] - a.p[P - sy]) * gy;
            else dp = (a.p[P + 1] - a.p[P - 1]) * gz;
            double divtau = 0.0;
            if (les) {
                // tau[l][m] with symmetric storage 11,12,13,22,23,33.
                const int t1 = l == 0 ? 0 : l == 1 ? 1 : 2;
                const int t2 = l == 0 ? 1 : l == 1 ? 3 : 4;
                const int t3 = l == 0 ? 2 : l == 1 ? 4 : 5;
                divtau = (a.tau[t1][P + sx] - a.tau[t1][P - sx]) * gx +
                         (a.tau[t2][P + sy] - a.tau[t2][P - sy]) * gy +
                         (a.tau[t3][P + 1] - a.tau[t3][P - 1]) * gz;
            }
            const double fl = a.force ? a.force[l * n + P] : ff[l];
            a.b[l][P] = -dt / 2 * (3 * Nl - a.Np[l][P]) - dt * dp + cdiag * uc + kW * uW + kE * uE + kS * uS +
                        kN * uN + kD * uD + kU * uU + dt * fl - dt * divtau;
        }
    }
}

// ------------------------------------------------------------------------
// Initial guess of the momentum solve: u* from u^n (NaN on solid cells,
// where the solve's rows are the identity on a zero right-hand side, is
// replaced by 0).
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_velocity_guess(const long long n, const double *__restrict__ u0, const double *__restrict__ u1,
                 const double *__restrict__ u2, double *__restrict__ x) {
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        const double a = u0[P], b = u1[P], c = u2[P];
        x[P] = a == a ? a : 0.0;
        x[n + P] = b == b ? b : 0.0;
        x[2 * n + P] = c == c ? c : 0.0;
    }
}

void launch_velocity_guess(cudaStream_t s, const Grid &g, double *const u[3], double *x) {
    k_velocity_guess<<<grid_for(g.ncell, 256), 256, 0, s>>>(g.ncell, u[0], u[1], u[2], x);
    note_launches(1);
}

void launch_conv_rhs(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                     const BCSet &bc, const uint8_t *flag, const ConvArgs &a, double dt, const double f[3],
                     int les) {
    k_conv_rhs<<<grid_for(g.ncell, 256), 256, 0, s>>>(g, ax, ay, az, bc, flag, a, dt, f[0], f[1], f[2], les);
    note_launches(1);
}

// ------------------------------------------------------------------------
// Smagorinsky stress (src/ibm3d_turb.c:8-82): S_ij by central differences,
// Delta = 2 cbrt(dx dy dz), l = min(Cs Delta, 0.41 phi), tau = -2 l^2 |S| S
// on fluid cells; other cells keep their (zero) value.
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_smagorinsky(const Grid g, const Axis ax, const Axis ay, const Axis az, const uint8_t *__restrict__ flag,
              const double *__restrict__ lvset, const double *__restrict__ u1, const double *__restrict__ u2,
              const double *__restrict__ u3, TauArgs t, const double cs) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        ijk_interior(g, q, i, j, k);
        const long long P = cidx(g, i, j, k);
        if (flag[P] != FLUID) continue;
        const long long sx = g.sx, sy = g.sy;
        const double gx = ax.rdcc[i + 2], gy = ay.rdcc[j + 2], gz = az.rdcc[k + 2];
        const double S11 = (u1[P + sx] - u1[P - sx]) * gx;
        const double S12 = 0.5 * ((u1[P + sy] - u1[P - sy]) * gy + (u2[P + sx] - u2[P - sx]) * gx);
        const double S13 = 0.5 * ((u1[P + 1] - u1[P - 1]) * gz + (u3[P + sx] - u3[P - sx]) * gx);
        const double S22 = (u2[P + sy] - u2[P - sy]) * gy;
        const double S23 = 0.5 * ((u2[P + 1] - u2[P - 1]) * gz + (u3[P + sy] - u3[P - sy]) * gy);
        const double S33 = (u3[P + 1] - u3[P - 1]) * gz;
        const double delta = 2 * cbrt(ax.d[i + 2] * ay.d[j + 2] * az.d[k + 2]);
        double sm = 0;
        sm += 2 * (S11 * S11); sm += 2 * (S12 * S12); sm += 2 * (S13 * S13);
        sm += 2 * (S12 * S12); sm += 2 * (S22 * S22); sm += 2 * (S23 * S23);
        sm += 2 * (S13 * S13); sm += 2 * (S23 * S23); sm += 2 * (S33 * S33);
        sm = sqrt(sm);
        const double a = cs * delta, b = 0.41 * lvset[P];
        const double l = a < b ? a : b;
        const double c = -2 * (l * l) * sm;
        t.tau[0][P] = c * S11; t.tau[1][P] = c * S12; t.tau[2][P] = c * S13;
        t.tau[3][P] = c * S22; t.tau[4][P] = c * S23; t.tau[5][P] = c * S33;
    }
}

void launch_smagorinsky(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                        const uint8_t *flag, const double *lvset, const double *const u[3], const TauArgs &t,
                        double cs) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    k_smagorinsky<<<grid_for(n, 256), 256, 0, s>>>(g, ax, ay, az, flag, lvset, u[0], u[1], u[2], t, cs);
    note_launches(1);
}

// ------------------------------------------------------------------------
// calc_u_tilde + calc_U_star (src/ibm3d_fracstep.c:388-487) fused with the
// pressure-Poisson right-hand side (src/ibm3d_fracstep.c:530-647).  u~ is
// formed on the fly; each thread writes the low face of its cell on each
// axis (and the high face for the last cell) and recomputes the high faces
// for its divergence.  Outer rows of b are the pressure-BC increments,
// which are 0 for constant boundary values.
// ------------------------------------------------------------------------
__device__ inline double face_ustar(const double *__restrict__ us, const double *__restrict__ p,
                                    const Axis &a, int ii, long long Pm, long long Pp, long long s,
                                    bool fluid_ghost, double dt) {
    // Face between cells Pm (index ii-1) and Pp (index ii) along stride s.
    if (fluid_ghost) return us[Pm] * a.wm[ii + 2] + us[Pp] * a.wp[ii + 2];
    const double tm = us[Pm] + dt * (p[Pm + s] - p[Pm - s]) * a.rdcc[ii + 1];
    const double tp = us[Pp] + dt * (p[Pp + s] - p[Pp - s]) * a.rdcc[ii + 2];
    return tm * a.wm[ii + 2] + tp * a.wp[ii + 2] - dt * (p[Pp] - p[Pm]) * a.rdc[ii + 2];
}

__device__ inline bool fg_pair(uint8_t a, uint8_t b) {
    return (a == FLUID && b == GHOST) || (a == GHOST && b == FLUID);
}

__global__ void __launch_bounds__(256)
k_ustar_prhs(const Grid g, const Axis ax, const Axis ay, const Axis az, const BCSet bc,
             const uint8_t *__restrict__ flag, UstarArgs a, const double dt, const double Re) {
    const long long n = g.ncell;
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cijk_g(g, P, i, j, k);
        int layer;
        const int face = owner_face(g, i, j, k, layer);
        if (face >= 0) {
            // Pressure-Dirichlet rows: p_bc(t + dt) - p_bc(t), zero for
            // constant values (src/ibm3d_fracstep.c:556-645).
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
        const double Uw = face_ustar(a.us[0], a.p, ax, i, P - sx, P, sx, fg_pair(flag[P - sx], fc), dt);
        const double Ue = face_ustar(a.us[0], a.p, ax, i + 1, P, P + sx, sx, fg_pair(fc, flag[P + sx]), dt);
        const double Vs = face_ustar(a.us[1], a.p, ay, j, P - sy, P, sy, fg_pair(flag[P - sy], fc), dt);
        const double Vn = face_ustar(a.us[1], a.p, ay, j + 1, P, P + sy, sy, fg_pair(fc, flag[P + sy]), dt);
        const double Wd = face_ustar(a.us[2], a.p, az, k, P - 1, P, 1, fg_pair(flag[P - 1], fc), dt);
        const double Wu = face_ustar(a.us[2], a.p, az, k + 1, P, P + 1, 1, fg_pair(fc, flag[P + 1]), dt);
        a.Us[0][P] = Uw;
        a.Us[1][P] = Vs;
        a.Us[2][P] = Wd;
        if (i == g.nx - 1) a.Us[0][P + sx] = Ue;
        if (j == g.ny - 1) a.Us[1][P + sy] = Vn;
        if (k == g.nz - 1) a.Us[2][P + 1] = Wu;
        double rhs = 0.0;
        if (bc.p_singular && i == 0 && j == 0 && k == 0) {
            rhs = 0.0;
        } else if (fc == FLUID) {
            const int I = i + 2, J = j + 2, K = k + 2;
            const double csum = ay.kp[J] + ax.kp[I] + ay.km[J] + ax.km[I] + az.km[K] + az.kp[K];
            rhs = -1 / (2 * Re) * ((Ue - Uw) * ax.rd[I] + (Vn - Vs) * ay.rd[J] + (Wu - Wd) * az.rd[K]);
            rhs /= csum;
        }
        a.b[P] = rhs;
    }
}

void launch_ustar_prhs(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                       const BCSet &bc, const uint8_t *flag, const UstarArgs &a, double dt, double Re) {
    k_ustar_prhs<<<grid_for(g.ncell, 256), 256, 0, s>>>(g, ax, ay, az, bc, flag, a, dt, Re);
    note_launches(1);
}

// ------------------------------------------------------------------------
// update_outer (src/ibm3d_fracstep.c:855-1906): velocity and pressure
// outer-layer fills.  Three launches keep the reference's face order
// (x faces, then y faces reading the x-filled edges, then z faces).
// ------------------------------------------------------------------------
__device__ inline void fill_line(const BCFace &F, int f, const double *smp, double *u0, double *u1, double *u2,
                                 double *p, long long c0, long long c1, long long o1, long long o2, long long img1,
                                 long long img2) {
    double *u[3] = {u0, u1, u2};
    const int axis = face_axis(f);
    switch (F.type) {
    case BCT_VELOCITY:
        for (int l = 0; l < 3; l++) {
            const double v = smp ? smp[l * F.nt] : F.val[l];
            u[l][o1] = F.fv_a[0] * v - F.fv_b[0] * u[l][c0];
            u[l][o2] = F.fv_a[1] * v - F.fv_b[1] * u[l][c1];
        }
        break;
    case BCT_PRESSURE:
        for (int l = 0; l < 3; l++) {
            u[l][o1] = F.fe_a[0] * u[l][c0] - F.fe_b[0] * u[l][c1];
            u[l][o2] = F.fe_a[1] * u[l][o1] - F.fe_b[1] * u[l][c0];
        }
        break;
    case BCT_SLIP:
        for (int l = 0; l < 3; l++) {
            if (l == axis) {
                u[l][o1] = -F.fv_b[0] * u[l][c0];
                u[l][o2] = -F.fv_b[1] * u[l][c1];
            } else {
                u[l][o1] = u[l][c0];
                u[l][o2] = u[l][c1];
            }
        }
        break;
    case BCT_PERIODIC:
    case BCT_VELPERIODIC:
        for (int l = 0; l < 3; l++) {
            u[l][o1] = u[l][img1];
            u[l][o2] = u[l][img2];
        }
        break;
    default:;
    }
    switch (F.type) {
    case BCT_VELOCITY:
    case BCT_SLIP:
        p[o1] = p[c0];
        p[o2] = p[c1];
        break;
    case BCT_PRESSURE:
    case BCT_VELPERIODIC: {
        const double v = smp ? smp[3 * F.nt] : F.pval;
        p[o1] = F.fp_a[0] * v - F.fp_b[0] * p[c0];
        p[o2] = F.fp_a[1] * v - F.fp_b[1] * p[c1];
        break;
    }
    case BCT_PERIODIC:
        p[o1] = p[img1];
        p[o2] = p[img2];
        break;
    default:;
    }
}

__global__ void k_fill_outer(const Grid g, const BCSet bc, const int axis, const int when, double *u0, double *u1,
                             double *u2, double *p) {
    // axis 0: lines over (j,k) interior; axis 1: (i in [-2,nx+2), k interior);
    // axis 2: (i in [-2,nx+2), j in [-2,ny+2)).
    long long n;
    int na, nb;
    if (axis == 0) { na = g.ny; nb = g.nz; }
    else if (axis == 1) { na = g.nx + 4; nb = g.nz; }
    else { na = g.nx + 4; nb = g.ny + 4; }
    n = (long long)na * nb;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int A = (int)(q / nb), B = (int)(q % nb);
        long long s, base_lo, base_hi;
        int N;
        if (axis == 0) {
            s = g.sx; N = g.nx;
            base_lo = cidx(g, 0, A, B);
        } else if (axis == 1) {
            s = g.sy; N = g.ny;
            base_lo = cidx(g, A - 2, 0, B);
        } else {
            s = 1; N = g.nz;
            base_lo = cidx(g, A - 2, B - 2, 0);
        }
        base_hi = base_lo + (long long)(N - 1) * s;
        const int flo = axis == 0 ? F_W : axis == 1 ? F_S : F_D;
        const int fhi = axis == 0 ? F_E : axis == 1 ? F_N : F_U;
        // Outer line of this (A, B): same position on both faces of the axis.
        const int line = axis == 0 ? (A + 2) * (g.nz + 4) + (B + 2) : axis == 1 ? A * (g.nz + 4) + (B + 2)
                                                                                : A * (g.ny + 4) + B;
        const BCFace &Flo = bc.f[flo], &Fhi = bc.f[fhi];
        const double *slo = Flo.scur ? (when ? Flo.snxt : Flo.scur) + line : nullptr;
        const double *shi = Fhi.scur ? (when ? Fhi.snxt : Fhi.scur) + line : nullptr;
        // Low face: c0 = 0, c1 = 1, o1 = -1, o2 = -2; periodic images N-1, N-2.
        fill_line(Flo, flo, slo, u0, u1, u2, p, base_lo, base_lo + s, base_lo - s, base_lo - 2 * s,
                  base_lo + (long long)(N - 1) * s, base_lo + (long long)(N - 2) * s);
        // High face: c0 = N-1, c1 = N-2, o1 = N, o2 = N+1; periodic images 0, 1.
        fill_line(Fhi, fhi, shi, u0, u1, u2, p, base_hi, base_hi - s, base_hi + s, base_hi + 2 * s, base_lo,
                  base_lo + s);
    }
}

void launch_fill_outer(cudaStream_t s, const Grid &g, const BCSet &bc, double *const u[3], double *p, int when) {
    const long long nx = (long long)g.ny * g.nz, ny = (long long)(g.nx + 4) * g.nz,
                    nz = (long long)(g.nx + 4) * (g.ny + 4);
    k_fill_outer<<<grid_for(nx, 128), 128, 0, s>>>(g, bc, 0, when, u[0], u[1], u[2], p);
    k_fill_outer<<<grid_for(ny, 128), 128, 0, s>>>(g, bc, 1, when, u[0], u[1], u[2], p);
    k_fill_outer<<<grid_for(nz, 128), 128, 0, s>>>(g, bc, 2, when, u[0], u[1], u[2], p);
    note_launches(3);
}

// ------------------------------------------------------------------------
// interp_stag_vel (src/ibm3d_fracstep.c:807-845): face velocities from the
// cell velocities, including the outer tangential range.
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_interp_stag(const Grid g, const Axis ax, const Axis ay, const Axis az, const double *__restrict__ u1,
              const double *__restrict__ u2, const double *__restrict__ u3, double *U1, double *U2, double *U3) {
    const long long n = g.ncell;
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cijk_g(g, P, i, j, k);
        if (i >= 0 && i <= g.nx) U1[P] = u1[P - g.sx] * ax.wm[i + 2] + u1[P] * ax.wp[i + 2];
        if (j >= 0 && j <= g.ny) U2[P] = u2[P - g.sy] * ay.wm[j + 2] + u2[P] * ay.wp[j + 2];
        if (k >= 0 && k <= g.nz) U3[P] = u3[P - 1] * az.wm[k + 2] + u3[P] * az.wp[k + 2];
    }
}

void launch_interp_stag(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                        const double *const u[3], double *const U[3]) {
    k_interp_stag<<<grid_for(g.ncell, 256), 256, 0, s>>>(g, ax, ay, az, u[0], u[1], u[2], U[0], U[1], U[2]);
    note_launches(1);
}

// ------------------------------------------------------------------------
// update_ghost (src/ibm3d_fracstep.c:1915-1976).  The reference sweeps the
// ghost cells in lexicographic order and updates them in place, so a ghost
// whose stencil holds a ghost with a lower index sees its new value and one
// with a higher index sees the value left in the array.  Ghosts are sorted
// into dependency levels at assembly; values of "higher" ghosts are
// snapshotted first, then the levels run in order inside one block.
// ------------------------------------------------------------------------
// The ghosts' rows are FP64 (interpolation sums and the reference's
// divisions): spread over the whole GPU - one launch snapshots the values
// "higher" ghosts read, then one launch per level (a level reads only the
// snapshot, fluid cells and earlier levels) - rather than inside one
// block, whose single SM's FP64 pipe bound it.
__global__ void __launch_bounds__(256)
k_ghost_snapshot(GhostArgs a, const double *u0, const double *u1, const double *u2, const double *p) {
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.nghost) return;
    const long long c = a.cell[g];
    a.old[4 * g + 0] = u0[c];
    a.old[4 * g + 1] = u1[c];
    a.old[4 * g + 2] = u2[c];
    a.old[4 * g + 3] = p[c];
}

__global__ void __launch_bounds__(128)
k_ghost_level(GhostArgs a, const int g0, const int g1, double *u0, double *u1, double *u2, double *p) {
    pdl_enter();
    const int g = g0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= g1) return;
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (int e = 0; e < 8; e++) {
        const int kind = a.kind[8 * g + e];
        if (kind == GK_SKIP) continue;
        const double w = a.w[8 * g + e];
        if (kind == GK_OLD) {
            const int h = a.ref[8 * g + e];
            s0 += w * a.old[4 * h + 0];
            s1 += w * a.old[4 * h + 1];
            s2 += w * a.old[4 * h + 2];
            s3 += w * a.old[4 * h + 3];
        } else {
            const long long c = a.ref[8 * g + e];
            s0 += w * u0[c];
            s1 += w * u1[c];
            s2 += w * u2[c];
            s3 += w * p[c];
        }
    }
    const long long c = a.cell[g];
    const double lu = 1 + a.wself[g], lp = 1 - a.wself[g];
    u0[c] = -s0 / lu;
    u1[c] = -s1 / lu;
    u2[c] = -s2 / lu;
    if (lp != 0) p[c] = s3 / lp;
}

void launch_ghost_update(cudaStream_t s, const GhostArgs &a, double *const u[3], double *p) {
    if (a.nghost == 0) return;
    launch_pdl(k_ghost_snapshot, (a.nghost + 255) / 256, 256, 0, s, a, (const double *)u[0], (const double *)u[1],
               (const double *)u[2], (const double *)p);
    for (int lev = 0; lev < a.nlevels; lev++) {
        const int g0 = a.hlevel_start[lev], g1 = a.hlevel_start[lev + 1];
        if (g1 > g0) launch_pdl(k_ghost_level, (g1 - g0 + 127) / 128, 128, 0, s, a, g0, g1, u[0], u[1], u[2], p);
    }
    note_launches(1 + a.nlevels);
}

// Interior solid cells -> NaN (the SOLID branch of update_ghost).
__global__ void k_solid_nan(const Grid g, const uint8_t *__restrict__ flag, double *u0, double *u1, double *u2,
                            double *p) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const double NaN = __longlong_as_double(0x7ff8000000000000LL);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        ijk_interior(g, q, i, j, k);
        const long long P = cidx(g, i, j, k);
        if (flag[P] == SOLID) u0[P] = u1[P] = u2[P] = p[P] = NaN;
    }
}

void launch_solid_nan(cudaStream_t s, const Grid &g, const uint8_t *flag, double *const u[3], double *p) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    k_solid_nan<<<grid_for(n, 256), 256, 0, s>>>(g, flag, u[0], u[1], u[2], p);
    note_launches(1);
}

// ------------------------------------------------------------- export ---
// Result export (src/ibm3d_export.c:71-141): the four FP64 fields become
// float arrays in the file's [z][y][x] order over the padded grid, and
// vorticity magnitude and Q follow from those float values with the
// reference's arithmetic: each gradient is a float difference divided by
// a double coordinate difference, rounded to float; products and sums in
// float, left to right; |omega| = float(sqrt(double(sum of squares))).
// Neighbour indices are clamped to the padded range [0, N+3].

// Tiled transpose: a 32x32 (i, k) tile of plane j, read k-contiguous and
// written i-contiguous.
__global__ void __launch_bounds__(256)
k_export_transpose(const Grid g, const double *__restrict__ f0, const double *__restrict__ f1,
                   const double *__restrict__ f2, const double *__restrict__ f3, float *__restrict__ out) {
    __shared__ float tile[4][32][33];
    const int NX = g.nx + 4, NY = g.ny + 4, NZ = g.nz + 4;
    const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32, j = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const double *src[4] = {f0, f1, f2, f3};
    for (int r = 0; r < 32; r += 8) {
        const int i = i0 + ty + r, k = k0 + tx;
        if (i < NX && k < NZ) {
            const long long P = (long long)i * g.sx + (long long)j * g.sy + k;
#pragma unroll
            for (int f = 0; f < 4; f++) tile[f][ty + r][tx] = __double2float_rn(src[f][P]);
        }
    }
    __syncthreads();
    const long long plane = (long long)NX * NY * NZ;
    for (int r = 0; r < 32; r += 8) {
        const int k = k0 + ty + r, i = i0 + tx;
        if (i < NX && k < NZ) {
            const long long o = ((long long)k * NY + j) * NX + i;
#pragma unroll
            for (int f = 0; f < 4; f++) out[f * plane + o] = tile[f][tx][ty + r];
        }
    }
}

__device__ __forceinline__ float export_grad(float a, float b, double ca, double cb) {
    return __double2float_rn(__ddiv_rn((double)__fsub_rn(a, b), __dsub_rn(ca, cb)));
}

// out holds u, v, w, p (NX*NY*NZ floats each, x fastest); vorticity and Q
// are written after them.
__global__ void __launch_bounds__(256)
k_export_vort_q(const Grid g, const double *__restrict__ xc, const double *__restrict__ yc,
                const double *__restrict__ zc, float *__restrict__ out) {
    const int NX = g.nx + 4, NY = g.ny + 4, NZ = g.nz + 4;
    const long long plane = (long long)NX * NY * NZ;
    const float *u = out, *v = out + plane, *w = out + 2 * plane;
    float *vort = out + 4 * plane, *q = out + 5 * plane;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < plane;
         o += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(o % NX);
        const int j = (int)(o / NX % NY);
        const int k = (int)(o / ((long long)NX * NY));
        const int ip = max(i - 1, 0), in = min(i + 1, NX - 1);
        const int jp = max(j - 1, 0), jn = min(j + 1, NY - 1);
        const int kp = max(k - 1, 0), kn = min(k + 1, NZ - 1);
        const long long xn = o - i + in, xp = o - i + ip;
        const long long yn = o + (long long)(jn - j) * NX, yp = o + (long long)(jp - j) * NX;
        const long long zn = o + (long long)(kn - k) * NX * NY, zp = o + (long long)(kp - k) * NX * NY;
        const double cxn = xc[in], cxp = xc[ip], cyn = yc[jn], cyp = yc[jp], czn = zc[kn], czp = zc[kp];
        const float dudx = export_grad(u[xn], u[xp], cxn, cxp);
        const float dudy = export_grad(u[yn], u[yp], cyn, cyp);
        const float dudz = export_grad(u[zn], u[zp], czn, czp);
        const float dvdx = export_grad(v[xn], v[xp], cxn, cxp);
        const float dvdy = export_grad(v[yn], v[yp], cyn, cyp);
        const float dvdz = export_grad(v[zn], v[zp], czn, czp);
        const float dwdx = export_grad(w[xn], w[xp], cxn, cxp);
        const float dwdy = export_grad(w[yn], w[yp], cyn, cyp);
        const float dwdz = export_grad(w[zn], w[zp], czn, czp);
        const float ox = __fsub_rn(dwdy, dvdz), oy = __fsub_rn(dudz, dwdx), oz = __fsub_rn(dvdx, dudy);
        const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(ox, ox), __fmul_rn(oy, oy)), __fmul_rn(oz, oz));
        vort[o] = __double2float_rn(__dsqrt_rn((double)s2));
        float t = __fadd_rn(__fmul_rn(dudx, dvdy), __fmul_rn(dvdy, dwdz));
        t = __fadd_rn(t, __fmul_rn(dwdz, dudx));
        t = __fsub_rn(t, __fmul_rn(dudy, dvdx));
        t = __fsub_rn(t, __fmul_rn(dvdz, dwdy));
        t = __fsub_rn(t, __fmul_rn(dudz, dwdx));
        q[o] = t;
    }
}

void launch_export_fields(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                          const double *const u[3], const double *p, float *out) {
    const int NX = g.nx + 4, NY = g.ny + 4, NZ = g.nz + 4;
    const dim3 tgrid((NX + 31) / 32, (NZ + 31) / 32, NY);
    k_export_transpose<<<tgrid, dim3(32, 8), 0, s>>>(g, u[0], u[1], u[2], p, out);
    const long long plane = (long long)NX * NY * NZ;
    const long long blocks = std::min<long long>((plane + 255) / 256, 152LL * 64);
    k_export_vort_q<<<(unsigned)blocks, 256, 0, s>>>(g, ax.c, ay.c, az.c, out);
    note_launches(2);
}

// ------------------------------------------------------------------------
// Initial guess of a warm-started pressure solve: with two earlier
// increments, the linear extrapolation 2 p'_{n-1} - p'_{n-2}; otherwise the
// last increment as it stands.  prev receives p'_{n-1}.  The history count
// is read here and advanced by k_pressure_history after this launch.
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_pressure_guess(const long long n, double *__restrict__ pp, double *__restrict__ prev, const int *hist) {
    const bool extrapolate = *hist >= 2;
    for (long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x; P < n;
         P += (long long)gridDim.x * blockDim.x) {
        const double a = pp[P];
        if (extrapolate) pp[P] = 2 * a - prev[P];
        prev[P] = a;
    }
}

__global__ void k_pressure_history(int *hist) {
    if (*hist < 2) *hist += 1;
}

void launch_pressure_guess(cudaStream_t s, long long n, double *pp, double *prev, int *hist) {
    k_pressure_guess<<<grid_for(n, 256 * 8), 256, 0, s>>>(n, pp, prev, hist);
    k_pressure_history<<<1, 1, 0, s>>>(hist);
    note_launches(2);
}

// ------------------------------------------------------------------------
// FMA throughput: 8 independent register chains per thread, no memory
// traffic but one store per thread.
// ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_fma_rate(T *out, const T a, const T b, const int iters) {
    T x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = (T)(threadIdx.x * 1e-3 + q);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int q = 0; q < 8; q++) x[q] = x[q] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) s += x[q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

double fma_rate(int which) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = 8 * (sms > 0 ? sms : 1), threads = 256;
    const int iters = which == 0 ? 1024 : 65536;
    void *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        if (which == 0) k_fma_rate<double><<<blocks, threads>>>((double *)out, 0.999, 1e-3, iters);
        else k_fma_rate<float><<<blocks, threads>>>((float *)out, 0.999f, 1e-3f, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    note_launches(3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return -1;
    return 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
}

}  // namespace ibm
