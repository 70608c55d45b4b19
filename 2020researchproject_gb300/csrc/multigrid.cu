// Geometric multigrid preconditioner for the pressure-Poisson rows (see
// multigrid.h for the design).  All smoothers are colour-ordered
// Gauss-Seidel with a fixed colour order, so results are bitwise
// reproducible run to run.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "krylov.h"
#include "multigrid.h"

namespace ibm {

#define GRID_STRIDE(q, n)                                                              \
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (n); \
         q += (long long)gridDim.x * blockDim.x)

static inline unsigned nblk(long long n, int t) {
    long long b = (n + t - 1) / t;
    if (b < 1) b = 1;
    if (b > 4096) b = 4096;
    return (unsigned)b;
}

// Colour of a cell: red/black by parity, plus 2 on the seam of an
// odd-length periodic axis (where red/black would put two neighbours in
// the same colour across the wrap).
__host__ __device__ inline int cell_color(int i, int j, int k, int nx, int ny, int nz, const int *per) {
    const bool seam = (per[0] && (nx & 1) && nx > 1 && i == nx - 1) || (per[1] && (ny & 1) && ny > 1 && j == ny - 1) ||
                      (per[2] && (nz & 1) && nz > 1 && k == nz - 1);
    return ((i + j + k) & 1) + (seam ? 2 : 0);
}

struct Per3 {
    int p[3];
};

// ------------------------------------------------------------ level 0 --
__global__ void __launch_bounds__(256)
k_mg0_color(const OpCtx c, const double *__restrict__ r, double *z, const int color, const Per3 per) {
    const Grid &g = c.g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    GRID_STRIDE(q, n) {
        const int k = (int)(q % g.nz);
        const int j = (int)((q / g.nz) % g.ny);
        const int i = (int)(q / ((long long)g.nz * g.ny));
        if (cell_color(i, j, k, g.nx, g.ny, g.nz, per.p) != color) continue;
        const long long P = cidx(g, i, j, k);
        const uint8_t fl = c.flag[P];
        if (fl == GHOST) continue;
        if (fl != FLUID || (c.bc.p_singular && i == 0 && j == 0 && k == 0)) {
            z[P] = r[P];
            continue;
        }
        const int I = i + 2, J = j + 2, K = k + 2;
        const long long sx = g.sx, sy = g.sy;
        const double nb = c.ax.km[I] * z[P - sx] + c.ax.kp[I] * z[P + sx] + c.ay.km[J] * z[P - sy] +
                          c.ay.kp[J] * z[P + sy] + c.az.km[K] * z[P - 1] + c.az.kp[K] * z[P + 1];
        z[P] = r[P] + c.dinv[P] * nb;
    }
}

__global__ void k_mg0_ghost(const OpCtx c, const double *__restrict__ r, const double *__restrict__ z,
                            const int *__restrict__ gcell, const int ng, double *tmp) {
    GRID_STRIDE(g, (long long)ng) {
        const int P = gcell[g];
        const int id = c.gid[P];
        double sum = 0;
        for (int e = 0; e < 8; e++) {
            const int q = c.gidx[8 * id + e];
            if (q >= 0) sum += c.gw[8 * id + e] * z[q];
        }
        const double ws = c.gwself[id];
        const double d = 1 - ws;
        tmp[g] = d >= 0.25 ? (r[P] + sum) / d : ws * z[P] + r[P] + sum;
    }
}

__global__ void k_mg0_ghost_scatter(const int *__restrict__ gcell, const int ng, const double *__restrict__ tmp,
                                    double *z) {
    GRID_STRIDE(g, (long long)ng) z[gcell[g]] = tmp[g];
}

// Outer boundary rows of the pressure operator, solved for the outer value.
__global__ void k_mg0_outer(const OpCtx c, const double *__restrict__ r, double *z, const int *__restrict__ outer,
                            const int nout) {
    GRID_STRIDE(q, (long long)nout) {
        const long long P = outer[q];
        int i, j, k, L;
        cijk(c.g, P, i, j, k);
        const int f = owner_face(c.g, i, j, k, L);
        const BCFace &F = c.bc.f[f];
        const int axis = face_axis(f);
        const long long s = axis == 0 ? c.g.sx : axis == 1 ? c.g.sy : 1;
        const long long m = P + (2 * L - 1) * (face_low(f) ? s : -s);
        switch (F.type) {
        case BCT_PRESSURE:
        case BCT_VELPERIODIC: z[P] = (r[P] - F.dir_m[L - 1] * z[m]) / F.dir_o[L - 1]; break;
        case BCT_PERIODIC: z[P] = r[P] + z[periodic_image(c.g, i, j, k)]; break;
        default: z[P] = r[P] + z[m]; break;
        }
    }
}

// Residual of the fine normalised rows, scaled to conductance form
// (Vol * coeffsum * r) and summed into the level-1 cells.
__global__ void __launch_bounds__(256)
k_mg0_restrict(const OpCtx c, const double *__restrict__ r, const double *__restrict__ z, MGLevel<double> L1) {
    const Grid &g = c.g;
    GRID_STRIDE(q, L1.n) {
        const int K = (int)(q % L1.nz);
        const int J = (int)((q / L1.nz) % L1.ny);
        const int I = (int)(q / ((long long)L1.nz * L1.ny));
        double acc = 0;
        const int i0 = L1.cx ? 2 * I : I, i1 = L1.cx ? min(2 * I + 1, g.nx - 1) : I;
        const int j0 = L1.cy ? 2 * J : J, j1 = L1.cy ? min(2 * J + 1, g.ny - 1) : J;
        const int k0 = L1.cz ? 2 * K : K, k1 = L1.cz ? min(2 * K + 1, g.nz - 1) : K;
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    const long long P = cidx(g, i, j, k);
                    if (c.flag[P] != FLUID || (c.bc.p_singular && i == 0 && j == 0 && k == 0)) continue;
                    const int Ii = i + 2, Jj = j + 2, Kk = k + 2;
                    const double kW = c.ax.km[Ii], kE = c.ax.kp[Ii], kS = c.ay.km[Jj], kN = c.ay.kp[Jj];
                    const double kD = c.az.km[Kk], kU = c.az.kp[Kk];
                    const double nb = kW * z[P - g.sx] + kE * z[P + g.sx] + kS * z[P - g.sy] + kN * z[P + g.sy] +
                                      kD * z[P - 1] + kU * z[P + 1];
                    const double res = r[P] - (z[P] - c.dinv[P] * nb);
                    const double vol = c.ax.d[Ii] * c.ay.d[Jj] * c.az.d[Kk];
                    acc += vol * (kN + kE + kS + kW + kD + kU) * res;
                }
        L1.R[q] = acc;
    }
}

__global__ void __launch_bounds__(256)
k_mg0_prolong(const OpCtx c, double *z, const MGLevel<double> L1) {
    const Grid &g = c.g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    GRID_STRIDE(q, n) {
        const int k = (int)(q % g.nz);
        const int j = (int)((q / g.nz) % g.ny);
        const int i = (int)(q / ((long long)g.nz * g.ny));
        const long long P = cidx(g, i, j, k);
        const uint8_t fl = c.flag[P];
        if (fl != FLUID && fl != GHOST) continue;
        if (c.bc.p_singular && i == 0 && j == 0 && k == 0) continue;
        const int I = L1.cx ? i >> 1 : i, J = L1.cy ? j >> 1 : j, K = L1.cz ? k >> 1 : k;
        z[P] += L1.Z[((long long)I * L1.ny + J) * L1.nz + K];
    }
}

// ------------------------------------------------------ level building --
// Level 1 from the fine grid: conductances Vol*k of fluid-fluid faces,
// pressure-Dirichlet boundary conductances, periodic wraps.
__global__ void k_mg_build1(const OpCtx c, MGLevel<double> L, double *Gx, double *Gy, double *Gz, const Per3 per) {
    const Grid &g = c.g;
    GRID_STRIDE(q, L.n) {
        const int K = (int)(q % L.nz);
        const int J = (int)((q / L.nz) % L.ny);
        const int I = (int)(q / ((long long)L.nz * L.ny));
        const int i0 = L.cx ? 2 * I : I, i1 = L.cx ? min(2 * I + 1, g.nx - 1) : I;
        const int j0 = L.cy ? 2 * J : J, j1 = L.cy ? min(2 * J + 1, g.ny - 1) : J;
        const int k0 = L.cz ? 2 * K : K, k1 = L.cz ? min(2 * K + 1, g.nz - 1) : K;
        auto active = [&](int i, int j, int k) {
            return c.flag[cidx(g, i, j, k)] == FLUID && !(c.bc.p_singular && i == 0 && j == 0 && k == 0);
        };
        auto vol = [&](int i, int j, int k) { return c.ax.d[i + 2] * c.ay.d[j + 2] * c.az.d[k + 2]; };
        double tx = 0, ty = 0, tz = 0, gx = 0, gy = 0, gz = 0;
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    if (!active(i, j, k)) continue;
                    const double v = vol(i, j, k);
                    // Low x face of the coarse cell: fine faces at i == i0.
                    if (i == i0) {
                        if (i > 0) { if (active(i - 1, j, k)) tx += v * c.ax.km[i + 2]; }
                        else if (per.p[0] && g.nx > 1) { if (active(g.nx - 1, j, k)) tx += v * c.ax.km[2]; }
                    }
                    if (j == j0) {
                        if (j > 0) { if (active(i, j - 1, k)) ty += v * c.ay.km[j + 2]; }
                        else if (per.p[1] && g.ny > 1) { if (active(i, g.ny - 1, k)) ty += v * c.ay.km[2]; }
                    }
                    if (k == k0) {
                        if (k > 0) { if (active(i, j, k - 1)) tz += v * c.az.km[k + 2]; }
                        else if (per.p[2] && g.nz > 1) { if (active(i, j, g.nz - 1)) tz += v * c.az.km[2]; }
                    }
                    // Pressure-Dirichlet boundaries (homogeneous fold of the
                    // interpolation rows).
                    const BCFace &W = c.bc.f[F_W], &E = c.bc.f[F_E], &S = c.bc.f[F_S], &N = c.bc.f[F_N];
                    const BCFace &D = c.bc.f[F_D], &U = c.bc.f[F_U];
                    auto dir = [](int t) { return t == BCT_PRESSURE || t == BCT_VELPERIODIC; };
                    if (i == 0 && dir(W.type)) gx += v * c.ax.km[2] * (1 + W.dir_m[0] / W.dir_o[0]);
                    if (i == g.nx - 1 && dir(E.type)) gx += v * c.ax.kp[g.nx + 1] * (1 + E.dir_m[0] / E.dir_o[0]);
                    if (j == 0 && dir(S.type)) gy += v * c.ay.km[2] * (1 + S.dir_m[0] / S.dir_o[0]);
                    if (j == g.ny - 1 && dir(N.type)) gy += v * c.ay.kp[g.ny + 1] * (1 + N.dir_m[0] / N.dir_o[0]);
                    if (k == 0 && dir(D.type)) gz += v * c.az.km[2] * (1 + D.dir_m[0] / D.dir_o[0]);
                    if (k == g.nz - 1 && dir(U.type)) gz += v * c.az.kp[g.nz + 1] * (1 + U.dir_m[0] / U.dir_o[0]);
                }
        const double fx = L.cx ? 0.5 : 1.0, fy = L.cy ? 0.5 : 1.0, fz = L.cz ? 0.5 : 1.0;
        L.Tx[q] = (I == 0 && L.nx == 1) ? 0.0 : fx * tx;
        L.Ty[q] = (J == 0 && L.ny == 1) ? 0.0 : fy * ty;
        L.Tz[q] = (K == 0 && L.nz == 1) ? 0.0 : fz * tz;
        Gx[q] = fx * gx;
        Gy[q] = fy * gy;
        Gz[q] = fz * gz;
    }
}

// Coarse level c from level f.
__global__ void k_mg_buildc(const MGLevel<double> F, const double *__restrict__ fGx, const double *__restrict__ fGy,
                            const double *__restrict__ fGz, MGLevel<double> C, double *Gx, double *Gy, double *Gz) {
    GRID_STRIDE(q, C.n) {
        const int K = (int)(q % C.nz);
        const int J = (int)((q / C.nz) % C.ny);
        const int I = (int)(q / ((long long)C.nz * C.ny));
        const int i0 = C.cx ? 2 * I : I, i1 = C.cx ? min(2 * I + 1, F.nx - 1) : I;
        const int j0 = C.cy ? 2 * J : J, j1 = C.cy ? min(2 * J + 1, F.ny - 1) : J;
        const int k0 = C.cz ? 2 * K : K, k1 = C.cz ? min(2 * K + 1, F.nz - 1) : K;
        double tx = 0, ty = 0, tz = 0, gx = 0, gy = 0, gz = 0;
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    const long long f = ((long long)i * F.ny + j) * F.nz + k;
                    if (i == i0) tx += F.Tx[f];
                    if (j == j0) ty += F.Ty[f];
                    if (k == k0) tz += F.Tz[f];
                    gx += fGx[f];
                    gy += fGy[f];
                    gz += fGz[f];
                }
        const double fx = C.cx ? 0.5 : 1.0, fy = C.cy ? 0.5 : 1.0, fz = C.cz ? 0.5 : 1.0;
        C.Tx[q] = (I == 0 && C.nx == 1) ? 0.0 : fx * tx;
        C.Ty[q] = (J == 0 && C.ny == 1) ? 0.0 : fy * ty;
        C.Tz[q] = (K == 0 && C.nz == 1) ? 0.0 : fz * tz;
        Gx[q] = fx * gx;
        Gy[q] = fy * gy;
        Gz[q] = fz * gz;
    }
}

__host__ __device__ inline long long lidx(const MGLevel<double> &L, int I, int J, int K) {
    return ((long long)I * L.ny + J) * L.nz + K;
}

// Couplings of a coarse cell: calls fn(neighbour index, conductance).
template <typename Fn>
__device__ inline void for_neighbours(const MGLevel<double> &L, int I, int J, int K, const int *per, Fn fn) {
    const long long q = lidx(L, I, J, K);
    if (I > 0) fn(q - (long long)L.ny * L.nz, L.Tx[q]);
    else if (per[0] && L.nx > 1) fn(lidx(L, L.nx - 1, J, K), L.Tx[q]);
    if (I < L.nx - 1) fn(q + (long long)L.ny * L.nz, L.Tx[q + (long long)L.ny * L.nz]);
    else if (per[0] && L.nx > 1) fn(lidx(L, 0, J, K), L.Tx[lidx(L, 0, J, K)]);
    if (J > 0) fn(q - L.nz, L.Ty[q]);
    else if (per[1] && L.ny > 1) fn(lidx(L, I, L.ny - 1, K), L.Ty[q]);
    if (J < L.ny - 1) fn(q + L.nz, L.Ty[q + L.nz]);
    else if (per[1] && L.ny > 1) fn(lidx(L, I, 0, K), L.Ty[lidx(L, I, 0, K)]);
    if (K > 0) fn(q - 1, L.Tz[q]);
    else if (per[2] && L.nz > 1) fn(lidx(L, I, J, L.nz - 1), L.Tz[q]);
    if (K < L.nz - 1) fn(q + 1, L.Tz[q + 1]);
    else if (per[2] && L.nz > 1) fn(lidx(L, I, J, 0), L.Tz[lidx(L, I, J, 0)]);
}

__global__ void k_mg_diag(MGLevel<double> L, const double *__restrict__ Gx, const double *__restrict__ Gy,
                          const double *__restrict__ Gz, const Per3 per) {
    GRID_STRIDE(q, L.n) {
        const int K = (int)(q % L.nz);
        const int J = (int)((q / L.nz) % L.ny);
        const int I = (int)(q / ((long long)L.nz * L.ny));
        double d = Gx[q] + Gy[q] + Gz[q];
        for_neighbours(L, I, J, K, per.p, [&](long long, double t) { d += t; });
        L.diag[q] = d;
    }
}

// ----------------------------------------------------- coarse kernels --
__device__ inline void coarse_relax(const MGLevel<double> &L, long long q, const int *per) {
    const int K = (int)(q % L.nz);
    const int J = (int)((q / L.nz) % L.ny);
    const int I = (int)(q / ((long long)L.nz * L.ny));
    const double d = L.diag[q];
    if (d == 0.0) {
        L.Z[q] = 0.0;
        return;
    }
    double s = L.R[q];
    for_neighbours(L, I, J, K, per, [&](long long m, double t) { s += t * L.Z[m]; });
    L.Z[q] = s / d;
}

__device__ inline double coarse_residual(const MGLevel<double> &L, long long q, const int *per) {
    const int K = (int)(q % L.nz);
    const int J = (int)((q / L.nz) % L.ny);
    const int I = (int)(q / ((long long)L.nz * L.ny));
    if (L.diag[q] == 0.0) return 0.0;
    double s = L.R[q] - L.diag[q] * L.Z[q];
    for_neighbours(L, I, J, K, per, [&](long long m, double t) { s += t * L.Z[m]; });
    return s;
}

__device__ inline int lcolor(const MGLevel<double> &L, long long q, const int *per) {
    const int K = (int)(q % L.nz);
    const int J = (int)((q / L.nz) % L.ny);
    const int I = (int)(q / ((long long)L.nz * L.ny));
    return cell_color(I, J, K, L.nx, L.ny, L.nz, per);
}

__global__ void k_mgc_color(MGLevel<double> L, const int color, const Per3 per) {
    GRID_STRIDE(q, L.n) {
        if (lcolor(L, q, per.p) == color) coarse_relax(L, q, per.p);
    }
}

__global__ void k_mgc_restrict(const MGLevel<double> F, MGLevel<double> C, const Per3 per) {
    GRID_STRIDE(q, C.n) {
        const int K = (int)(q % C.nz);
        const int J = (int)((q / C.nz) % C.ny);
        const int I = (int)(q / ((long long)C.nz * C.ny));
        const int i0 = C.cx ? 2 * I : I, i1 = C.cx ? min(2 * I + 1, F.nx - 1) : I;
        const int j0 = C.cy ? 2 * J : J, j1 = C.cy ? min(2 * J + 1, F.ny - 1) : J;
        const int k0 = C.cz ? 2 * K : K, k1 = C.cz ? min(2 * K + 1, F.nz - 1) : K;
        double acc = 0;
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) acc += coarse_residual(F, lidx(F, i, j, k), per.p);
        C.R[q] = acc;
    }
}

__global__ void k_mgc_prolong(const MGLevel<double> C, MGLevel<double> F) {
    GRID_STRIDE(q, F.n) {
        if (F.diag[q] == 0.0) continue;
        const int K = (int)(q % F.nz);
        const int J = (int)((q / F.nz) % F.ny);
        const int I = (int)(q / ((long long)F.nz * F.ny));
        F.Z[q] += C.Z[lidx(C, C.cx ? I >> 1 : I, C.cy ? J >> 1 : J, C.cz ? K >> 1 : K)];
    }
}

__global__ void k_zero(double *a, long long n) { GRID_STRIDE(q, n) a[q] = 0.0; }

// Whole V-cycle over levels [first, nlev) inside one thread block.  R of
// level `first` is set; Z of level `first` is produced.
__global__ void __launch_bounds__(1024)
k_mg_tail(const MGLevel<double> *__restrict__ lv, const int first, const int nlev, const int nu1, const int nu2,
          const int csweeps, const Per3 per) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int l = first; l < nlev; l++) {
        const MGLevel<double> L = lv[l];
        for (long long q = tid; q < L.n; q += nt) L.Z[q] = 0.0;
        __syncthreads();
        const int sweeps = (l == nlev - 1) ? csweeps : nu1;
        for (int s = 0; s < sweeps; s++)
            for (int col = 0; col < 4; col++) {
                for (long long q = tid; q < L.n; q += nt)
                    if (lcolor(L, q, per.p) == col) coarse_relax(L, q, per.p);
                __syncthreads();
            }
        if (l < nlev - 1) {
            const MGLevel<double> C = lv[l + 1];
            for (long long q = tid; q < C.n; q += nt) {
                const int K = (int)(q % C.nz);
                const int J = (int)((q / C.nz) % C.ny);
                const int I = (int)(q / ((long long)C.nz * C.ny));
                const int i0 = C.cx ? 2 * I : I, i1 = C.cx ? min(2 * I + 1, L.nx - 1) : I;
                const int j0 = C.cy ? 2 * J : J, j1 = C.cy ? min(2 * J + 1, L.ny - 1) : J;
                const int k0 = C.cz ? 2 * K : K, k1 = C.cz ? min(2 * K + 1, L.nz - 1) : K;
                double acc = 0;
                for (int i = i0; i <= i1; i++)
                    for (int j = j0; j <= j1; j++)
                        for (int k = k0; k <= k1; k++) acc += coarse_residual(L, lidx(L, i, j, k), per.p);
                C.R[q] = acc;
            }
            __syncthreads();
        }
    }
    for (int l = nlev - 2; l >= first; l--) {
        const MGLevel<double> L = lv[l], C = lv[l + 1];
        for (long long q = tid; q < L.n; q += nt) {
            if (L.diag[q] == 0.0) continue;
            const int K = (int)(q % L.nz);
            const int J = (int)((q / L.nz) % L.ny);
            const int I = (int)(q / ((long long)L.nz * L.ny));
            L.Z[q] += C.Z[lidx(C, C.cx ? I >> 1 : I, C.cy ? J >> 1 : J, C.cz ? K >> 1 : K)];
        }
        __syncthreads();
        for (int s = 0; s < nu2; s++)
            for (int col = 0; col < 4; col++) {
                for (long long q = tid; q < L.n; q += nt)
                    if (lcolor(L, q, per.p) == col) coarse_relax(L, q, per.p);
                __syncthreads();
            }
    }
}

// ------------------------------------------------------------- host --
GMG::~GMG() {
    for (void *p : allocs_) cudaFree(p);
}

int GMG::setup(cudaStream_t s, const OpCtx &ctx, const int *ghost_cell, int nghost, double, double,
               const GMGConfig &cfg) {
    ctx_ = ctx;
    cfg_ = cfg;
    ghost_cell_ = ghost_cell;
    nghost_ = nghost;
    const Grid &g = ctx.g;
    per_[0] = ctx.bc.f[F_W].type == BCT_PERIODIC;
    per_[1] = ctx.bc.f[F_S].type == BCT_PERIODIC;
    per_[2] = ctx.bc.f[F_D].type == BCT_PERIODIC;
    auto dalloc = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        cudaMemsetAsync(p, 0, bytes, s);
        allocs_.push_back(p);
        return p;
    };
    if (nghost > 0) ghost_tmp_ = (double *)dalloc(sizeof(double) * nghost);
    // Outer-cell list.
    std::vector<int> outer;
    for (int i = -2; i < g.nx + 2; i++)
        for (int j = -2; j < g.ny + 2; j++)
            for (int k = -2; k < g.nz + 2; k++) {
                int L;
                if (owner_face(g, i, j, k, L) >= 0) outer.push_back((int)cidx(g, i, j, k));
            }
    nouter_ = (int)outer.size();
    outer_ = (int *)dalloc(sizeof(int) * std::max(1, nouter_));
    cudaMemcpyAsync(outer_, outer.data(), sizeof(int) * nouter_, cudaMemcpyHostToDevice, s);

    // Level dimensions.
    int nx = g.nx, ny = g.ny, nz = g.nz;
    std::vector<double *> G;  // Gx,Gy,Gz per level
    Per3 per{{per_[0], per_[1], per_[2]}};
    while (true) {
        const bool cx = nx >= 2, cy = ny >= 2, cz = nz >= 2;
        if (!cx && !cy && !cz) break;
        if ((long long)nx * ny * nz <= 64 && !levels_.empty()) break;
        MGLevel<double> L{};
        L.cx = cx; L.cy = cy; L.cz = cz;
        L.nx = cx ? (nx + 1) / 2 : nx;
        L.ny = cy ? (ny + 1) / 2 : ny;
        L.nz = cz ? (nz + 1) / 2 : nz;
        L.n = (long long)L.nx * L.ny * L.nz;
        const size_t b = sizeof(double) * L.n;
        L.Tx = (double *)dalloc(b); L.Ty = (double *)dalloc(b); L.Tz = (double *)dalloc(b);
        L.diag = (double *)dalloc(b); L.R = (double *)dalloc(b); L.Z = (double *)dalloc(b);
        if (!L.Tx || !L.Ty || !L.Tz || !L.diag || !L.R || !L.Z) return -1;
        double *gx = (double *)dalloc(b), *gy = (double *)dalloc(b), *gz = (double *)dalloc(b);
        if (levels_.empty()) {
            k_mg_build1<<<nblk(L.n, 128), 128, 0, s>>>(ctx, L, gx, gy, gz, per);
        } else {
            const MGLevel<double> &F = levels_.back();
            double **fg = &G[G.size() - 3];
            k_mg_buildc<<<nblk(L.n, 128), 128, 0, s>>>(F, fg[0], fg[1], fg[2], L, gx, gy, gz);
        }
        k_mg_diag<<<nblk(L.n, 128), 128, 0, s>>>(L, gx, gy, gz, per);
        G.push_back(gx); G.push_back(gy); G.push_back(gz);
        levels_.push_back(L);
        nx = L.nx; ny = L.ny; nz = L.nz;
        if (L.n <= 64) break;
    }
    tail_ = (int)levels_.size();
    for (int l = 0; l < (int)levels_.size(); l++)
        if (levels_[l].n <= cfg_.tail_cells) { tail_ = l; break; }
    if (!levels_.empty()) {
        dlevels_ = (MGLevel<double> *)dalloc(sizeof(MGLevel<double>) * levels_.size());
        cudaMemcpyAsync(dlevels_, levels_.data(), sizeof(MGLevel<double>) * levels_.size(), cudaMemcpyHostToDevice, s);
    }
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -1;
}

void GMG::smooth0(cudaStream_t s, const double *r, double *z, int sweeps) {
    const Grid &g = ctx_.g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    Per3 per{{per_[0], per_[1], per_[2]}};
    const bool seam = (per_[0] && (g.nx & 1)) || (per_[1] && (g.ny & 1)) || (per_[2] && (g.nz & 1));
    for (int it = 0; it < sweeps; it++) {
        for (int col = 0; col < (seam ? 4 : 2); col++)
            k_mg0_color<<<nblk(n, 256), 256, 0, s>>>(ctx_, r, z, col, per);
            note_launches(1);
        if (nghost_ > 0) {
            k_mg0_ghost<<<nblk(nghost_, 128), 128, 0, s>>>(ctx_, r, z, ghost_cell_, nghost_, ghost_tmp_);
            note_launches(1);
            k_mg0_ghost_scatter<<<nblk(nghost_, 128), 128, 0, s>>>(ghost_cell_, nghost_, ghost_tmp_, z);
            note_launches(1);
        }
        k_mg0_outer<<<nblk(nouter_, 256), 256, 0, s>>>(ctx_, r, z, outer_, nouter_);
        note_launches(1);
    }
}

void GMG::apply(cudaStream_t s, const double *r, double *z) {
    const Grid &g = ctx_.g;
    cudaMemsetAsync(z, 0, sizeof(double) * g.ncell, s);
    if (levels_.empty()) {
        smooth0(s, r, z, cfg_.nu_pre + cfg_.nu_post + 4);
        return;
    }
    Per3 per{{per_[0], per_[1], per_[2]}};
    smooth0(s, r, z, cfg_.nu_pre);
    k_mg0_restrict<<<nblk(levels_[0].n, 256), 256, 0, s>>>(ctx_, r, z, levels_[0]);
    note_launches(1);
    const int nl = (int)levels_.size();
    for (int l = 0; l < tail_; l++) {
        MGLevel<double> &L = levels_[l];
        cudaMemsetAsync(L.Z, 0, sizeof(double) * L.n, s);
        for (int it = 0; it < cfg_.nu_pre; it++)
            for (int col = 0; col < 4; col++) k_mgc_color<<<nblk(L.n, 256), 256, 0, s>>>(L, col, per);
        k_mgc_restrict<<<nblk(levels_[l + 1].n, 256), 256, 0, s>>>(L, levels_[l + 1], per);
        note_launches(1);
    }
    k_mg_tail<<<1, 1024, 0, s>>>(dlevels_, tail_, nl, cfg_.nu_pre, cfg_.nu_post, cfg_.coarse_sweeps, per);
    note_launches(1);
    for (int l = tail_ - 1; l >= 0; l--) {
        MGLevel<double> &L = levels_[l];
        k_mgc_prolong<<<nblk(L.n, 256), 256, 0, s>>>(levels_[l + 1], L);
        note_launches(1);
        for (int it = 0; it < cfg_.nu_post; it++)
            for (int col = 0; col < 4; col++) k_mgc_color<<<nblk(L.n, 256), 256, 0, s>>>(L, col, per);
    }
    k_mg0_prolong<<<nblk((long long)g.nx * g.ny * g.nz, 256), 256, 0, s>>>(ctx_, z, levels_[0]);
    note_launches(1);
    smooth0(s, r, z, cfg_.nu_post);
}

}  // namespace ibm
