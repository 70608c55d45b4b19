// Geometric multigrid preconditioner for the pressure-Poisson rows (see
// multigrid.h for the design), instantiated in FP64 and FP32.
#include <algorithm>
#include <cmath>
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

// The first colour pass of a coarse level on Z = 0, applied to one cell by
// the restriction that has just computed its R (saves the level its
// separate init launch): colour-0 cells take R / diag, the others 0.
template <typename T>
__device__ __forceinline__ void restrict_init(const MGLevel<T> &L, long long q, int I, int J, int K, T R,
                                              const Per3 &per) {
    L.Z[q] = cell_color(I, J, K, L.nx, L.ny, L.nz, per.p) == 0 ? R * L.idiag[q] : (T)0;
}

// Every V-cycle kernel returns at once while *gate (when given) is not
// KS_RUN: the solve it serves has converged.
#define MG_GATE(gate)                       \
    pdl_enter();                            \
    if ((gate) && *(gate) != KS_RUN) return;

template <typename T>
__host__ __device__ inline long long lidx(const MGLevel<T> &L, int I, int J, int K) {
    return ((long long)I * L.ny + J) * L.nz + K;
}

// Whether a coarse diagonal marks an active cell, as an integer test on
// its bits (inactive cells hold exactly +0), off the FP64 pipe.
__device__ __forceinline__ bool active_bits(double d) { return __double_as_longlong(d) != 0; }
__device__ __forceinline__ bool active_bits(float d) { return __float_as_int(d) != 0; }

// Trilinear blend of the 8 coarse values v[a][b][c] (act: 1 active, 0
// inactive or absent) with weights wxs[a] wys[b] wzs[c].  With all eight
// active the weights sum to one: nested blend, no division (the common
// case; FP64 division is slow on this part).  Otherwise the weights of the
// active cells are renormalised.
template <typename T>
__device__ __forceinline__ T trilinear(const T (&v)[2][2][2], const bool (&act)[2][2][2], const T (&wxs)[2],
                                       const T (&wys)[2], const T (&wzs)[2]) {
    bool all = true;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
            for (int c = 0; c < 2; c++) all = all && act[a][b][c];
    if (all) {
        const T y0 = wys[0] * (wzs[0] * v[0][0][0] + wzs[1] * v[0][0][1]) + wys[1] * (wzs[0] * v[0][1][0] + wzs[1] * v[0][1][1]);
        const T y1 = wys[0] * (wzs[0] * v[1][0][0] + wzs[1] * v[1][0][1]) + wys[1] * (wzs[0] * v[1][1][0] + wzs[1] * v[1][1][1]);
        return wxs[0] * y0 + wxs[1] * y1;
    }
    T acc = 0, ws = 0;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (!act[a][b][c]) continue;
                const T w = wxs[a] * wys[b] * wzs[c];
                acc += w * v[a][b][c];
                ws += w;
            }
    return ws > (T)0 ? acc / ws : (T)0;
}

// Trilinear correction of fine cell (i, j, k) from coarse level C, over
// active coarse cells only.
template <typename T>
__device__ inline T prolong_value(const MGLevel<T> &C, int i, int j, int k) {
    const int I = C.pa[0][i], J = C.pa[1][j], K = C.pa[2][k];
    const int xs[2] = {I, C.po[0][i]}, ys[2] = {J, C.po[1][j]}, zs[2] = {K, C.po[2][k]};
    const T wx = C.pw[0][i], wy = C.pw[1][j], wz = C.pw[2][k];
    const T wxs[2] = {wx, (T)1 - wx}, wys[2] = {wy, (T)1 - wy}, wzs[2] = {wz, (T)1 - wz};
    T v[2][2][2];
    bool act[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
            for (int c = 0; c < 2; c++) {
                v[a][b][c] = 0;
                act[a][b][c] = false;
                if (xs[a] < 0 || ys[b] < 0 || zs[c] < 0) continue;
                const long long q = lidx(C, xs[a], ys[b], zs[c]);
                v[a][b][c] = C.Z[q];
                act[a][b][c] = active_bits(C.diag[q]);
            }
    return trilinear(v, act, wxs, wys, wzs);
}

// ------------------------------------------------------------ level 0 --
// One colour pass of Gauss-Seidel on the fine rows.  Without a periodic
// seam the colours are red/black and each thread takes the cell of its
// colour in one (k, k+1) pair of MG0_PLANES consecutive planes, loading
// all of them before any update (no cell of the pass is a neighbour of
// another: the updated cells share one colour): grid (ceil(nz/64),
// ceil(ny/8), ceil(nx/MG0_PLANES)) of 32 x 8 threads, no index division.
// With a seam (4 colours) each thread takes one cell per plane and tests
// its colour.  init = 1 (colour 0 only, z undefined on entry) applies the
// pass to z = 0: colour-0 cells get r, every other padded cell 0 (the
// sweep over all cells then covers the whole array).
constexpr int MG0_PLANES = 2;

template <typename T, bool SPLIT>
__global__ void __launch_bounds__(256)
k_mg0_color(const OpT<T> c, const FineRows<T> fr, T *__restrict__ z, const int color, const int pairs,
            const Per3 per, const T omega, const int *gate) {
    MG_GATE(gate);
    const Grid &g = c.g;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i0 = blockIdx.z * MG0_PLANES;
    const long long sx = g.sx, sy = g.sy;
    // Branch-free: every load of every plane is issued before any update
    // (cells off the grid or of the other colour read cell (0,0,0) and are
    // masked at the store), so the loads of all planes overlap.
    long long Ps[MG0_PLANES];
    T val[MG0_PLANES];
    bool upd[MG0_PLANES];
    const int jj = min(j, g.ny - 1);
    const T kmy = c.km[1][jj + 2], kpy = c.kp[1][jj + 2];
#pragma unroll
    for (int p = 0; p < MG0_PLANES; p++) {
        const int i = min(i0 + p, g.nx - 1);
        int k;
        bool ok = j < g.ny && i0 + p < g.nx;
        if (pairs) {
            k = 2 * (blockIdx.x * 32 + threadIdx.x) + ((i + jj + color) & 1);
        } else {
            k = blockIdx.x * 32 + threadIdx.x;
            ok = ok && k < g.nz && cell_color(i, jj, k, g.nx, g.ny, g.nz, per.p) == color;
        }
        ok = ok && k < g.nz;
        k = min(k, g.nz - 1);
        const long long P = cidx(g, i, jj, k), q = SPLIT ? fr.split_index(i, jj, k) : P;
        const uint8_t fl = fr.flag[q];
        const T rv = fr.r[q], dv = fr.dinv[q];
        const T zw = z[P - sx], ze = z[P + sx], zs = z[P - sy], zn = z[P + sy], zd = z[P - 1], zu = z[P + 1];
        const T zc = z[P];
        const int I = i + 2, K = k + 2;
        const T nb = c.km[0][I] * zw + c.kp[0][I] * ze + kmy * zs + kpy * zn + c.km[2][K] * zd + c.kp[2][K] * zu;
        const bool fluid = fl == FLUID && !(c.p_singular && P == c.pinned);
        const T gs = rv + dv * nb;
        val[p] = fluid ? (omega == (T)1 ? gs : zc + omega * (gs - zc)) : rv;
        upd[p] = ok && fl != GHOST;
        Ps[p] = P;
    }
#pragma unroll
    for (int p = 0; p < MG0_PLANES; p++)
        if (upd[p]) z[Ps[p]] = val[p];
}

// The first sweep's two colour passes on z = 0 in one launch (red/black
// without a periodic seam, where no ghost stencil reaches an outer cell):
// each thread takes the (k, k+1) pair of each of its planes.  The colour-0
// cell takes its value after the first pass (r, or 0 on a ghost row), the
// colour-1 cell the Gauss-Seidel update from its neighbours' values after
// that pass (r of interior non-ghost neighbours, 0 elsewhere; 0 on a ghost
// row): the same arithmetic as k_mg0_init3 followed by the colour-1 pass of
// k_mg0_color, one launch fewer per V-cycle.  Outer cells are left as they
// are: nothing reads them before the sweep's outer rows set them.
template <typename T, bool SPLIT>
__global__ void __launch_bounds__(256)
k_mg0_first(const OpT<T> c, const FineRows<T> fr, T *__restrict__ z, const T omega, const int *gate) {
    MG_GATE(gate);
    const Grid &g = c.g;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i0 = blockIdx.z * MG0_PLANES;
    const long long sx = g.sx, sy = g.sy;
    const int jj = min(j, g.ny - 1);
    const T kmy = c.km[1][jj + 2], kpy = c.kp[1][jj + 2];
    long long P0s[MG0_PLANES], P1s[MG0_PLANES];
    T v0[MG0_PLANES], v1[MG0_PLANES];
    bool ok0[MG0_PLANES], ok1[MG0_PLANES];
    // A colour-0 cell's value after the first pass (a neighbour of the
    // colour-1 cell; its padded index Q and layout index always exist).
    auto first = [&](int a, int b, int e, long long Q) -> T {
        const bool in = a >= 0 && a < g.nx && b >= 0 && b < g.ny && e >= 0 && e < g.nz;
        const T rn = fr.r[SPLIT ? fr.split_index(a, b, e) : Q];
        return in && c.flag[Q] != GHOST ? rn : (T)0;
    };
#pragma unroll
    for (int p = 0; p < MG0_PLANES; p++) {
        const int i = min(i0 + p, g.nx - 1);
        const bool okp = j < g.ny && i0 + p < g.nx;
        const int kb = 2 * (blockIdx.x * 32 + threadIdx.x);
        const int k0 = kb + ((i + jj) & 1), k1 = kb + ((i + jj + 1) & 1);
        ok0[p] = okp && k0 < g.nz;
        ok1[p] = okp && k1 < g.nz;
        const int k0c = min(k0, g.nz - 1), k1c = min(k1, g.nz - 1);
        const long long P0 = cidx(g, i, jj, k0c), P1 = cidx(g, i, jj, k1c);
        const long long q0 = SPLIT ? fr.split_index(i, jj, k0c) : P0, q1 = SPLIT ? fr.split_index(i, jj, k1c) : P1;
        v0[p] = c.flag[P0] != GHOST ? fr.r[q0] : (T)0;
        const uint8_t fl = fr.flag[q1];
        const T rv = fr.r[q1], dv = fr.dinv[q1];
        const T zw = first(i - 1, jj, k1c, P1 - sx), ze = first(i + 1, jj, k1c, P1 + sx);
        const T zs = first(i, jj - 1, k1c, P1 - sy), zn = first(i, jj + 1, k1c, P1 + sy);
        const T zd = first(i, jj, k1c - 1, P1 - 1), zu = first(i, jj, k1c + 1, P1 + 1);
        const T zc = 0;
        const int I = i + 2, K = k1c + 2;
        const T nb = c.km[0][I] * zw + c.kp[0][I] * ze + kmy * zs + kpy * zn + c.km[2][K] * zd + c.kp[2][K] * zu;
        const bool fluid = fl == FLUID && !(c.p_singular && P1 == c.pinned);
        const T gs = rv + dv * nb;
        v1[p] = fl == GHOST ? (T)0 : fluid ? (omega == (T)1 ? gs : zc + omega * (gs - zc)) : rv;
        P0s[p] = P0;
        P1s[p] = P1;
    }
#pragma unroll
    for (int p = 0; p < MG0_PLANES; p++) {
        if (ok0[p]) z[P0s[p]] = v0[p];
        if (ok1[p]) z[P1s[p]] = v1[p];
    }
}

// The first colour pass of a V-cycle on z = 0, as one pass over the whole
// padded array: colour-0 interior rows take r (r + dinv * 0, and r for
// solid and pinned rows), every other cell 0.  A 3-D launch over the
// padded box (threads along k, no index division), each thread on
// MG0_IPLANES consecutive planes: grid (ceil((nz+4)/32), ceil((ny+4)/8),
// ceil((nx+4)/MG0_IPLANES)).
constexpr int MG0_IPLANES = 4;

template <typename T, bool SPLIT>
__global__ void __launch_bounds__(256)
k_mg0_init3(const OpT<T> c, const FineRows<T> fr, T *__restrict__ z, const Per3 per, const int *gate) {
    MG_GATE(gate);
    const Grid &g = c.g;
    const int K = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y;
    if (K >= g.nz + 4 || J >= g.ny + 4) return;
    const int j = J - 2, k = K - 2;
    const bool jk = j >= 0 && j < g.ny && k >= 0 && k < g.nz;
#pragma unroll
    for (int q = 0; q < MG0_IPLANES; q++) {
        const int I = blockIdx.z * MG0_IPLANES + q, i = I - 2;
        if (I >= g.nx + 4) break;
        const long long P = (long long)I * g.sx + (long long)J * g.sy + K;
        T v = 0;
        if (jk && i >= 0 && i < g.nx && cell_color(i, j, k, g.nx, g.ny, g.nz, per.p) == 0 && c.flag[P] != GHOST)
            v = fr.r[SPLIT ? fr.split_index(i, j, k) : P];
        z[P] = v;
    }
}

// A padded natural array into the colour-split layout of FineRows (at
// set-up: 1/coeffsum and the flags).  3-D launch over the padded box: grid
// (ceil(NZ/32), ceil(NY/8), NX) of 32 x 8 threads.
template <typename D, typename S>
__global__ void __launch_bounds__(256)
k_to_split(const S *__restrict__ a, D *__restrict__ b, const int NY, const int NZ, const int NZH, const long long H,
           const int *gate) {
    MG_GATE(gate);
    const int K = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y, I = blockIdx.z;
    if (K >= NZ || J >= NY) return;
    const long long row = (long long)I * NY + J;
    b[((I + J + K) & 1) * H + row * NZH + (K >> 1)] = (D)a[row * NZ + K];
}

// The right-hand side of an FP32 cycle (FP64, double-float (its high
// word), or FP32 from an FP32 solve) into the colour-split layout: each thread takes one (K, K+1) pair of a
// padded row on MG0_NPLANES consecutive planes; its two values go to the
// two colour halves at the same position (coalesced reads and writes), an
// FP64 value rounded on the integer pipe (d2f_int: FP64 <-> FP32
// conversions issue at the FP64 rate on this part).  Grid (ceil(NZH/32),
// ceil(NY/8), ceil(NX/MG0_NPLANES)).
constexpr int MG0_NPLANES = 4;

__device__ __forceinline__ float to32(double x) { return d2f_int(x); }
__device__ __forceinline__ float to32(float x) { return x; }
__device__ __forceinline__ float to32(dfloat x) { return x.hi; }

template <typename S>
__global__ void __launch_bounds__(256)
k_narrow_split(const S *__restrict__ r, float *__restrict__ rs, const int NX, const int NY, const int NZ,
               const int NZH, const long long H, const int *gate) {
    MG_GATE(gate);
    const int kp = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y;
    if (kp >= NZH || J >= NY) return;
    const int K = 2 * kp;
    const bool two = K + 1 < NZ;
    const int I0 = blockIdx.z * MG0_NPLANES;
#pragma unroll
    for (int p = 0; p < MG0_NPLANES; p++) {
        const int I = I0 + p;
        if (I >= NX) break;
        const long long row = (long long)I * NY + J;
        const S a = r[row * NZ + K];
        const S b = two ? r[row * NZ + K + 1] : (S)0;
        const long long c = (I + J) & 1;   // colour of the even K
        rs[c * H + row * NZH + kp] = to32(a);
        if (two) rs[(1 - c) * H + row * NZH + kp] = to32(b);
    }
}

// Ghost rows of the smoother, Jacobi-style among ghosts (each reads the
// values before the pass): a pass into tmp, then a scatter.  The row
// (1 - ws) z - sum(w z_stencil) = r is relaxed as
// z += (r + sum - (1 - ws) z) * gidiv, with gidiv = 1 / max(1 - ws,
// 2 sum|w on other ghosts|, 1e-3) set up per ghost: the exact row solve
// wherever the ghost block is diagonally dominant by a factor two (then
// the Jacobi pass over ghosts contracts), damped elsewhere.  Ghosts close
// to the surface have 1 - ws down to ~0.01; relaxing them only partly
// leaves a slowly converging error that doubled the Krylov iterations.

template <typename T>
__device__ __forceinline__ T ghost_value(const OpT<T> &c, const T rP, const T *__restrict__ z, int P,
                                         const T *__restrict__ gidiv) {
    const int id = c.gid[P];
    T sum = 0;
    for (int e = 0; e < 8; e++) {
        const int q = c.gidx[8 * id + e];
        if (q >= 0) sum += c.gw[8 * id + e] * z[q];
    }
    const T zp = z[P];
    return zp + (rP + sum - ((T)1 - c.gwself[id]) * zp) * gidiv[id];
}

template <typename T>
__global__ void k_mg0_ghost_scatter(const int *__restrict__ gcell, const int ng, const T *__restrict__ tmp, T *z,
                                    const int *gate) {
    MG_GATE(gate);
    GRID_STRIDE(g, (long long)ng) z[gcell[g]] = tmp[g];
}

// Outer boundary rows of the pressure operator, solved for the outer
// values.  The row of an outer cell couples it to a partner one coordinate
// further in (its mirror, or its periodic image): an interior cell for
// face cells, a face cell for edges, an edge cell for corners.  Each
// thread follows its cell's chain of partners down to an interior cell and
// evaluates the rows back up, so every outer value is a function of
// interior values alone: one launch, no ordering between outer cells, and
// no thread reads an outer value another thread writes.
template <typename T>
__device__ __forceinline__ T outer_chain_value(const OpT<T> &c, const FineRows<T> &fr, const T *z, long long P0) {
    long long chain[4];
    int face[4], layer[4];
    int n = 0;
    long long Q = P0;
    T v = 0;
    while (n < 4) {
        int i, j, k, L;
        cijk_fast(c.g, c.fdx, c.fdy, Q, i, j, k);
        const int f = owner_face(c.g, i, j, k, L);
        if (f < 0) {
            v = z[Q];
            break;
        }
        chain[n] = fr.at(Q, i, j, k);
        face[n] = f;
        layer[n] = L;
        n++;
        const BCRow<T> &F = c.bc[f];
        if (F.type == BCT_PERIODIC) {
            Q = periodic_image(c.g, i, j, k);
        } else {
            const int axis = face_axis(f);
            const long long s = axis == 0 ? c.g.sx : axis == 1 ? c.g.sy : 1;
            Q += (2 * L - 1) * (face_low(f) ? s : -s);
        }
    }
    for (int q = n - 1; q >= 0; q--) {
        const BCRow<T> &F = c.bc[face[q]];
        const T rv = fr.r[chain[q]];
        switch (F.type) {
        case BCT_PRESSURE:
        case BCT_VELPERIODIC: v = (rv - F.dir_m[layer[q] - 1] * v) / F.dir_o[layer[q] - 1]; break;
        default: v = rv + v; break;
        }
    }
    return v;
}

// The outer rows and the ghost rows of one smoother sweep in one launch:
// blocks [0, gblocks) compute the ghost values into tmp (from z before the
// pass, Jacobi-style), the others set the outer cells by chains; a chain
// that ends on a ghost cell reads its value before the pass as well.  The
// ghost values reach z in the following scatter launch.
template <typename T>
__global__ void __launch_bounds__(256)
k_mg0_outer(const OpT<T> c, const FineRows<T> fr, T *z, const int *__restrict__ outer, const int nout,
            const int *__restrict__ gcell, const long long *__restrict__ grow, const int ng, const int gblocks, T *tmp,
            const T *__restrict__ gidiv, const int *gate) {
    MG_GATE(gate);
    if ((int)blockIdx.x < gblocks) {
        const int g = blockIdx.x * blockDim.x + threadIdx.x;
        if (g < ng) tmp[g] = ghost_value(c, fr.r[grow[g]], z, gcell[g], gidiv);
        return;
    }
    const int t = (blockIdx.x - gblocks) * blockDim.x + threadIdx.x;
    if (t >= nout) return;
    z[outer[t]] = outer_chain_value(c, fr, z, outer[t]);
}

// 3-D launch over an (nx, ny, nz) box: threads along k, blocks along
// (k, j) tiles and i, so no thread divides an index.
constexpr int L3_TK = 32, L3_TJ = 8;
static inline dim3 l3_grid(int nx, int ny, int nz) {
    return dim3((unsigned)((nz + L3_TK - 1) / L3_TK), (unsigned)((ny + L3_TJ - 1) / L3_TJ), (unsigned)nx);
}
static inline dim3 l3_block() { return dim3(L3_TK, L3_TJ, 1); }
#define L3_INDEX(I, J, K, NY, NZ)                                      \
    const int K = blockIdx.x * L3_TK + threadIdx.x;                     \
    const int J = blockIdx.y * L3_TJ + threadIdx.y;                     \
    const int I = blockIdx.z;                                           \
    if (K >= (NZ) || J >= (NY)) return;

// Restriction of the fine normalised rows' residual, scaled to
// conductance form (Vol * coeffsum * r), into a level 1 whose groups are
// uneven.  Tiles: coarse ranges [segj[b], segj[b+1]) x [segk[b], segk[b+1])
// cut on the host so that each covers at most 8 fine rows and 32 fine
// columns (as many as fit), ending on group boundaries.  A block takes one
// tile of MG0_RPLANES consecutive coarse planes; its 32 x 8 threads each
// take one fine (j, k) (coalesced rows along k) and, per coarse plane, sum
// the one or two fine planes of its group into shared memory - in FP32 both
// fine planes loaded before either is tested (a one-plane group reads its
// plane twice and adds it once), every plane's loads in flight together;
// the tile's tables read once; then one thread per coarse cell and plane
// adds up its one to four entries.  Grid (nsegk, nsegj, ceil(nx1 /
// MG0_RPLANES)).
constexpr int MG0_RPLANES = 4;

template <typename T, bool SPLIT>
__global__ void __launch_bounds__(256)
k_mg0_restrict_g(const OpT<T> c, const FineRows<T> fr, const T *__restrict__ z, MGLevel<T> L1,
                 const int *__restrict__ segj, const int *__restrict__ segk, const Per3 per, const int init,
                 const int *gate) {
    MG_GATE(gate);
    __shared__ T part[MG0_RPLANES][8][33];
    const Grid &g = c.g;
    const int J0 = segj[blockIdx.y], J1 = segj[blockIdx.y + 1];
    const int K0 = segk[blockIdx.x], K1 = segk[blockIdx.x + 1];
    const int jb = L1.ch[1][J0], je = L1.ch[1][J1];
    const int kb = L1.ch[2][K0], ke = L1.ch[2][K1];
    const bool live = (int)threadIdx.y < je - jb && (int)threadIdx.x < ke - kb;
    const int j = live ? jb + threadIdx.y : jb, k = live ? kb + threadIdx.x : kb;
    const int Jj = j + 2, Kk = k + 2;
    const T vyz = c.d[1][Jj] * c.d[2][Kk];
    const T kyz = c.ks[1][Jj] + c.ks[2][Kk];
    const T kmy = c.km[1][Jj], kpy = c.kp[1][Jj], kmz = c.km[2][Kk], kpz = c.kp[2][Kk];
    const int Ib = blockIdx.z * MG0_RPLANES;
#pragma unroll
    for (int q = 0; q < MG0_RPLANES; q++) {
        const int I = min(Ib + q, L1.nx - 1);
        const int i0 = L1.ch[0][I], two = L1.ch[0][I + 1] - i0 > 1;
        T res[2] = {0, 0}, w[2] = {0, 0};
        bool use[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int i = i0 + (h & two);
            const long long P = cidx(g, i, j, k), q = SPLIT ? fr.split_index(i, j, k) : P;
            const int Ii = i + 2;
            use[h] = live && (h == 0 || two) && fr.flag[q] == FLUID && !(c.p_singular && P == c.pinned);
            // FP64 rows are computed only where used: the FP64 pipe, not
            // the latency, bounds that form.
            if (sizeof(T) == 4 || use[h]) {
                const T nb = c.km[0][Ii] * z[P - g.sx] + c.kp[0][Ii] * z[P + g.sx] + kmy * z[P - g.sy] +
                             kpy * z[P + g.sy] + kmz * z[P - 1] + kpz * z[P + 1];
                res[h] = fr.r[q] - (z[P] - fr.dinv[q] * nb);
                w[h] = c.d[0][Ii] * vyz * (c.ks[0][Ii] + kyz);
            }
        }
        T acc = 0;
#pragma unroll
        for (int h = 0; h < 2; h++) acc = use[h] ? acc + w[h] * res[h] : acc;
        part[q][threadIdx.y][threadIdx.x] = acc;
    }
    __syncthreads();
    const int nk = K1 - K0, ncell = (J1 - J0) * nk;
    for (int t = threadIdx.y * 32 + threadIdx.x; t < MG0_RPLANES * ncell; t += 256) {
        const int q = t / ncell, e = t - q * ncell;
        const int I = Ib + q;
        if (I >= L1.nx) break;
        const int J = J0 + e / nk, K = K0 + e % nk;
        const int ja = L1.ch[1][J] - jb, jz = L1.ch[1][J + 1] - jb;
        const int ka = L1.ch[2][K] - kb, kz = L1.ch[2][K + 1] - kb;
        T sum = 0;
        for (int y = ja; y < jz; y++)
            for (int x = ka; x < kz; x++) sum += part[q][y][x];
        const long long c1 = lidx(L1, I, J, K);
        L1.R[c1] = sum;
        if (init) restrict_init(L1, c1, I, J, K, sum, per);
    }
}

// Prolongation into the fine grid from a level 1 of uneven groups: each
// thread takes one fine (j, k) on mg0_pplanes<T>() consecutive planes (four
// in FP32; one in FP64, whose blend is bound by the FP64 pipe rather than
// by latency), reads its j and k transfer tables once, addresses coarse
// cells in 32-bit arithmetic (a level has fewer than 2^31 cells) and
// issues every load (flags, z, the x tables, the coarse values) before any
// store; a cell that takes no correction stores z back.  Same arithmetic
// as prolong_value.  Grid (ceil(nz/32), ceil(ny/8), ceil(nx/planes)) of
// 32 x 8 threads.
template <typename T>
__host__ __device__ constexpr int mg0_pplanes() { return sizeof(T) == 4 ? 4 : 1; }

template <typename T>
__global__ void __launch_bounds__(256)
k_mg0_prolong(const OpT<T> c, T *z, const MGLevel<T> C, const int *gate) {
    constexpr int MG0_PPLANES = mg0_pplanes<T>();
    MG_GATE(gate);
    const Grid &g = c.g;
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    if (k >= g.nz || j >= g.ny) return;
    const int cny = C.ny, cnz = C.nz;
    const int ys[2] = {C.pa[1][j], C.po[1][j]}, zs[2] = {C.pa[2][k], C.po[2][k]};
    const T wy = C.pw[1][j], wz = C.pw[2][k];
    const T wys[2] = {wy, (T)1 - wy}, wzs[2] = {wz, (T)1 - wz};
    const int i0 = blockIdx.z * MG0_PPLANES;
    long long Ps[MG0_PPLANES];
    T out[MG0_PPLANES];
#pragma unroll
    for (int p = 0; p < MG0_PPLANES; p++) {
        const int i = min(i0 + p, g.nx - 1);
        const long long P = cidx(g, i, j, k);
        const uint8_t fl = c.flag[P];
        const T zp = z[P];
        const int xs[2] = {C.pa[0][i], C.po[0][i]};
        const T wx = C.pw[0][i];
        const T wxs[2] = {wx, (T)1 - wx};
        T v[2][2][2];
        bool act[2][2][2];
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int cc = 0; cc < 2; cc++) {
                    v[a][b][cc] = 0;
                    act[a][b][cc] = false;
                    if (xs[a] < 0 || ys[b] < 0 || zs[cc] < 0) continue;
                    const int q = (xs[a] * cny + ys[b]) * cnz + zs[cc];
                    v[a][b][cc] = C.Z[q];
                    act[a][b][cc] = active_bits(C.diag[q]);
                }
        const bool take = (fl == FLUID || fl == GHOST) && !(c.p_singular && P == c.pinned);
        // As in the restriction: the FP64 blend only where it is used.
        const T corr = sizeof(T) == 4 || take ? trilinear(v, act, wxs, wys, wzs) : (T)0;
        out[p] = take ? zp + corr : zp;
        Ps[p] = P;
    }
#pragma unroll
    for (int p = 0; p < MG0_PPLANES; p++)
        if (i0 + p < g.nx) z[Ps[p]] = out[p];
}

// Restriction when level 1 halves every axis: one thread per fine (j, k)
// and coarse plane I (both fine planes 2I, 2I+1), the k pair summed by a
// lane shuffle and the j pair through shared memory, so every load is a
// coalesced row and the whole fine grid is in flight at once.  Grid
// (ceil(nz/32), ceil(ny/8), L1.nx) of 32 x 8 threads.
template <typename T, bool SPLIT>
__global__ void __launch_bounds__(256)
k_mg0_restrict2(const OpT<T> c, const FineRows<T> fr, const T *__restrict__ z, MGLevel<T> L1, const Per3 per,
                const int init, const int *gate) {
    MG_GATE(gate);
    __shared__ T part[8][33];
    const Grid &g = c.g;
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, I = blockIdx.z;
    T acc = 0;
    if (j < g.ny && k < g.nz) {
        const int Jj = j + 2, Kk = k + 2;
        const T vyz = c.d[1][Jj] * c.d[2][Kk];
        const T kyz = c.ks[1][Jj] + c.ks[2][Kk];
        const T kmy = c.km[1][Jj], kpy = c.kp[1][Jj], kmz = c.km[2][Kk], kpz = c.kp[2][Kk];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int i = 2 * I + h;
            if (i >= g.nx) break;
            const long long P = cidx(g, i, j, k), q = SPLIT ? fr.split_index(i, j, k) : P;
            if (fr.flag[q] != FLUID || (c.p_singular && P == c.pinned)) continue;
            const int Ii = i + 2;
            const T nb = c.km[0][Ii] * z[P - g.sx] + c.kp[0][Ii] * z[P + g.sx] + kmy * z[P - g.sy] +
                         kpy * z[P + g.sy] + kmz * z[P - 1] + kpz * z[P + 1];
            const T res = fr.r[q] - (z[P] - fr.dinv[q] * nb);
            acc += c.d[0][Ii] * vyz * (c.ks[0][Ii] + kyz) * res;
        }
    }
    acc += __shfl_down_sync(0xffffffffu, acc, 1);
    part[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if ((threadIdx.y & 1) || (threadIdx.x & 1)) return;
    const int J = blockIdx.y * 4 + (threadIdx.y >> 1), K = blockIdx.x * 16 + (threadIdx.x >> 1);
    if (J < L1.ny && K < L1.nz) {
        const long long c1 = lidx(L1, I, J, K);
        const T R = part[threadIdx.y][threadIdx.x] + part[threadIdx.y + 1][threadIdx.x];
        L1.R[c1] = R;
        if (init) restrict_init(L1, c1, I, J, K, R, per);
    }
}

// Prolongation when level 1 halves every axis: the block's fine tile (one
// plane, 8 j x 32 k) reads its coarse neighbourhood (the two coarse planes
// it touches, 6 x 18 cells of each) into shared memory once; the few
// neighbours outside it (periodic wraps) are read from global memory.
// Same arithmetic as prolong_value.
template <typename T>
__global__ void __launch_bounds__(256)
k_mg0_prolong2(const OpT<T> c, T *z, const MGLevel<T> C, const int *gate) {
    MG_GATE(gate);
    constexpr int TJ = 6, TK = 18;
    __shared__ T tz[2][TJ][TK];
    __shared__ bool ta[2][TJ][TK];
    const int i = blockIdx.z;
    const int k0 = blockIdx.x * 32, j0 = blockIdx.y * 8;
    const int Jmin = (j0 >> 1) - 1, Kmin = (k0 >> 1) - 1;
    const int Ipl[2] = {i >> 1, C.po[0][i]};
    const int t = threadIdx.y * 32 + threadIdx.x;
    if (t < 2 * TJ * TK) {
        const int pl = t / (TJ * TK), jj = (t / TK) % TJ, kk = t % TK;
        const int Ic = Ipl[pl], Jc = Jmin + jj, Kc = Kmin + kk;
        T zv = 0;
        bool av = false;
        if (Ic >= 0 && Jc >= 0 && Jc < C.ny && Kc >= 0 && Kc < C.nz) {
            const long long q = lidx(C, Ic, Jc, Kc);
            zv = C.Z[q];
            av = active_bits(C.diag[q]);
        }
        tz[pl][jj][kk] = zv;
        ta[pl][jj][kk] = av;
    }
    __syncthreads();
    const int k = k0 + threadIdx.x, j = j0 + threadIdx.y;
    if (k >= c.g.nz || j >= c.g.ny) return;
    const long long P = cidx(c.g, i, j, k);
    const uint8_t fl = c.flag[P];
    if (fl != FLUID && fl != GHOST) return;
    if (c.p_singular && P == c.pinned) return;
    const int ys[2] = {j >> 1, C.po[1][j]}, zs[2] = {k >> 1, C.po[2][k]};
    const T wx = C.pw[0][i], wy = C.pw[1][j], wz = C.pw[2][k];
    const T wxs[2] = {wx, (T)1 - wx}, wys[2] = {wy, (T)1 - wy}, wzs[2] = {wz, (T)1 - wz};
    T v[2][2][2];
    bool act[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                v[a][b][cc] = 0;
                act[a][b][cc] = false;
                if (Ipl[a] < 0 || ys[b] < 0 || zs[cc] < 0) continue;
                const int jj = ys[b] - Jmin, kk = zs[cc] - Kmin;
                if (jj >= 0 && jj < TJ && kk >= 0 && kk < TK) {
                    v[a][b][cc] = tz[a][jj][kk];
                    act[a][b][cc] = ta[a][jj][kk];
                } else {
                    const long long q = lidx(C, Ipl[a], ys[b], zs[cc]);
                    v[a][b][cc] = C.Z[q];
                    act[a][b][cc] = active_bits(C.diag[q]);
                }
            }
    z[P] += trilinear(v, act, wxs, wys, wzs);
}

// ------------------------------------------------------ level building --
// Centre-distance ratios of a new level, per axis (n + 1 entries): [I] for
// the low face of cell I (I = 0: the low boundary, or the periodic wrap),
// [n] for the high boundary; each is (finer centre distance) / (coarse
// centre distance) across the face (to the mirrored centre at a boundary).
struct FaceRatio {
    const double *r[3];
};

// Level 1 from the fine grid (FP64): conductances Vol*k of fluid-fluid
// faces, pressure-Dirichlet boundary conductances, periodic wraps.
__global__ void k_mg_build1(const OpT<double> c, MGLevel<double> L, double *Gx, double *Gy, double *Gz,
                            const Per3 per, const FaceRatio fr) {
    const Grid &g = c.g;
    GRID_STRIDE(q, L.n) {
        const int K = (int)(q % L.nz);
        const int J = (int)((q / L.nz) % L.ny);
        const int I = (int)(q / ((long long)L.nz * L.ny));
        const int i0 = L.ch[0][I], i1 = L.ch[0][I + 1] - 1;
        const int j0 = L.ch[1][J], j1 = L.ch[1][J + 1] - 1;
        const int k0 = L.ch[2][K], k1 = L.ch[2][K + 1] - 1;
        auto active = [&](int i, int j, int k) {
            const long long P = cidx(g, i, j, k);
            return c.flag[P] == FLUID && !(c.p_singular && P == c.pinned);
        };
        auto dirf = [](int t) { return t == BCT_PRESSURE || t == BCT_VELPERIODIC; };
        double tx = 0, ty = 0, tz = 0, gl[3] = {0, 0, 0}, gh[3] = {0, 0, 0};
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    if (!active(i, j, k)) continue;
                    const double v = c.d[0][i + 2] * c.d[1][j + 2] * c.d[2][k + 2];
                    if (i == i0) {
                        if (i > 0) { if (active(i - 1, j, k)) tx += v * c.km[0][i + 2]; }
                        else if (per.p[0] && g.nx > 1) { if (active(g.nx - 1, j, k)) tx += v * c.km[0][2]; }
                    }
                    if (j == j0) {
                        if (j > 0) { if (active(i, j - 1, k)) ty += v * c.km[1][j + 2]; }
                        else if (per.p[1] && g.ny > 1) { if (active(i, g.ny - 1, k)) ty += v * c.km[1][2]; }
                    }
                    if (k == k0) {
                        if (k > 0) { if (active(i, j, k - 1)) tz += v * c.km[2][k + 2]; }
                        else if (per.p[2] && g.nz > 1) { if (active(i, j, g.nz - 1)) tz += v * c.km[2][2]; }
                    }
                    const BCRow<double> &W = c.bc[F_W], &E = c.bc[F_E], &S = c.bc[F_S], &N = c.bc[F_N];
                    const BCRow<double> &D = c.bc[F_D], &U = c.bc[F_U];
                    if (i == 0 && dirf(W.type)) gl[0] += v * c.km[0][2] * (1 + W.dir_m[0] / W.dir_o[0]);
                    if (i == g.nx - 1 && dirf(E.type)) gh[0] += v * c.kp[0][g.nx + 1] * (1 + E.dir_m[0] / E.dir_o[0]);
                    if (j == 0 && dirf(S.type)) gl[1] += v * c.km[1][2] * (1 + S.dir_m[0] / S.dir_o[0]);
                    if (j == g.ny - 1 && dirf(N.type)) gh[1] += v * c.kp[1][g.ny + 1] * (1 + N.dir_m[0] / N.dir_o[0]);
                    if (k == 0 && dirf(D.type)) gl[2] += v * c.km[2][2] * (1 + D.dir_m[0] / D.dir_o[0]);
                    if (k == g.nz - 1 && dirf(U.type)) gh[2] += v * c.kp[2][g.nz + 1] * (1 + U.dir_m[0] / U.dir_o[0]);
                }
        L.Tx[q] = (I == 0 && L.nx == 1) ? 0.0 : fr.r[0][I] * tx;
        L.Ty[q] = (J == 0 && L.ny == 1) ? 0.0 : fr.r[1][J] * ty;
        L.Tz[q] = (K == 0 && L.nz == 1) ? 0.0 : fr.r[2][K] * tz;
        Gx[q] = fr.r[0][0] * gl[0] + fr.r[0][L.nx] * gh[0];
        Gy[q] = fr.r[1][0] * gl[1] + fr.r[1][L.ny] * gh[1];
        Gz[q] = fr.r[2][0] * gl[2] + fr.r[2][L.nz] * gh[2];
    }
}

// Coarse level c from level f (FP64).
__global__ void k_mg_buildc(const MGLevel<double> F, const double *__restrict__ fGx, const double *__restrict__ fGy,
                            const double *__restrict__ fGz, MGLevel<double> C, double *Gx, double *Gy, double *Gz,
                            const FaceRatio fr) {
    GRID_STRIDE(q, C.n) {
        const int K = (int)(q % C.nz);
        const int J = (int)((q / C.nz) % C.ny);
        const int I = (int)(q / ((long long)C.nz * C.ny));
        const int i0 = C.ch[0][I], i1 = C.ch[0][I + 1] - 1;
        const int j0 = C.ch[1][J], j1 = C.ch[1][J + 1] - 1;
        const int k0 = C.ch[2][K], k1 = C.ch[2][K + 1] - 1;
        // A Dirichlet conductance sits on a cell at the low or high end of
        // its axis (both ends at once only on a one-cell axis, ratio 1).
        auto bscale = [&](int a, int i, int nf, int nc) {
            return i == 0 ? fr.r[a][0] : i == nf - 1 ? fr.r[a][nc] : 1.0;
        };
        double tx = 0, ty = 0, tz = 0, gx = 0, gy = 0, gz = 0;
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    const long long f = lidx(F, i, j, k);
                    if (i == i0) tx += F.Tx[f];
                    if (j == j0) ty += F.Ty[f];
                    if (k == k0) tz += F.Tz[f];
                    gx += bscale(0, i, F.nx, C.nx) * fGx[f];
                    gy += bscale(1, j, F.ny, C.ny) * fGy[f];
                    gz += bscale(2, k, F.nz, C.nz) * fGz[f];
                }
        C.Tx[q] = (I == 0 && C.nx == 1) ? 0.0 : fr.r[0][I] * tx;
        C.Ty[q] = (J == 0 && C.ny == 1) ? 0.0 : fr.r[1][J] * ty;
        C.Tz[q] = (K == 0 && C.nz == 1) ? 0.0 : fr.r[2][K] * tz;
        Gx[q] = gx;
        Gy[q] = gy;
        Gz[q] = gz;
    }
}

// Couplings of a coarse cell: calls fn(neighbour index, conductance).
template <typename T, typename Fn>
__device__ inline void for_neighbours(const MGLevel<T> &L, int I, int J, int K, const int *per, Fn fn) {
    const long long q = lidx(L, I, J, K);
    const long long sx = (long long)L.ny * L.nz, sy = L.nz;
    if (I > 0) fn(q - sx, L.Tx[q]);
    else if (per[0] && L.nx > 1) fn(lidx(L, L.nx - 1, J, K), L.Tx[q]);
    if (I < L.nx - 1) fn(q + sx, L.Tx[q + sx]);
    else if (per[0] && L.nx > 1) fn(lidx(L, 0, J, K), L.Tx[lidx(L, 0, J, K)]);
    if (J > 0) fn(q - sy, L.Ty[q]);
    else if (per[1] && L.ny > 1) fn(lidx(L, I, L.ny - 1, K), L.Ty[q]);
    if (J < L.ny - 1) fn(q + sy, L.Ty[q + sy]);
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

// 1 / diag of a level (computed in FP64), 0 for inactive cells.
template <typename T>
__global__ void k_inverse(const double *__restrict__ d, T *b, long long n) {
    GRID_STRIDE(q, n) b[q] = d[q] == 0.0 ? (T)0 : (T)(1.0 / d[q]);
}

template <typename T>
__global__ void k_convert(const double *__restrict__ a, T *b, long long n) {
    GRID_STRIDE(q, n) b[q] = (T)a[q];
}

// ----------------------------------------------------- coarse kernels --
template <typename T>
__device__ inline void coarse_relax(const MGLevel<T> &L, int I, int J, int K, const int *per) {
    const long long q = lidx(L, I, J, K);
    const T d = L.diag[q];
    if (d == (T)0) {
        L.Z[q] = 0;
        return;
    }
    T s = L.R[q];
    for_neighbours(L, I, J, K, per, [&](long long m, T t) { s += t * L.Z[m]; });
    L.Z[q] = L.idiag ? s * L.idiag[q] : s / d;
}

template <typename T>
__device__ inline T coarse_residual(const MGLevel<T> &L, int I, int J, int K, const int *per) {
    const long long q = lidx(L, I, J, K);
    if (L.diag[q] == (T)0) return 0;
    T s = L.R[q] - L.diag[q] * L.Z[q];
    for_neighbours(L, I, J, K, per, [&](long long m, T t) { s += t * L.Z[m]; });
    return s;
}

// Colours a level needs: 4 with a seam on an odd periodic axis, else 2.
template <typename T>
__host__ __device__ inline int level_colors(const MGLevel<T> &L, const int *per) {
    const bool seam = (per[0] && (L.nx & 1) && L.nx > 1) || (per[1] && (L.ny & 1) && L.ny > 1) ||
                      (per[2] && (L.nz & 1) && L.nz > 1);
    return seam ? 4 : 2;
}

// The residual of cell (I, J, K) on a level without periodic axes, every
// load issued up front (as coarse_relax_open).
template <typename T>
__device__ __forceinline__ T coarse_residual_open(const MGLevel<T> &L, int I, int J, int K) {
    const long long sx = (long long)L.ny * L.nz, sy = L.nz;
    const long long q = lidx(L, I, J, K);
    const bool he = I < L.nx - 1, hn = J < L.ny - 1, hu = K < L.nz - 1;
    const long long qw = I > 0 ? q - sx : q, qe = he ? q + sx : q;
    const long long qs = J > 0 ? q - sy : q, qn = hn ? q + sy : q;
    const long long qd = K > 0 ? q - 1 : q, qu = hu ? q + 1 : q;
    const T d = L.diag[q], R = L.R[q], zc = L.Z[q];
    const T tw = L.Tx[q], te = L.Tx[qe], ts = L.Ty[q], tn = L.Ty[qn], td = L.Tz[q], tu = L.Tz[qu];
    const T zw = L.Z[qw], ze = L.Z[qe], zs = L.Z[qs], zn = L.Z[qn], zd = L.Z[qd], zu = L.Z[qu];
    T s = R - d * zc;
    s += tw * zw;
    s += (he ? te : (T)0) * ze;
    s += ts * zs;
    s += (hn ? tn : (T)0) * zn;
    s += td * zd;
    s += (hu ? tu : (T)0) * zu;
    return d == (T)0 ? (T)0 : s;
}

// Restricted residual of coarse cell (I, J, K): the sum over the finer
// cells it covers.  skip >= 0: the finer level's last pass was a red/black
// Gauss-Seidel pass over colour `skip`, whose cells then have zero
// residual up to rounding; they are left out.
template <typename T>
__device__ inline T coarse_restrict_value(const MGLevel<T> &F, const MGLevel<T> &C, int I, int J, int K,
                                          const int *per, int skip) {
    const int i0 = C.ch[0][I], i1 = C.ch[0][I + 1] - 1;
    const int j0 = C.ch[1][J], j1 = C.ch[1][J + 1] - 1;
    const int k0 = C.ch[2][K], k1 = C.ch[2][K + 1] - 1;
    const bool open = !per[0] && !per[1] && !per[2];
    T acc = 0;
    for (int i = i0; i <= i1; i++)
        for (int j = j0; j <= j1; j++)
            for (int k = k0; k <= k1; k++) {
                if (((i + j + k) & 1) == skip) continue;
                acc += open ? coarse_residual_open(F, i, j, k) : coarse_residual(F, i, j, k, per);
            }
    return acc;
}

template <typename T>
__global__ void k_fill0(T *z, const long long n, const int *gate) {
    MG_GATE(gate);
    GRID_STRIDE(q, n) z[q] = 0;
}


// Branch-free relaxation of coarse cell (I, J, K) on a level without
// periodic axes: every load is issued up front (low-face conductances are
// 0 on the first cell of an axis; high neighbours off the level are read
// at the cell itself and weighted 0).
template <typename T>
__device__ __forceinline__ void coarse_relax_open(const MGLevel<T> &L, int I, int J, int K) {
    const long long sx = (long long)L.ny * L.nz, sy = L.nz;
    const long long q = lidx(L, I, J, K);
    const bool he = I < L.nx - 1, hn = J < L.ny - 1, hu = K < L.nz - 1;
    const long long qw = I > 0 ? q - sx : q, qe = he ? q + sx : q;
    const long long qs = J > 0 ? q - sy : q, qn = hn ? q + sy : q;
    const long long qd = K > 0 ? q - 1 : q, qu = hu ? q + 1 : q;
    const T R = L.R[q];
    const T tw = L.Tx[q], te = L.Tx[qe], ts = L.Ty[q], tn = L.Ty[qn], td = L.Tz[q], tu = L.Tz[qu];
    const T zw = L.Z[qw], ze = L.Z[qe], zs = L.Z[qs], zn = L.Z[qn], zd = L.Z[qd], zu = L.Z[qu];
    T s = R;
    s += tw * zw;
    s += (he ? te : (T)0) * ze;
    s += ts * zs;
    s += (hn ? tn : (T)0) * zn;
    s += td * zd;
    s += (hu ? tu : (T)0) * zu;
    // An inactive cell has 1/diag = 0 (and R = 0, no conductances): Z = 0.
    L.Z[q] = s * L.idiag[q];
}

// One colour pass on a coarse level; k pairs as on the fine grid when the
// level has no periodic seam (pairs = 1, grid ceil(nz/64) wide in k).
template <typename T>
__global__ void __launch_bounds__(256)
k_mgc_color(MGLevel<T> L, const int color, const int pairs, const Per3 per, const int *gate) {
    MG_GATE(gate);
    const int I = blockIdx.z, J = blockIdx.y * L3_TJ + threadIdx.y;
    const bool open = !per.p[0] && !per.p[1] && !per.p[2];
    if (pairs) {
        const int K = 2 * (blockIdx.x * L3_TK + threadIdx.x) + ((I + J + color) & 1);
        if (J < L.ny && K < L.nz) {
            if (open) coarse_relax_open(L, I, J, K);
            else coarse_relax(L, I, J, K, per.p);
        }
    } else {
        const int K = blockIdx.x * L3_TK + threadIdx.x;
        if (J < L.ny && K < L.nz && cell_color(I, J, K, L.nx, L.ny, L.nz, per.p) == color)
            coarse_relax(L, I, J, K, per.p);
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_mgc_restrict(const MGLevel<T> F, MGLevel<T> C, const Per3 per, const int skip, const int init, const int *gate) {
    MG_GATE(gate);
    L3_INDEX(I, J, K, C.ny, C.nz);
    const long long q = lidx(C, I, J, K);
    const T R = coarse_restrict_value(F, C, I, J, K, per.p, skip);
    C.R[q] = R;
    if (init) restrict_init(C, q, I, J, K, R, per);
}

template <typename T>
__global__ void __launch_bounds__(256) k_mgc_prolong(const MGLevel<T> C, MGLevel<T> F, const int *gate) {
    MG_GATE(gate);
    L3_INDEX(I, J, K, F.ny, F.nz);
    const long long q = lidx(F, I, J, K);
    if (F.diag[q] == (T)0) return;
    F.Z[q] += prolong_value(C, I, J, K);
}

// Whole V-cycle over levels [first, nlev) inside one thread block, with
// every level's arrays and its transfer tables (groups, parents,
// prolongation weights) copied into shared memory; each thread takes cells
// tid, tid + TAIL_THREADS, ... (levels of at most TAIL_CELLS cells).  R of
// level `first` is read from global memory and its Z written back.
constexpr int TAIL_THREADS = 1024;
constexpr int TAIL_CELLS = TAIL_THREADS;
constexpr size_t TAIL_SMEM_MAX = 200 * 1024;

template <typename T>
__global__ void __launch_bounds__(TAIL_THREADS)
k_mg_tail(const TailDesc<T> d, const uint4 *__restrict__ img, const int nu1, const int nu2, const int csweeps,
          const Per3 per, const int singular, const int *gate) {
    MG_GATE(gate);
    extern __shared__ __align__(16) unsigned char tail_smem[];
    __shared__ MGLevel<T> loc[TAIL_MAXL];
    const int tid = threadIdx.x;
    const int first = 0, nlev = d.ntl;
    // The image: every level's constants and zeroed R, Z, in one pass of
    // independent 16-byte loads.
    uint4 *dst = reinterpret_cast<uint4 *>(tail_smem);
    for (int q = tid; q < d.words16; q += TAIL_THREADS) dst[q] = __ldg(img + q);
    if (tid < nlev) {
        const TailLevel &t = d.lv[tid];
        MGLevel<T> L{};
        L.nx = t.nx;
        L.ny = t.ny;
        L.nz = t.nz;
        L.n = t.n;
        L.cx = t.cx;
        L.cy = t.cy;
        L.cz = t.cz;
        T *arr[7];
        for (int a = 0; a < 7; a++) arr[a] = reinterpret_cast<T *>(tail_smem + t.off[a]);
        L.Tx = arr[0];
        L.Ty = arr[1];
        L.Tz = arr[2];
        L.diag = arr[3];
        L.R = arr[4];
        L.Z = arr[5];
        L.idiag = arr[6];
        for (int a = 0; a < 3; a++) {
            L.pw[a] = tid > 0 ? reinterpret_cast<const T *>(tail_smem + t.opw[a]) : nullptr;
            L.po[a] = tid > 0 ? reinterpret_cast<const int *>(tail_smem + t.opo[a]) : nullptr;
            L.pa[a] = tid > 0 ? reinterpret_cast<const int *>(tail_smem + t.opa[a]) : nullptr;
            L.ch[a] = tid > 0 ? reinterpret_cast<const int *>(tail_smem + t.och[a]) : nullptr;
        }
        loc[tid] = L;
    }
    __syncthreads();
    {
        const MGLevel<T> &L = loc[0];
        for (int c = tid; c < L.n; c += TAIL_THREADS) L.R[c] = d.R_first[c];
    }
    __syncthreads();
    // Thread tid takes cell tid of a level (a level holds at most
    // TAIL_THREADS cells): its coordinates and colour, computed once per
    // phase of the level.
    struct Pos {
        int I, J, K, col;
    };
    auto pos = [&](const MGLevel<T> &L) {
        Pos p{0, 0, 0, -1};
        if (tid < L.n) {
            const int nyz = L.ny * L.nz;
            p.I = tid / nyz;
            const int rem = tid - p.I * nyz;
            p.J = rem / L.nz;
            p.K = rem - p.J * L.nz;
            p.col = cell_color(p.I, p.J, p.K, L.nx, L.ny, L.nz, per.p);
        }
        return p;
    };
    // Colour passes of a level.  With two colours thread t takes (k, k+1)
    // pair t of the level and relaxes its cell of the pass's colour (half
    // the warps of one cell per thread, and no lane idles on the other
    // colour), through the branch-free relaxation on levels without
    // periodic axes; with four, cell t and a colour test.  Work of at most
    // 32 threads runs in warp 0 alone, its passes separated by warp
    // barriers, and one block barrier after the last.
    const bool open = !per.p[0] && !per.p[1] && !per.p[2];
    auto sweep = [&](const MGLevel<T> &L, int nsw) {
        const int ncol = level_colors(L, per.p);
        const bool pairs = ncol == 2;
        const int nzw = pairs ? (L.nz + 1) / 2 : L.nz;
        const int items = L.nx * L.ny * nzw;
        int I = 0, J = 0, kw = 0, cc = -1;
        if (tid < items) {
            const int nyz = L.ny * nzw;
            I = tid / nyz;
            const int rem = tid - I * nyz;
            J = rem / nzw;
            kw = rem - J * nzw;
            if (!pairs) cc = cell_color(I, J, kw, L.nx, L.ny, L.nz, per.p);
        }
        auto pass = [&](int col) {
            if (tid >= items) return;
            if (pairs) {
                const int K = 2 * kw + ((I + J + col) & 1);
                if (K >= L.nz) return;
                if (open) coarse_relax_open(L, I, J, K);
                else coarse_relax(L, I, J, K, per.p);
            } else if (cc == col) {
                coarse_relax(L, I, J, kw, per.p);
            }
        };
        if (items <= 32) {
            if (tid < 32)
                for (int s = 0; s < nsw; s++)
                    for (int col = 0; col < ncol; col++) {
                        pass(col);
                        __syncwarp();
                    }
            __syncthreads();
            return;
        }
        for (int s = 0; s < nsw; s++)
            for (int col = 0; col < ncol; col++) {
                pass(col);
                __syncthreads();
            }
    };
    for (int l = first; l < nlev; l++) {
        const MGLevel<T> &L = loc[l - first];
        if (l == nlev - 1 && singular && tid < 32) {
            // Without a pressure boundary value the coarse operators are
            // singular (constants are their null space) and the restricted
            // residual need not sum to zero (the fine grid's pinned row
            // absorbs the difference): the coarsest sweeps would drift along
            // the constants.  Its right-hand side is made consistent first:
            // the mean over active cells is removed.
            T sum = 0, cnt = 0;
            for (int c = tid; c < L.n; c += 32)
                if (L.diag[c] != (T)0) {
                    sum += L.R[c];
                    cnt += (T)1;
                }
            for (int o = 16; o > 0; o >>= 1) {
                sum += __shfl_xor_sync(0xffffffffu, sum, o);
                cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            }
            const T mean = cnt > (T)0 ? sum / cnt : (T)0;
            __syncwarp();
            for (int c = tid; c < L.n; c += 32)
                if (L.diag[c] != (T)0) L.R[c] -= mean;
        }
        if (l == nlev - 1) __syncthreads();
        sweep(L, l == nlev - 1 ? csweeps : nu1);
        if (l < nlev - 1) {
            const MGLevel<T> &C = loc[l + 1 - first];
            const Pos p = pos(C);
            const int skip = nu1 > 0 && level_colors(L, per.p) == 2 ? 1 : -1;
            if (tid < C.n) C.R[tid] = coarse_restrict_value(L, C, p.I, p.J, p.K, per.p, skip);
            __syncthreads();
        }
    }
    for (int l = nlev - 2; l >= first; l--) {
        const MGLevel<T> &L = loc[l - first], &C = loc[l + 1 - first];
        const Pos p = pos(L);
        if (tid < L.n && L.diag[tid] != (T)0) L.Z[tid] += prolong_value(C, p.I, p.J, p.K);
        __syncthreads();
        sweep(L, nu2);
    }
    const MGLevel<T> &L = loc[0];
    for (int c = tid; c < L.n; c += TAIL_THREADS) d.Z_first[c] = L.Z[c];
}

// Shared memory the tail kernel needs for levels [first, nlev): seven
// arrays per level and the transfer tables of the levels below `first`.
template <typename T>
static size_t tail_bytes(const std::vector<MGLevel<T>> &lv, int first) {
    size_t b = 0;
    for (int l = first; l < (int)lv.size(); l++) b += 7 * sizeof(T) * (size_t)lv[l].n;
    for (int l = first + 1; l < (int)lv.size(); l++) {
        const int nf[3] = {lv[l - 1].nx, lv[l - 1].ny, lv[l - 1].nz}, nc[3] = {lv[l].nx, lv[l].ny, lv[l].nz};
        for (int a = 0; a < 3; a++) b += (sizeof(T) + 2 * sizeof(int)) * (size_t)nf[a] + sizeof(int) * (nc[a] + 1);
    }
    return b;
}

// The tail's image (see TailDesc): the same layout as tail_bytes counts,
// arrays per level (Tx, Ty, Tz, diag, R, Z, idiag), then the weight tables
// and the int tables of the levels below the first; 16-byte aligned.
template <typename T>
static int build_tail_image(const std::vector<MGLevel<T>> &lv, int first, TailDesc<T> &d,
                            std::vector<unsigned char> &img) {
    const int nl = (int)lv.size();
    d.ntl = nl - first;
    if (d.ntl > TAIL_MAXL) return -1;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += bytes;
        return (int)at;
    };
    for (int l = first; l < nl; l++) {
        TailLevel &t = d.lv[l - first];
        const MGLevel<T> &L = lv[l];
        t.nx = L.nx, t.ny = L.ny, t.nz = L.nz, t.cx = L.cx, t.cy = L.cy, t.cz = L.cz, t.n = L.n;
        for (int a = 0; a < 7; a++) t.off[a] = take(sizeof(T) * (size_t)L.n);
    }
    for (int l = first + 1; l < nl; l++) {
        const int nf[3] = {lv[l - 1].nx, lv[l - 1].ny, lv[l - 1].nz};
        for (int a = 0; a < 3; a++) d.lv[l - first].opw[a] = take(sizeof(T) * (size_t)nf[a]);
    }
    for (int l = first + 1; l < nl; l++) {
        const int nf[3] = {lv[l - 1].nx, lv[l - 1].ny, lv[l - 1].nz}, nc[3] = {lv[l].nx, lv[l].ny, lv[l].nz};
        for (int a = 0; a < 3; a++) {
            d.lv[l - first].opo[a] = take(sizeof(int) * (size_t)nf[a]);
            d.lv[l - first].opa[a] = take(sizeof(int) * (size_t)nf[a]);
            d.lv[l - first].och[a] = take(sizeof(int) * (size_t)(nc[a] + 1));
        }
    }
    img.assign((off + 15) & ~(size_t)15, 0);
    d.words16 = (int)(img.size() / 16);
    auto fetch = [&](int at, const void *src, size_t bytes) {
        return cudaMemcpy(img.data() + at, src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess;
    };
    bool ok = true;
    for (int l = first; l < nl; l++) {
        const TailLevel &t = d.lv[l - first];
        const MGLevel<T> &L = lv[l];
        const size_t b = sizeof(T) * (size_t)L.n;
        ok = ok && fetch(t.off[0], L.Tx, b) && fetch(t.off[1], L.Ty, b) && fetch(t.off[2], L.Tz, b) &&
             fetch(t.off[3], L.diag, b) && fetch(t.off[6], L.idiag, b);   // R, Z stay zero
    }
    for (int l = first + 1; l < nl; l++) {
        const TailLevel &t = d.lv[l - first];
        const int nf[3] = {lv[l - 1].nx, lv[l - 1].ny, lv[l - 1].nz}, nc[3] = {lv[l].nx, lv[l].ny, lv[l].nz};
        for (int a = 0; a < 3; a++) {
            ok = ok && fetch(t.opw[a], lv[l].pw[a], sizeof(T) * (size_t)nf[a]) &&
                 fetch(t.opo[a], lv[l].po[a], sizeof(int) * (size_t)nf[a]) &&
                 fetch(t.opa[a], lv[l].pa[a], sizeof(int) * (size_t)nf[a]) &&
                 fetch(t.och[a], lv[l].ch[a], sizeof(int) * (size_t)(nc[a] + 1));
        }
    }
    d.R_first = lv[first].R;
    d.Z_first = lv[first].Z;
    return ok ? 0 : -1;
}

// ------------------------------------------------------------- host --
// Groups of one axis of a new level: the first finer cell of each coarse
// cell, then nf.  Halving: pairs (0, 1), (2, 3), ... (an odd last cell
// alone; a one-cell axis stays).
static std::vector<int> halve_groups(int nf) {
    std::vector<int> ch;
    for (int i = 0; i < nf; i += nf >= 2 ? 2 : 1) ch.push_back(i);
    ch.push_back(nf);
    return ch;
}

// By spacing: from the low end, a cell and its neighbour merge when their
// joint width is at most H (finer faces ff).
static std::vector<int> spacing_groups(const std::vector<double> &ff, double H) {
    const int nf = (int)ff.size() - 1;
    std::vector<int> ch;
    int i = 0;
    while (i < nf) {
        ch.push_back(i);
        i += (i + 1 < nf && ff[i + 2] - ff[i] <= H) ? 2 : 1;
    }
    ch.push_back(nf);
    return ch;
}

// Centre-distance ratios of one axis (FaceRatio) for groups ch of the
// finer faces ff.
static std::vector<double> face_ratios(const std::vector<double> &ff, const std::vector<int> &ch, bool periodic) {
    const int nf = (int)ff.size() - 1, nc = (int)ch.size() - 1;
    std::vector<double> xf(nf), xc(nc), r(nc + 1, 1.0);
    for (int i = 0; i < nf; i++) xf[i] = 0.5 * (ff[i] + ff[i + 1]);
    for (int I = 0; I < nc; I++) xc[I] = 0.5 * (ff[ch[I]] + ff[ch[I + 1]]);
    for (int I = 1; I < nc; I++) r[I] = (xf[ch[I]] - xf[ch[I] - 1]) / (xc[I] - xc[I - 1]);
    if (periodic) {
        const double Lp = ff[nf] - ff[0];
        if (nc > 1) r[0] = r[nc] = (xf[0] + Lp - xf[nf - 1]) / (xc[0] + Lp - xc[nc - 1]);
    } else {
        r[0] = (xf[0] - ff[0]) / (xc[0] - ff[0]);
        r[nc] = (ff[nf] - xf[nf - 1]) / (ff[nf] - xc[nc - 1]);
    }
    return r;
}

// Prolongation tables of one axis: fine centres (fine faces ff, nf cells)
// into coarse centres (coarse faces cf, nc cells); pa: the coarse cell
// covering each fine cell.  A fine cell alone in its group shares its
// parent's centre (weight 1).
static void prolong_axis(const std::vector<double> &ff, const std::vector<double> &cf, const std::vector<int> &pa,
                         bool periodic, std::vector<int> &po, std::vector<double> &pw) {
    const int nf = (int)ff.size() - 1, nc = (int)cf.size() - 1;
    po.assign(nf, -1);
    pw.assign(nf, 1.0);
    if (nc == nf) return;
    std::vector<double> cc(nc);
    for (int I = 0; I < nc; I++) cc[I] = 0.5 * (cf[I] + cf[I + 1]);
    const double Lp = cf[nc] - cf[0];
    for (int i = 0; i < nf; i++) {
        const double x = 0.5 * (ff[i] + ff[i + 1]);
        const int I = pa[i];
        int o = x < cc[I] ? I - 1 : I + 1;
        double co;
        if (o < 0 || o >= nc) {
            if (!periodic || nc < 2) continue;
            if (o < 0) {
                o = nc - 1;
                co = cc[nc - 1] - Lp;
            } else {
                o = 0;
                co = cc[0] + Lp;
            }
        } else {
            co = cc[o];
        }
        po[i] = o;
        pw[i] = (x - co) / (cc[I] - co);
    }
}

template <typename T>
GMG<T>::~GMG() {
    for (void *p : allocs_) cudaFree(p);
}

template <typename T>
int GMG<T>::setup(cudaStream_t s, const OpT<double> &A64, const OpT<T> &A, const int *ghost_cell, int nghost,
                  const MGGeometry &geom, const GMGConfig &cfg) {
    A_ = A;
    cfg_ = cfg;
    ghost_cell_ = ghost_cell;
    nghost_ = nghost;
    const Grid &g = A.g;
    per_[0] = A.bc[F_W].type == BCT_PERIODIC;
    per_[1] = A.bc[F_S].type == BCT_PERIODIC;
    per_[2] = A.bc[F_D].type == BCT_PERIODIC;
    // Colour-split fine rows for FP32 cycles on grids without a seam.
    const bool seam = (per_[0] && (g.nx & 1)) || (per_[1] && (g.ny & 1)) || (per_[2] && (g.nz & 1));
    NZH_ = (g.nz + 5) / 2;
    H_ = (long long)(g.nx + 4) * (g.ny + 4) * NZH_;
    split_ = sizeof(T) == 4 && !seam && 2 * H_ < (1LL << 31);
    std::vector<void *> tmp;
    auto dalloc = [&](size_t bytes, bool keep) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        cudaMemsetAsync(p, 0, bytes ? bytes : 16, s);
        (keep ? allocs_ : tmp).push_back(p);
        return p;
    };
    if (nghost > 0) ghost_tmp_ = (T *)dalloc(sizeof(T) * nghost, true);
    if (split_) {
        rs_ = (T *)dalloc(sizeof(T) * 2 * H_, true);
        ds_ = (T *)dalloc(sizeof(T) * 2 * H_, true);
        fs_ = (uint8_t *)dalloc(2 * H_, true);
        if (!rs_ || !ds_ || !fs_) return -1;
        const dim3 gs((g.nz + 35) / 32, (g.ny + 11) / 8, g.nx + 4);
        k_to_split<T, T><<<gs, dim3(32, 8), 0, s>>>(A.dinv, ds_, g.ny + 4, g.nz + 4, NZH_, H_, nullptr);
        k_to_split<uint8_t, uint8_t><<<gs, dim3(32, 8), 0, s>>>(A.flag, fs_, g.ny + 4, g.nz + 4, NZH_, H_, nullptr);
    }
    // Does any ghost interpolation stencil reach an outer cell?  Then the
    // ghost and outer rows of a sweep cannot share a launch.
    {
        std::vector<int> o1;
        for (int i = -1; i <= g.nx; i++)
            for (int j = -1; j <= g.ny; j++)
                for (int k = -1; k <= g.nz; k++) {
                    const int out = (i < 0 || i >= g.nx) + (j < 0 || j >= g.ny) + (k < 0 || k >= g.nz);
                    if (out == 1) o1.push_back((int)cidx(g, i, j, k));
                }
        nout1_ = (int)o1.size();
        outer1_ = (int *)dalloc(sizeof(int) * std::max<size_t>(1, o1.size()), true);
        if (!outer1_) return -1;
        if (!o1.empty())  // after dalloc's clearing, on the same stream (pageable source: staged at the call)
            cudaMemcpyAsync(outer1_, o1.data(), sizeof(int) * o1.size(), cudaMemcpyHostToDevice, s);
    }
    ghost_reads_outer_ = false;
    if (nghost > 0) {
        std::vector<int> gidx(8 * (size_t)nghost), gcell(nghost);
        std::vector<double> gw(8 * (size_t)nghost), gws(nghost);
        cudaMemcpy(gidx.data(), A.gidx, sizeof(int) * gidx.size(), cudaMemcpyDeviceToHost);
        cudaMemcpy(gcell.data(), ghost_cell, sizeof(int) * nghost, cudaMemcpyDeviceToHost);
        // Each ghost's row in the fine-row layout in use.
        {
            const FineRows<T> fr{nullptr, nullptr, nullptr, split_ ? 1 : 0, H_, g.ny + 4, NZH_,
                                 (long long)(g.ny + 4) * NZH_};
            std::vector<long long> grow(nghost);
            for (int t = 0; t < nghost; t++) {
                int i, j, k;
                cijk(g, gcell[t], i, j, k);
                grow[t] = fr.at(gcell[t], i, j, k);
            }
            grow_ = (long long *)dalloc(sizeof(long long) * nghost, true);
            if (!grow_) return -1;
            // After dalloc's clearing, on the same stream (pageable source: staged at the call).
            cudaMemcpyAsync(grow_, grow.data(), sizeof(long long) * nghost, cudaMemcpyHostToDevice, s);
        }
        cudaMemcpy(gw.data(), A64.gw, sizeof(double) * gw.size(), cudaMemcpyDeviceToHost);
        cudaMemcpy(gws.data(), A64.gwself, sizeof(double) * nghost, cudaMemcpyDeviceToHost);
        for (int q : gidx) {
            if (q < 0) continue;
            int i, j, k;
            cijk(g, q, i, j, k);
            if (i < 0 || i >= g.nx || j < 0 || j >= g.ny || k < 0 || k >= g.nz) ghost_reads_outer_ = true;
        }
        // Inverse divisors of the ghost relaxation (ghost_value), per
        // ghost id (ghost id t is the ghost at padded cell gcell[t]).
        std::vector<int> sorted(gcell);
        std::sort(sorted.begin(), sorted.end());
        std::vector<T> idiv(nghost);
        for (int t = 0; t < nghost; t++) {
            double wgg = 0.0;
            for (int e = 0; e < 8; e++) {
                const int q = gidx[8 * (size_t)t + e];
                if (q >= 0 && q != gcell[t] && std::binary_search(sorted.begin(), sorted.end(), q))
                    wgg += std::fabs(gw[8 * (size_t)t + e]);
            }
            idiv[t] = (T)(1.0 / std::max({1.0 - gws[t], 2.0 * wgg, 1e-3}));
        }
        ghost_idiv_ = (T *)dalloc(sizeof(T) * nghost, true);
        if (!ghost_idiv_) return -1;
        cudaMemcpyAsync(ghost_idiv_, idiv.data(), sizeof(T) * nghost, cudaMemcpyHostToDevice, s);
    }

    Per3 per{{per_[0], per_[1], per_[2]}};
    int nx = g.nx, ny = g.ny, nz = g.nz;
    std::vector<double> faces[3] = {geom.f[0], geom.f[1], geom.f[2]};
    std::vector<MGLevel<double>> lv64;
    std::vector<double *> G;
    // Host tables are copied by cudaMemcpyAsync from pageable memory, which
    // stages them at the call: the vectors may go out of scope after it.
    auto upload = [&](const void *src, size_t bytes, bool keep) -> void * {
        void *p = dalloc(bytes, keep);
        if (p && bytes) cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, s);
        return p;
    };
    // Finest width of the grid over the axes that can coarsen.
    double hmin0 = 0.0;
    for (int a = 0; a < 3; a++) {
        if (geom.f[a].size() < 3) continue;
        for (size_t i = 0; i + 1 < geom.f[a].size(); i++) {
            const double w = geom.f[a][i + 1] - geom.f[a][i];
            if (hmin0 == 0.0 || w < hmin0) hmin0 = w;
        }
    }
    for (int level = 0;; level++) {
        const int fn[3] = {nx, ny, nz};
        if (nx < 2 && ny < 2 && nz < 2) break;
        if ((long long)nx * ny * nz <= 64 && !lv64.empty()) break;
        std::vector<int> ch[3];
        for (int a = 0; a < 3; a++) ch[a] = halve_groups(fn[a]);
        if (cfg.coarsening == MG_COARSEN_SPACING) {
            // Widest pair on any axis: at that threshold every pair merges.
            double hmax = 0.0;
            for (int a = 0; a < 3; a++)
                for (int i = 0; i + 2 < (int)faces[a].size(); i++) hmax = std::max(hmax, faces[a][i + 2] - faces[a][i]);
            const long long nfine = (long long)nx * ny * nz;
            for (double H = cfg.width_ratio * std::ldexp(hmin0, level + 1);; H *= 1.25) {
                long long m = 1;
                for (int a = 0; a < 3; a++) {
                    ch[a] = spacing_groups(faces[a], H);
                    m *= (long long)ch[a].size() - 1;
                }
                if (2 * m <= nfine || H >= hmax) break;
            }
        }
        MGLevel<double> L{};
        L.cx = nx >= 2 && ch[0] == halve_groups(nx);
        L.cy = ny >= 2 && ch[1] == halve_groups(ny);
        L.cz = nz >= 2 && ch[2] == halve_groups(nz);
        L.nx = (int)ch[0].size() - 1;
        L.ny = (int)ch[1].size() - 1;
        L.nz = (int)ch[2].size() - 1;
        L.n = (long long)L.nx * L.ny * L.nz;
        if (L.n == nx * (long long)ny * nz) break;  // nothing merges
        const int cn[3] = {L.nx, L.ny, L.nz};
        MGLevel<T> LT{};
        LT.nx = L.nx; LT.ny = L.ny; LT.nz = L.nz; LT.n = L.n; LT.cx = L.cx; LT.cy = L.cy; LT.cz = L.cz;
        std::vector<double> cfs[3];
        FaceRatio fr{};
        for (int a = 0; a < 3; a++) {
            std::vector<int> pa(fn[a]);
            for (int I = 0; I < cn[a]; I++)
                for (int i = ch[a][I]; i < ch[a][I + 1]; i++) pa[i] = I;
            std::vector<double> &cf = cfs[a];
            cf.resize(cn[a] + 1);
            for (int I = 0; I <= cn[a]; I++) cf[I] = faces[a][ch[a][I]];
            const std::vector<double> rat = face_ratios(faces[a], ch[a], per_[a]);
            std::vector<int> po;
            std::vector<double> pw;
            prolong_axis(faces[a], cf, pa, per_[a], po, pw);
            std::vector<T> pwt(pw.begin(), pw.end());
            const int *dch = (const int *)upload(ch[a].data(), sizeof(int) * ch[a].size(), true);
            const int *dpa = (const int *)upload(pa.data(), sizeof(int) * pa.size(), true);
            const int *dpo = (const int *)upload(po.data(), sizeof(int) * po.size(), true);
            const T *dpw = (const T *)upload(pwt.data(), sizeof(T) * pwt.size(), true);
            fr.r[a] = (const double *)upload(rat.data(), sizeof(double) * rat.size(), false);
            if (!dch || !dpa || !dpo || !dpw || !fr.r[a]) return -1;
            L.ch[a] = LT.ch[a] = dch;
            L.pa[a] = LT.pa[a] = dpa;
            LT.po[a] = dpo;
            LT.pw[a] = dpw;
        }
        const size_t b = sizeof(double) * L.n;
        L.Tx = (double *)dalloc(b, false); L.Ty = (double *)dalloc(b, false); L.Tz = (double *)dalloc(b, false);
        L.diag = (double *)dalloc(b, false);
        double *gx = (double *)dalloc(b, false), *gy = (double *)dalloc(b, false), *gz = (double *)dalloc(b, false);
        if (!L.Tx || !L.Ty || !L.Tz || !L.diag || !gx || !gy || !gz) return -1;
        if (lv64.empty()) {
            k_mg_build1<<<nblk(L.n, 128), 128, 0, s>>>(A64, L, gx, gy, gz, per, fr);
        } else {
            double **fg = &G[G.size() - 3];
            k_mg_buildc<<<nblk(L.n, 128), 128, 0, s>>>(lv64.back(), fg[0], fg[1], fg[2], L, gx, gy, gz, fr);
        }
        k_mg_diag<<<nblk(L.n, 128), 128, 0, s>>>(L, gx, gy, gz, per);
        G.push_back(gx); G.push_back(gy); G.push_back(gz);
        for (int a = 0; a < 3; a++) faces[a] = cfs[a];
        if (lv64.empty())
            for (int a = 0; a < 3; a++) ch1_[a] = ch[a];
        const size_t bt = sizeof(T) * L.n;
        LT.Tx = (T *)dalloc(bt, true); LT.Ty = (T *)dalloc(bt, true); LT.Tz = (T *)dalloc(bt, true);
        LT.diag = (T *)dalloc(bt, true); LT.R = (T *)dalloc(bt, true); LT.Z = (T *)dalloc(bt, true);
        LT.idiag = (T *)dalloc(bt, true);
        if (!LT.Tx || !LT.Ty || !LT.Tz || !LT.diag || !LT.R || !LT.Z || !LT.idiag) return -1;
        k_inverse<T><<<nblk(L.n, 256), 256, 0, s>>>(L.diag, LT.idiag, L.n);
        k_convert<T><<<nblk(L.n, 256), 256, 0, s>>>(L.Tx, LT.Tx, L.n);
        k_convert<T><<<nblk(L.n, 256), 256, 0, s>>>(L.Ty, LT.Ty, L.n);
        k_convert<T><<<nblk(L.n, 256), 256, 0, s>>>(L.Tz, LT.Tz, L.n);
        k_convert<T><<<nblk(L.n, 256), 256, 0, s>>>(L.diag, LT.diag, L.n);
        lv64.push_back(L);
        levels_.push_back(LT);
        nx = L.nx; ny = L.ny; nz = L.nz;
        if (L.n <= 64) break;
    }
    // Tiles of the restriction into level 1 (k_mg0_restrict_g): coarse
    // ranges covering at most 8 fine rows (j) and 32 fine columns (k).
    if (!lv64.empty()) {
        auto cut = [](const std::vector<int> &chv, int width) {
            std::vector<int> seg{0};
            const int nc = (int)chv.size() - 1;
            for (int K = 0; K < nc;) {
                int K1 = K + 1;
                while (K1 < nc && chv[K1 + 1] - chv[K] <= width) K1++;
                seg.push_back(K1);
                K = K1;
            }
            return seg;
        };
        const std::vector<int> sj = cut(ch1_[1], 8), sk = cut(ch1_[2], 32);
        nsegj_ = (int)sj.size() - 1;
        nsegk_ = (int)sk.size() - 1;
        segj_ = (int *)upload(sj.data(), sizeof(int) * sj.size(), true);
        segk_ = (int *)upload(sk.data(), sizeof(int) * sk.size(), true);
        if (!segj_ || !segk_) return -1;
    }
    // The coarsest levels with at most TAIL_THREADS cells each run in the tail.
    tail_ = (int)levels_.size() - 1;
    while (tail_ > 0 && levels_[tail_ - 1].n <= TAIL_CELLS && (int)levels_.size() - (tail_ - 1) <= 16 &&
           tail_bytes(levels_, tail_ - 1) <= TAIL_SMEM_MAX)
        tail_--;
    if (!levels_.empty()) {
        if (levels_[tail_].n > TAIL_CELLS) return -1;  // the tail takes one cell per thread
        tail_smem_ = tail_bytes(levels_, tail_);
        // The limit is a property of the kernel, shared by every solver in
        // the process: only ever raise it.
        cudaFuncAttributes fa{};
        if (cudaFuncGetAttributes(&fa, k_mg_tail<T>) != cudaSuccess) return -1;
        if ((size_t)fa.maxDynamicSharedSizeBytes < tail_smem_ &&
            cudaFuncSetAttribute(k_mg_tail<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tail_smem_) !=
                cudaSuccess)
            return -1;
    }
    if (!levels_.empty()) {
        if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
        std::vector<unsigned char> img;
        if (build_tail_image(levels_, tail_, tail_desc_, img) != 0) return -1;
        tail_img_ = (const uint4 *)upload(img.data(), img.size(), true);
        if (!tail_img_) return -1;
    }
    const bool ok = cudaStreamSynchronize(s) == cudaSuccess;
    for (void *p : tmp) cudaFree(p);
    return ok ? 0 : -1;
}

// Grid of a coarse colour pass (k pairs without a seam).
template <typename T>
static dim3 cgrid(const MGLevel<T> &L, int ncol) {
    const int kw = ncol == 2 ? 2 * L3_TK : L3_TK;
    return dim3((unsigned)((L.nz + kw - 1) / kw), (unsigned)((L.ny + L3_TJ - 1) / L3_TJ), (unsigned)L.nx);
}

template <typename T>
int GMG<T>::smooth0(cudaStream_t s, const FineRows<T> &fr, T *z, int sweeps, bool from_zero, const int *gate) {
    const Grid &g = A_.g;
    Per3 per{{per_[0], per_[1], per_[2]}};
    const bool seam = (per_[0] && (g.nx & 1)) || (per_[1] && (g.ny & 1)) || (per_[2] && (g.nz & 1));
    const dim3 blk(32, 8, 1);
    const dim3 grd(seam ? (g.nz + 31) / 32 : (g.nz + 63) / 64, (g.ny + 7) / 8, (g.nx + MG0_PLANES - 1) / MG0_PLANES);
    int k = 0;
    auto tb = [&](const char *nm) { return prof_ ? prof_->begin(nm) : -1; };
    auto te = [&](int t) {
        if (prof_) prof_->end(t);
    };
    for (int it = 0; it < sweeps; it++) {
        const int tc = tb("mg0_color");
        if (it == 0 && from_zero && !seam && !ghost_reads_outer_) {
            launch_pdl(fr.split ? k_mg0_first<T, true> : k_mg0_first<T, false>, grd, blk, 0, s, A_, fr, z, (T)cfg_.omega,
                       gate);
            k++;
        } else {
            for (int col = 0; col < (seam ? 4 : 2); col++, k++) {
                if (it == 0 && col == 0 && from_zero)
                    launch_pdl(fr.split ? k_mg0_init3<T, true> : k_mg0_init3<T, false>,
                               dim3((g.nz + 35) / 32, (g.ny + 11) / 8, (g.nx + 3 + MG0_IPLANES) / MG0_IPLANES),
                               dim3(32, 8), 0, s, A_, fr, z, per, gate);
                else
                    launch_pdl(fr.split ? k_mg0_color<T, true> : k_mg0_color<T, false>, grd, blk, 0, s, A_, fr, z,
                               col, seam ? 0 : 1, per, (T)cfg_.omega, gate);
            }
        }
        te(tc);
        const int to = tb("mg0_outer_ghost");
        const int gb = (nghost_ + 255) / 256, ob = (A_.sw.nout + 255) / 256;
        if (!ghost_reads_outer_) {
            // Before the last sweep only the layer-1 face cells (read by the
            // next colour pass); after it every outer cell.
            const bool last = it == sweeps - 1;
            const int *ol = last ? A_.sw.outer : outer1_;
            const int no = last ? A_.sw.nout : nout1_;
            launch_pdl(k_mg0_outer<T>, gb + (no + 255) / 256, 256, 0, s, A_, fr, z, ol, no, ghost_cell_,
                       (const long long *)grow_, nghost_, gb, ghost_tmp_, (const T *)ghost_idiv_, gate);
            k++;
        } else {  // a ghost stencil reaches an outer cell: ghosts first, outer rows after the scatter
            launch_pdl(k_mg0_outer<T>, gb, 256, 0, s, A_, fr, z, A_.sw.outer, 0, ghost_cell_, (const long long *)grow_,
                       nghost_, gb, ghost_tmp_, (const T *)ghost_idiv_, gate);
            k++;
        }
        if (nghost_ > 0) {
            launch_pdl(k_mg0_ghost_scatter<T>, nblk(nghost_, 128), 128, 0, s, ghost_cell_, nghost_, ghost_tmp_, z, gate);
            k++;
        }
        if (ghost_reads_outer_) {
            launch_pdl(k_mg0_outer<T>, ob, 256, 0, s, A_, fr, z, A_.sw.outer, A_.sw.nout, ghost_cell_,
                       (const long long *)grow_, 0, 0, ghost_tmp_, (const T *)ghost_idiv_, gate);
            k++;
        }
        te(to);
    }
    return k;
}

// The fine rows of an application with right-hand side r: r itself and
// the operator's 1/coeffsum and flags, or their colour-split copies (r
// split by the caller into rs_).
template <typename T>
FineRows<T> GMG<T>::rows(const T *r) const {
    const Grid &g = A_.g;
    if (split_) return FineRows<T>{rs_, ds_, fs_, 1, H_, g.ny + 4, NZH_, (long long)(g.ny + 4) * NZH_};
    return FineRows<T>{r, A_.dinv, A_.flag, 0, 0, g.ny + 4, 0, 0};
}

template <typename T>
void GMG<T>::apply(cudaStream_t s, const T *r, T *z, const int *gate) {
    if constexpr (sizeof(T) == 4) {
        if (split_) {
            const Grid &g = A_.g;
            launch_pdl(k_narrow_split<float>,
                       dim3((NZH_ + 31) / 32, (g.ny + 11) / 8, (g.nx + 3 + MG0_NPLANES) / MG0_NPLANES), dim3(32, 8), 0,
                       s, r, rs_, g.nx + 4, g.ny + 4, g.nz + 4, NZH_, H_, gate);
            note_launches(1);
            cycle(s, rows(r), z, gate);
            launches_++;
            return;
        }
    }
    cycle(s, rows(r), z, gate);
}

template <typename T>
bool GMG<T>::apply_from64(cudaStream_t s, const double *r, T *z, const int *gate) {
    if constexpr (sizeof(T) != 4) {
        return false;   // FP64 cycles keep the natural layout
    } else {
        if (!split_) return false;
        const Grid &g = A_.g;
        launch_pdl(k_narrow_split<double>, dim3((NZH_ + 31) / 32, (g.ny + 11) / 8, (g.nx + 3 + MG0_NPLANES) / MG0_NPLANES),
                   dim3(32, 8), 0, s, r, rs_, g.nx + 4, g.ny + 4, g.nz + 4, NZH_, H_, gate);
        note_launches(1);
        cycle(s, rows(nullptr), z, gate);
        launches_++;
        return true;
    }
}

template <typename T>
bool GMG<T>::apply_from_df(cudaStream_t s, const dfloat *r, T *z, const int *gate) {
    if constexpr (sizeof(T) != 4) {
        return false;
    } else {
        if (!split_) return false;
        const Grid &g = A_.g;
        launch_pdl(k_narrow_split<dfloat>, dim3((NZH_ + 31) / 32, (g.ny + 11) / 8, (g.nx + 3 + MG0_NPLANES) / MG0_NPLANES),
                   dim3(32, 8), 0, s, r, rs_, g.nx + 4, g.ny + 4, g.nz + 4, NZH_, H_, gate);
        note_launches(1);
        cycle(s, rows(nullptr), z, gate);
        launches_++;
        return true;
    }
}

// One V-cycle from z = 0: pre-smoothing on the fine rows, restriction, the
// coarse levels above the tail (each starting from Z = 0), the tail, then
// prolongation and post-smoothing back up.
template <typename T>
void GMG<T>::cycle(cudaStream_t s, const FineRows<T> &fr, T *z, const int *gate) {
    const Grid &g = A_.g;
    int k = 0;
    if (levels_.empty()) {
        k += smooth0(s, fr, z, cfg_.nu_pre + cfg_.nu_post + 4, true, gate);
        note_launches(k);
        launches_ = k;
        return;
    }
    Per3 per{{per_[0], per_[1], per_[2]}};
    auto tb = [&](const char *nm) { return prof_ ? prof_->begin(nm) : -1; };
    auto te = [&](int t) {
        if (prof_) prof_->end(t);
    };
    if (cfg_.nu_pre == 0) {   // no pre-smoothing: the cycle restricts r itself (z = 0)
        launch_pdl(k_fill0<T>, nblk(g.ncell, 256), 256, 0, s, z, (long long)g.ncell, gate);
        k++;
    }
    k += smooth0(s, fr, z, cfg_.nu_pre, true, gate);
    const MGLevel<T> &L1 = levels_[0];
    // The restriction into a coarse level above the tail also applies its
    // first colour pass (Z = R / diag on colour 0), so the level's own init
    // launch is left out.
    const int init1 = cfg_.nuc_pre > 0 && tail_ > 0 ? 1 : 0;
    int tp = tb("mg0_restrict");
    if (L1.cx && L1.cy && L1.cz)
        launch_pdl(fr.split ? k_mg0_restrict2<T, true> : k_mg0_restrict2<T, false>,
                   dim3((g.nz + 31) / 32, (g.ny + 7) / 8, L1.nx), dim3(32, 8), 0, s, A_, fr, z, L1, per, init1, gate);
    else
        launch_pdl(fr.split ? k_mg0_restrict_g<T, true> : k_mg0_restrict_g<T, false>,
                   dim3(nsegk_, nsegj_, (L1.nx + MG0_RPLANES - 1) / MG0_RPLANES), dim3(32, 8), 0, s, A_, fr, z, L1,
                   (const int *)segj_, (const int *)segk_, per, init1, gate);
    k++;
    te(tp);
    tp = tb("mgc_down");
    for (int l = 0; l < tail_; l++) {
        MGLevel<T> &L = levels_[l];
        const MGLevel<T> &C = levels_[l + 1];
        const int ncol = level_colors(L, per_);
        for (int it = 0; it < cfg_.nuc_pre; it++)
            for (int col = it == 0 ? 1 : 0; col < ncol; col++, k++)   // colour 0 of the first sweep: the restriction
                launch_pdl(k_mgc_color<T>, cgrid(L, ncol), l3_block(), 0, s, L, col, ncol == 2, per, gate);
        if (cfg_.nuc_pre == 0) {
            launch_pdl(k_fill0<T>, nblk(L.n, 256), 256, 0, s, L.Z, L.n, gate);
            k++;
        }
        // After a red/black pre-smoothing the last colour's residuals are 0.
        const int skip = cfg_.nuc_pre > 0 && ncol == 2 ? 1 : -1;
        launch_pdl(k_mgc_restrict<T>, l3_grid(C.nx, C.ny, C.nz), l3_block(), 0, s, L, C, per, skip,
                   cfg_.nuc_pre > 0 && l + 1 < tail_ ? 1 : 0, gate);
        k++;
    }
    te(tp);
    tp = tb("mg_tail");
    launch_pdl(k_mg_tail<T>, 1, TAIL_THREADS, tail_smem_, s, tail_desc_, tail_img_, cfg_.nuc_pre, cfg_.nuc_post,
               cfg_.coarse_sweeps, per, A_.p_singular ? 1 : 0, gate);
    k++;
    te(tp);
    tp = tb("mgc_up");
    for (int l = tail_ - 1; l >= 0; l--) {
        MGLevel<T> &L = levels_[l];
        const int ncol = level_colors(L, per_);
        launch_pdl(k_mgc_prolong<T>, l3_grid(L.nx, L.ny, L.nz), l3_block(), 0, s, levels_[l + 1], L, gate);
        k++;
        for (int it = 0; it < cfg_.nuc_post; it++)
            for (int col = 0; col < ncol; col++, k++)
                launch_pdl(k_mgc_color<T>, cgrid(L, ncol), l3_block(), 0, s, L, col, ncol == 2, per, gate);
    }
    te(tp);
    tp = tb("mg0_prolong");
    if (L1.cx && L1.cy && L1.cz)
        launch_pdl(k_mg0_prolong2<T>, l3_grid(g.nx, g.ny, g.nz), l3_block(), 0, s, A_, z, L1, gate);
    else
        launch_pdl(k_mg0_prolong<T>,
                   dim3((g.nz + 31) / 32, (g.ny + 7) / 8, (g.nx + mg0_pplanes<T>() - 1) / mg0_pplanes<T>()), dim3(32, 8), 0,
                   s, A_, z, L1, gate);
    k++;
    te(tp);
    k += smooth0(s, fr, z, cfg_.nu_post, false, gate);
    note_launches(k);
    launches_ = k;
}

template <typename T>
float GMG<T>::time_color(cudaStream_t s, const T *r, T *z, int reps, double *bytes, bool timed) {
    const Grid &g = A_.g;
    Per3 per{{per_[0], per_[1], per_[2]}};
    const bool seam = (per_[0] && (g.nx & 1)) || (per_[1] && (g.ny & 1)) || (per_[2] && (g.nz & 1));
    const dim3 blk(32, 8, 1);
    const dim3 grd(seam ? (g.nz + 31) / 32 : (g.nz + 63) / 64, (g.ny + 7) / 8, (g.nx + MG0_PLANES - 1) / MG0_PLANES);
    void (*color)(const OpT<T>, const FineRows<T>, T *, int, int, Per3, T, const int *) =
        split_ ? k_mg0_color<T, true> : k_mg0_color<T, false>;
    const double nint = (double)g.nx * g.ny * g.nz;
    *bytes = nint * sizeof(T) + 0.5 * nint * (3 * sizeof(T) + 1);
    if (!timed) {
        for (int q = 0; q < reps; q++)
            color<<<grd, blk, 0, s>>>(A_, rows(r), z, 1, seam ? 0 : 1, per, (T)cfg_.omega, nullptr);
        note_launches(reps);
        return 0.0f;
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    for (int q = 0; q < reps; q++)
        color<<<grd, blk, 0, s>>>(A_, rows(r), z, 1, seam ? 0 : 1, per, (T)cfg_.omega, nullptr);
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    note_launches(reps);
    return reps > 0 ? ms / reps : 0.0f;
}

template class GMG<double>;
template class GMG<float>;

}  // namespace ibm
