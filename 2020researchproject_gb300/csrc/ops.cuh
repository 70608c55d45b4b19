// Matrix-free rows of the momentum and pressure systems, in FP64 or FP32.
//
// The rows restate the matrices the reference assembles for hypre
// (create_matrix, src/ibm3d_setup.c:1566-2908):
//   fluid  : Crank-Nicolson Helmholtz (1 + sum k) x_P - sum k_nb x_nb    (type 1..3)
//            normalised Poisson      x_P - sum (k_nb / sum k) x_nb       (type 4)
//   ghost  : interpolation rows (1 + w_self) x_g + sum w x  (momentum)
//                               (1 - w_self) x_g - sum w x  (pressure)
//   solid  : identity; pinned p'(0,0,0) when no face fixes the pressure
//   outer  : per face and layer: Dirichlet interpolation, Neumann copy,
//            periodic copy or 3-point extrapolation.
// OpT<double> is the exact FP64 operator; OpT<float> the same rows in FP32
// for the inner solves of the mixed-precision path.
#pragma once

#include "common.cuh"

namespace ibm {

enum { OP_MOM = 0, OP_PRES = 1 };
enum { ROW_DIR = 0, ROW_NEU = 1, ROW_PER = 2, ROW_EXT = 3 };

// ------------------------------------------------------------- sweeps --
// A sweep over the padded grid in one launch: interior cells in tiles of
// SW_TK (k) x SW_TJ (j) columns, each thread marching over `pi` planes of
// i, so a thread needs no index division; outer cells from a precomputed
// list.  Blocks [0, nint) are interior tiles, the rest take consecutive
// chunks of SW_THREADS outer cells.
constexpr int SW_TK = 32, SW_TJ = 8, SW_THREADS = 256;

struct SweepGeom {
    int tk, tj, ti;   // interior tiles per axis
    int pi;           // planes per tile
    int nint;         // interior tiles
    int nout;         // outer cells
    int nblocks;      // nint + outer chunks
    const int *outer; // padded index of every outer cell (device)
};

template <typename T>
struct BCRow {
    int type;
    T dir_o[2], dir_m[2];
    T ext_o[2], ext_2[2];
};

template <typename T>
struct OpT {
    Grid g;
    FastDiv fdx, fdy;       // divisions by sx and sy
    const T *km[3], *kp[3]; // Crank-Nicolson coefficients per axis (index i+2)
    const T *ks[3];         // km + kp per axis
    const T *d[3];          // cell widths per axis
    BCRow<T> bc[6];
    int p_singular;
    long long pinned;       // padded index of (0,0,0)
    const uint8_t *flag;
    const int *gid;         // padded index -> ghost id, -1 elsewhere
    const int *gidx;        // [8*g+e] padded index of a kept stencil entry, -1 otherwise
    const T *gw;            // [8*g+e] normalised weight
    const T *gwself;        // [g]
    const T *dinv;          // 1/coeffsum on fluid rows
    const float *wdiv;      // 2 Re coeffsum on fluid, non-pinned interior cells; 0 elsewhere
    SweepGeom sw;           // launch geometry of sweeps over the padded grid
};

__host__ __device__ inline int outer_row_kind(int op, int type, int comp, int axis) {
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

// x may hold entries of another type X (FP32 entries under double-float
// rows), converted to T as they are read.
template <typename T, typename X>
__device__ __forceinline__ T outer_row(const OpT<T> &c, int op, int comp, const X *__restrict__ x, long long P, int i,
                                       int j, int k, int f, int L) {
    const BCRow<T> &F = c.bc[f];
    const int axis = face_axis(f);
    const long long s = axis == 0 ? c.g.sx : axis == 1 ? c.g.sy : 1;
    const long long in = face_low(f) ? s : -s;
    switch (outer_row_kind(op, F.type, comp, axis)) {
    case ROW_DIR: return F.dir_o[L - 1] * T(x[P]) + F.dir_m[L - 1] * T(x[P + (2 * L - 1) * in]);
    case ROW_NEU: return T(x[P]) - T(x[P + (2 * L - 1) * in]);
    case ROW_PER: return T(x[P]) - T(x[periodic_image(c.g, i, j, k)]);
    default: return F.ext_o[L - 1] * T(x[P]) - T(x[P + in]) + F.ext_2[L - 1] * T(x[P + 2 * in]);
    }
}

// Interior column of this thread: planes [i0, i1) at (j, k); false for
// blocks of the outer part.  Threads past the grid get j >= ny or k >= nz.
__device__ __forceinline__ bool sweep_column(const SweepGeom &s, const Grid &g, int &i0, int &i1, int &j, int &k) {
    int b = blockIdx.x;
    if (b >= s.nint) return false;
    const int bk = b % s.tk;
    b /= s.tk;
    const int bj = b % s.tj;
    const int bi = b / s.tj;
    k = bk * SW_TK + (threadIdx.x & (SW_TK - 1));
    j = bj * SW_TJ + (threadIdx.x / SW_TK);
    i0 = bi * s.pi;
    i1 = min(i0 + s.pi, g.nx);
    return true;
}

// Outer-list position of this thread (blocks past the interior part).
__device__ __forceinline__ int sweep_outer(const SweepGeom &s) {
    return (blockIdx.x - s.nint) * SW_THREADS + threadIdx.x;
}

// Per-column stencil coefficients (constant along i).
template <typename T>
struct Column {
    T kmy, kpy, kmz, kpz, ksy, ksz;
};

template <typename T>
__device__ __forceinline__ Column<T> column(const OpT<T> &c, int j, int k) {
    Column<T> q;
    q.kmy = c.km[1][j + 2];
    q.kpy = c.kp[1][j + 2];
    q.kmz = c.km[2][k + 2];
    q.kpz = c.kp[2][k + 2];
    q.ksy = c.ks[1][j + 2];
    q.ksz = c.ks[2][k + 2];
    return q;
}

// Row of an interior cell (i, j, k) at padded index P: the same arithmetic
// as op_row without the index decode and the outer-face test, and
// branch-free for fluid, solid and pinned rows (every load issued up
// front, the result selected); ghost rows, a few per thousand, branch.
template <typename T, typename X>
__device__ __forceinline__ T interior_row(const OpT<T> &c, int op, const X *__restrict__ x, long long P, int i,
                                          const Column<T> &q) {
    const uint8_t fl = c.flag[P];
    const int I = i + 2;
    const long long sx = c.g.sx, sy = c.g.sy;
    const T xc = T(x[P]), xw = T(x[P - sx]), xe = T(x[P + sx]), xs = T(x[P - sy]), xn = T(x[P + sy]),
            xd = T(x[P - 1]), xu = T(x[P + 1]);
    const T nb = sum6(c.km[0][I], xw, c.kp[0][I], xe, q.kmy, xs, q.kpy, xn, q.kmz, xd, q.kpz, xu);
    T y;
    if (op == OP_MOM) y = ((T)1 + c.ks[0][I] + q.ksy + q.ksz) * xc - nb;
    else y = sub_mul(xc, c.dinv[P], nb);
    const bool pinned = op == OP_PRES && c.p_singular && P == c.pinned;
    if (fl != FLUID || pinned) y = xc;
    if (fl == GHOST && !pinned) {
        const int g = c.gid[P];
        T sum = 0;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int m = c.gidx[8 * g + e];
            if (m >= 0) sum += c.gw[8 * g + e] * T(x[m]);
        }
        const T ws = c.gwself[g];
        y = op == OP_MOM ? ((T)1 + ws) * xc + sum : ((T)1 - ws) * xc - sum;
    }
    return y;
}

// One row of A applied to x (op OP_MOM with component comp, or OP_PRES).
template <typename T, typename X>
__device__ __forceinline__ T op_row(const OpT<T> &c, int op, int comp, const X *__restrict__ x, long long P) {
    int i, j, k;
    cijk_fast(c.g, c.fdx, c.fdy, P, i, j, k);
    int L;
    const int f = owner_face(c.g, i, j, k, L);
    if (f >= 0) return outer_row(c, op, comp, x, P, i, j, k, f, L);
    if (op == OP_PRES && c.p_singular && P == c.pinned) return T(x[P]);
    const uint8_t fl = c.flag[P];
    if (fl == FLUID) {
        const int I = i + 2, J = j + 2, K = k + 2;
        const long long sx = c.g.sx, sy = c.g.sy;
        const T nb = c.km[0][I] * T(x[P - sx]) + c.kp[0][I] * T(x[P + sx]) + c.km[1][J] * T(x[P - sy]) +
                     c.kp[1][J] * T(x[P + sy]) + c.km[2][K] * T(x[P - 1]) + c.kp[2][K] * T(x[P + 1]);
        if (op == OP_MOM) return ((T)1 + c.ks[0][I] + c.ks[1][J] + c.ks[2][K]) * T(x[P]) - nb;
        return T(x[P]) - c.dinv[P] * nb;
    }
    if (fl == GHOST) {
        const int g = c.gid[P];
        T sum = 0;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int q = c.gidx[8 * g + e];
            if (q >= 0) sum += c.gw[8 * g + e] * T(x[q]);
        }
        const T ws = c.gwself[g];
        return op == OP_MOM ? ((T)1 + ws) * T(x[P]) + sum : ((T)1 - ws) * T(x[P]) - sum;
    }
    return T(x[P]);
}

}  // namespace ibm
