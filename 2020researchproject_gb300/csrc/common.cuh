// Shared device-side definitions of the GB300 immersed-boundary time step.
//
// Layout (identical to the reference, src/utils.h:8-16): every field lives
// on the padded cell grid (Nx+4)(Ny+4)(Nz+4), k fastest, interior cell
// (i,j,k) at ((i+2)*sx + (j+2)*sy + (k+2)).  Face fields use the same
// padded cell layout: the x-face between cells i-1 and i is stored at cell
// (i,j,k), so all fields share one index and one allocation size.  1-D
// metric arrays have N+4 entries indexed i+2 (the reference's c1e()).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ibm {

enum { FLUID = 1, GHOST = 2, SOLID = 3 };

// Boundary-condition types, values as in the reference (src/ibm3d.h:37-45).
enum { BCT_VELOCITY = 0, BCT_PRESSURE = 1, BCT_WALL = 2, BCT_SLIP = 3,
       BCT_SYMMETRIC = 4, BCT_PERIODIC = 5, BCT_VELPERIODIC = 6 };

// Face order of the reference's bc[] array: north, east, south, west, down, up.
enum { F_N = 0, F_E = 1, F_S = 2, F_W = 3, F_D = 4, F_U = 5 };

// Exact unsigned 32-bit division by a run-time constant d >= 1 with one
// multiply-high (Granlund & Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, round-up variant):
//   t = mulhi(m, n); q = (t + ((n - t) >> 1)) >> (l - 1).
struct FastDiv {
    uint32_t d, m;
    int l;
};

inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    int l = 0;
    while ((1ull << l) < d) l++;
    f.l = l;
    f.m = d == 1 ? 0u : (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    return f;
}

__device__ __forceinline__ uint32_t fdiv(const FastDiv &f, uint32_t n) {
    if (f.d == 1) return n;
    const uint32_t t = __umulhi(f.m, n);
    return (t + ((n - t) >> 1)) >> (f.l - 1);
}

struct Grid {
    int nx, ny, nz;
    long long sx, sy;   // strides of i and j (k stride is 1)
    long long ncell;    // (nx+4)(ny+4)(nz+4)
    // Fast dividers (set with the sizes by set_grid_dividers): padded
    // strides sx, sy and interior sizes nz, ny.
    FastDiv dsx, dsy, dnz, dny;
};

inline void set_grid_dividers(Grid &g) {
    g.dsx = make_fastdiv((uint32_t)g.sx);
    g.dsy = make_fastdiv((uint32_t)g.sy);
    g.dnz = make_fastdiv((uint32_t)g.nz);
    g.dny = make_fastdiv((uint32_t)g.ny);
}

__host__ __device__ inline long long cidx(const Grid &g, int i, int j, int k) {
    return (long long)(i + 2) * g.sx + (long long)(j + 2) * g.sy + (k + 2);
}

// Padded index -> (i, j, k) with the two divisions done by FastDiv
// (padded grids stay below 2^31 cells).
__device__ __forceinline__ void cijk_fast(const Grid &g, const FastDiv &dx, const FastDiv &dy, long long idx, int &i,
                                          int &j, int &k) {
    const uint32_t P = (uint32_t)idx;
    const uint32_t I = fdiv(dx, P);
    const uint32_t r = P - I * (uint32_t)g.sx;
    const uint32_t J = fdiv(dy, r);
    i = (int)I - 2;
    j = (int)J - 2;
    k = (int)(r - J * (uint32_t)g.sy) - 2;
}

// cijk_fast with the grid's own dividers.
__device__ __forceinline__ void cijk_g(const Grid &g, long long idx, int &i, int &j, int &k) {
    cijk_fast(g, g.dsx, g.dsy, idx, i, j, k);
}

// Interior index q (k fastest, then j, then i) -> (i, j, k).
__device__ __forceinline__ void ijk_interior(const Grid &g, long long q, int &i, int &j, int &k) {
    const uint32_t Q = (uint32_t)q;
    const uint32_t r = fdiv(g.dnz, Q);
    k = (int)(Q - r * (uint32_t)g.nz);
    const uint32_t I = fdiv(g.dny, r);
    j = (int)(r - I * (uint32_t)g.ny);
    i = (int)I;
}

__host__ __device__ inline void cijk(const Grid &g, long long idx, int &i, int &j, int &k) {
    i = (int)(idx / g.sx) - 2;
    long long r = idx - (long long)(i + 2) * g.sx;
    j = (int)(r / g.sy) - 2;
    k = (int)(r - (long long)(j + 2) * g.sy) - 2;
}

// ------------------------------------------------ FP64 <-> FP32 on INT --
// On GB300 the conversion instructions between FP64 and FP32 run at the
// FP64 rate (measured: one conversion costs about one FP64 FMA, ~1/70 of
// an FP32 FMA), so the FP32 stages of the mixed step convert with 32-bit
// integer operations on the IEEE-754 bit patterns instead.
//
// d2f_int: FP64 -> FP32, rounding to nearest with ties away from zero
// (the first discarded mantissa bit is added to the kept ones; a carry
// into the exponent is the correct next binade).  Magnitudes below the
// smallest normal float give a signed zero, above the largest float Inf;
// NaN stays NaN.
__device__ __forceinline__ float d2f_int(double x) {
    const int hi = __double2hiint(x);
    const unsigned lo = (unsigned)__double2loint(x);
    const unsigned sgn = (unsigned)hi & 0x80000000u;
    const int em = hi & 0x7fffffff;     // exponent and the top 20 mantissa bits
    const int t = em - (896 << 20);     // exponent bias 1023 -> 127
    unsigned r = __funnelshift_l(lo, (unsigned)t, 3) + ((lo >> 28) & 1u);
    if (t < (1 << 20)) r = 0u;
    if (t >= (255 << 20)) r = (em > 0x7ff00000 || (em == 0x7ff00000 && lo != 0u)) ? 0x7fc00000u : 0x7f800000u;
    return __uint_as_float(sgn | r);
}

// f2d_int: FP32 -> FP64, exact for normal floats, zero and Inf/NaN
// (subnormal floats become signed zero).
__device__ __forceinline__ double f2d_int(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned sgn = b & 0x80000000u, m = b & 0x7fffffffu;
    unsigned hi = sgn | ((m >> 3) + (896u << 20)), lo = m << 29;
    if (m < 0x00800000u) {
        hi = sgn;
        lo = 0u;
    } else if (m >= 0x7f800000u) {
        hi = sgn | 0x7ff00000u | ((m & 0x7fffffu) ? 0x80000u : 0u);
        lo = 0u;
    }
    return __hiloint2double((int)hi, (int)lo);
}

// ------------------------------------------------------- double-float --
// dfloat: the unevaluated sum hi + lo of two FP32 values with
// |lo| <= ulp(hi) / 2, a 48-bit significand with FP32's exponent range
// (magnitudes below ~1e-38 lose the low word).  Its operations are
// error-free transformations on the FP32 pipe: TwoSum (Knuth, TAOCP vol. 2,
// 4.2.2, Theorem B), FastTwoSum (Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971) and TwoProduct
// with one fused multiply-add, combined as in the double-double addition
// and multiplication of Hida, Li and Bailey ("Algorithms for quad-double
// precision floating point arithmetic", ARITH-15, 2001) with FP32 words.
// An add takes 20 FP32 operations and a multiply 7, against one FP64
// operation at 1/72 of the FP32 issue rate on this part, so FP64-bound
// vector kernels run several times faster on double-float vectors.  The
// _rn intrinsics keep the compiler from contracting the transformations
// into fused operations, which would break their exactness.
struct dfloat {
    float hi, lo;
    dfloat() = default;
    __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr dfloat(int v) : hi((float)v), lo(0.0f) {}
    __host__ __device__ constexpr dfloat(float v) : hi(v), lo(0.0f) {}
    // Nearest double-float of an FP64 value: hi = x rounded to FP32, lo = the
    // rest (x - hi is exact in FP64) rounded to FP32.  On the device both
    // roundings run on the integer pipe; the subtraction is one FP64 add.
    __host__ __device__ dfloat(double x) {
#ifdef __CUDA_ARCH__
        hi = d2f_int(x);
        lo = d2f_int(x - f2d_int(hi));
#else
        hi = (float)x;
        lo = (float)(x - (double)hi);
#endif
    }
    // hi + lo in FP64 (one FP64 add; exact when the two words' bits span at
    // most 53 places).
    __host__ __device__ explicit operator double() const {
#ifdef __CUDA_ARCH__
        return f2d_int(hi) + f2d_int(lo);
#else
        return (double)hi + (double)lo;
#endif
    }
};

__device__ __forceinline__ dfloat two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return dfloat(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
// |a| >= |b| (or a = 0).
__device__ __forceinline__ dfloat fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return dfloat(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
    const dfloat s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
    dfloat u = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat &operator-=(dfloat &a, dfloat b) { return a = a - b; }

// Lazy accumulation of a sum of products (Ogita, Rump and Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26, 2005, Algorithm Dot2, with
// double-float factors): acc.hi carries the FP32 running sum, acc.lo the
// FP32 sum of every rounding error of the products and additions and of the
// products' low-word terms, not renormalised between terms (the
// double-float addition that combines such sums accepts them as they are).
// 12 FP32 operations per term against 27 for a double-float multiply and
// add; its error, a few units of 2^-48 of the sum of the terms'
// magnitudes up to a factor of the number of terms, is larger than the
// chained operations', which the vector updates keep.
__device__ __forceinline__ void df_mac(dfloat &acc, dfloat a, dfloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const dfloat s = two_sum(acc.hi, p);
    acc.hi = s.hi;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, e));
}

// The expressions the Krylov and operator kernels build from products,
// written once for FP32, FP64 and double-float entries (the same arithmetic
// as the inline expressions they replace).  Dot-product accumulation alone
// is lazy for double-floats: it only feeds the iteration's scalars.
template <typename T>
__device__ __forceinline__ void mac(T &acc, T a, T b) { acc += a * b; }
__device__ __forceinline__ void mac(dfloat &acc, dfloat a, dfloat b) { df_mac(acc, a, b); }
// x - a b
template <typename T>
__device__ __forceinline__ T sub_mul(T x, T a, T b) { return x - a * b; }
// x + (a p + b s)
template <typename T>
__device__ __forceinline__ T add_mul2(T x, T a, T p, T b, T s) { return x + (a * p + b * s); }
// r + beta (p - omega v)
template <typename T>
__device__ __forceinline__ T p_update(T r, T beta, T p, T om, T v) { return r + beta * (p - om * v); }
// a0 x0 + a1 x1 + ... + a5 x5 (a stencil's neighbour sum)
template <typename T>
__device__ __forceinline__ T sum6(T a0, T x0, T a1, T x1, T a2, T x2, T a3, T x3, T a4, T x4, T a5, T x5) {
    return a0 * x0 + a1 * x1 + a2 * x2 + a3 * x3 + a4 * x4 + a5 * x5;
}

// Per-axis 1-D tables (device pointers, N+4 entries, index i+2).
struct Axis {
    const double *d;     // cell width
    const double *c;     // centroid
    const double *wm;    // face i: weight of cell i-1 = d(i)/(d(i-1)+d(i))
    const double *wp;    // face i: weight of cell i   = d(i-1)/(d(i-1)+d(i))
    const double *rd;    // 1/d(i)
    const double *rdc;   // 1/(c(i)-c(i-1))        face-normal gradient
    const double *rdcc;  // 1/(c(i+1)-c(i-1))      cell-centred gradient
    const double *km;    // Crank-Nicolson coefficient toward i-1 (kx_W)
    const double *kp;    // Crank-Nicolson coefficient toward i+1 (kx_E)
};

// dt times the face-normal and cell-centred gradient reciprocals (FP64,
// per axis, index i+2): one product fewer per face on the FP64 pipe.
struct DtAxis {
    const double *dtrdc, *dtrdcc;
};

// FP32 copies of the tables the FP32 explicit stages read.
struct AxisF {
    const float *wm, *wp, *rd, *rdc, *rdcc, *km, *kp;
};

// Boundary face description with every coefficient the outer-layer rows
// and fills need, precomputed on the host from the reference's formulas
// (src/ibm3d_setup.c:1723-2903, src/ibm3d_fracstep.c:855-1906).
// Index [L-1] is the layer (1 = adjacent to the boundary, 2 = outermost).
struct BCFace {
    int type;            // BCT_*, after set_bc's rewrites (WALL->VELOCITY, SYMMETRIC->SLIP)
    double val[3];       // constant velocity value
    double pval;         // constant pressure value
    // Operator rows.
    double dir_o[2], dir_m[2];   // Dirichlet interpolation: dir_o*x_o + dir_m*x_m
    double ext_o[2], ext_2[2];   // 3-point extrapolation: ext_o*x_o - x_(o+1in) + ext_2*x_(o+2in)
    // Fills (update_outer).
    double fv_a[2], fv_b[2];     // velocity Dirichlet / slip: u_o = fv_a*bc - fv_b*u_m
    double fe_a[2], fe_b[2];     // extrapolation: u_o = fe_a*u_(o+1in) - fe_b*u_(o+2in)
    double fp_a[2], fp_b[2];     // pressure Dirichlet: p_o = fp_a*bc - fp_b*p_m
    // Sampled values of a VAL_FUNC face (null for constant values): one
    // entry per outer line of the face over its padded tangential range
    // (face_line), nt entries per quantity: u1, u2, u3 at [l*nt + t], p at
    // [3*nt + t].  scur holds the values at the step's start time, snxt at
    // its end time (src/ibm3d_fracstep.c:2001-2035).
    const double *scur, *snxt;
    int nt;
};

struct BCSet {
    BCFace f[6];
    int p_singular;      // no pressure / velocity-periodic face: pin p'(0,0,0)
};

// Which boundary face owns an outer cell (each outer cell is owned by
// exactly one face in the reference's matrix assembly: z faces own every
// cell with k outside, y faces every remaining cell with j outside, x faces
// the rest).  Returns -1 for interior cells; layer is 1 or 2.
__host__ __device__ inline int owner_face(const Grid &g, int i, int j, int k, int &layer) {
    if (k < 0) { layer = -k; return F_D; }
    if (k >= g.nz) { layer = k - g.nz + 1; return F_U; }
    if (j < 0) { layer = -j; return F_S; }
    if (j >= g.ny) { layer = j - g.ny + 1; return F_N; }
    if (i < 0) { layer = -i; return F_W; }
    if (i >= g.nx) { layer = i - g.nx + 1; return F_E; }
    layer = 0;
    return -1;
}

__host__ __device__ inline int face_axis(int f) { return (f == F_E || f == F_W) ? 0 : (f == F_N || f == F_S) ? 1 : 2; }

// Outer line of face f through padded cell (i, j, k): its position in the
// face's padded tangential range, (j, k) for x faces, (i, k) for y faces,
// (i, j) for z faces.
__host__ __device__ inline int face_line(const Grid &g, int f, int i, int j, int k) {
    const int ax = face_axis(f);
    if (ax == 0) return (j + 2) * (g.nz + 4) + (k + 2);
    if (ax == 1) return (i + 2) * (g.nz + 4) + (k + 2);
    return (i + 2) * (g.ny + 4) + (j + 2);
}

__host__ __device__ inline int face_lines(const Grid &g, int f) {
    const int ax = face_axis(f);
    return ax == 0 ? (g.ny + 4) * (g.nz + 4) : ax == 1 ? (g.nx + 4) * (g.nz + 4) : (g.nx + 4) * (g.ny + 4);
}
__host__ __device__ inline bool face_low(int f) { return f == F_W || f == F_S || f == F_D; }

// Periodic image of a padded cell: every outer coordinate wrapped into the
// interior, as the reference's cell_idx_periodic (src/ibm3d_setup.c:892-1074).
__host__ __device__ inline long long periodic_image(const Grid &g, int i, int j, int k) {
    if (i < 0) i += g.nx; else if (i >= g.nx) i -= g.nx;
    if (j < 0) j += g.ny; else if (j >= g.ny) j -= g.ny;
    if (k < 0) k += g.nz; else if (k >= g.nz) k -= g.nz;
    return cidx(g, i, j, k);
}

// ------------------------------------------------ dependent launches --
// The step's kernels are launched with programmatic dependent launch: each
// waits for its predecessor's results (griddepcontrol.wait) before any
// read, then at once lets its successor's blocks be scheduled
// (griddepcontrol.launch_dependents); a successor's blocks start only once
// every block of this grid has started, and then wait at their own top.
// This hides the launch gap between the many short kernels of a solve.
// Launched without the attribute, both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
}

// Launch with the programmatic-stream-serialization attribute.
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// ------------------------------------------------------------ reductions --
// Maximum that keeps NaN (fmax drops it): a non-finite value anywhere in a
// maximum reduction reaches the host, which turns it into a status.
__device__ __forceinline__ double nanmax(double a, double b) { return (a != a || b != b) ? a + b : fmax(a, b); }
__device__ __forceinline__ float nanmax(float a, float b) { return (a != a || b != b) ? a + b : fmaxf(a, b); }
__device__ __forceinline__ dfloat nanmax(dfloat a, dfloat b) {
    return (a.hi != a.hi || b.hi != b.hi) ? a + b : (a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo)) ? a : b;
}

// Warp shuffle of a reduction's accumulator type.
__device__ __forceinline__ double shfl_down(double x, int o) { return __shfl_down_sync(0xffffffffu, x, o); }
__device__ __forceinline__ float shfl_down(float x, int o) { return __shfl_down_sync(0xffffffffu, x, o); }
__device__ __forceinline__ dfloat shfl_down(dfloat x, int o) {
    return dfloat(__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o));
}

// Deterministic two-level reductions: every block writes its partials to
// partials[block][v]; the last block to finish reduces them in a fixed
// order.
template <int NV>
__device__ inline void block_sum(double (&v)[NV], double *smem /* [32*NV] */) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        v[q] = x;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) smem[warp * NV + q] = v[q];
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double x = lane < nw ? smem[lane * NV + q] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            v[q] = x;
        }
    }
}

template <int NV>
__device__ inline void block_max(double (&v)[NV], double *smem) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = nanmax(x, __shfl_down_sync(0xffffffffu, x, o));
        v[q] = x;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) smem[warp * NV + q] = v[q];
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double x = lane < nw ? smem[lane * NV + q] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = nanmax(x, __shfl_down_sync(0xffffffffu, x, o));
            v[q] = x;
        }
    }
}

// Block-level combine of NV per-thread values: entries [0, NS) summed,
// [NS, NV) maxed (all >= 0).  The warp stage runs in the accumulator type
// A (an FP32 kernel keeps its adds off the FP64 pipe); one value per warp
// is widened to double for the stage across warps.  Fixed shape, so the
// result is bitwise reproducible.  Valid in warp 0; smem holds 32 * NV
// doubles.
template <int NV, int NS, typename A>
__device__ inline void block_reduce(const A (&v)[NV], double (&out)[NV], double *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        A x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const A y = shfl_down(x, o);
            x = q < NS ? x + y : nanmax(x, y);
        }
        if (lane == 0) smem[warp * NV + q] = (double)x;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double x = lane < nw ? smem[lane * NV + q] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double y = __shfl_down_sync(0xffffffffu, x, o);
                x = q < NS ? x + y : nanmax(x, y);
            }
            out[q] = x;
        }
    }
}

// Publishes this block's NV partials; returns true in EVERY thread of the
// last block to finish (the same value across the block), which then
// reduces all blocks' partials with reduce_partials.
template <int NV>
__device__ inline bool publish_partials(const double (&v)[NV], double *partials, unsigned int *counter) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) partials[blockIdx.x * NV + q] = v[q];
        __threadfence();
        const unsigned int t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Reduces every block's partials inside the last block: entries [0, NS)
// are summed, entries [NS, NV) maxed (all maxed quantities are >= 0, so 0
// is their identity).  Thread t folds blocks t, t + blockDim, ... in that
// order and a fixed-shape tree combines the threads, so the result does
// not depend on block scheduling (bitwise reproducible).  Valid in thread
// 0; smem holds 32 * NV doubles and must be free on entry.
template <int NV, int NS>
__device__ inline void reduce_partials(const double *partials, int nblocks, double (&out)[NV], double *smem) {
    double v[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            const double x = __ldcg(partials + (size_t)b * NV + q);
            v[q] = q < NS ? v[q] + x : nanmax(v[q], x);
        }
    }
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, o);
            x = q < NS ? x + y : nanmax(x, y);
        }
        v[q] = x;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) smem[warp * NV + q] = v[q];
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double x = lane < nw ? smem[lane * NV + q] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double y = __shfl_down_sync(0xffffffffu, x, o);
                x = q < NS ? x + y : nanmax(x, y);
            }
            out[q] = x;
        }
    }
}

}  // namespace ibm
