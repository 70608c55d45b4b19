// Kernel argument structs and launch wrappers shared by the host code.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace ibm {

// Number of kernels this library has launched (for per-step launch counts);
// while a step is being recorded into a CUDA graph the count goes to the
// recording.
void note_launches(int n);

struct ConvArgs {
    const double *u[3];
    const double *U[3];
    const double *p;
    const double *Np[3];
    const double *tau[6];
    double *N[3];
    double *b[3];
    const double *force;   // sampled VAL_FUNC body force, 3 x ncell (null: the constant force)
};

struct TauArgs {
    double *tau[6];
};

struct UstarArgs {
    const double *us[3];
    const double *p;
    double *Us[3];
    double *b;
};

struct NextArgs {
    const double *us[3];
    const double *Us[3];
    const double *p;
    const double *pp;
    double *un[3];
    double *Un[3];
    double *pn;
};

// FP32 explicit stages of the IBM3D_MIXED32 step (step32_kernels.cu).
struct Conv32Args {
    const double *u[3];
    const double *U[3];
    const double *p;
    const float *Np[3];
    const double *tau[6];
    const double *force;   // sampled VAL_FUNC body force, 3 x ncell (null: the constant force)
    float *N[3];
    float *c;              // increment right-hand side, 3 x ncell
};

struct Ustar32Args {
    const double *u[3];    // u^n
    const float *e[3];     // momentum increment e = u* - u^n
    const double *p;
    const double *dinv;    // 1 / coeffsum on fluid rows
    double *Us[3];
    double *b;
};

struct Next32Args {
    const double *u[3];    // u^n
    const float *e[3];
    const double *Us[3];
    const double *p;
    const double *pp;
    double *un[3];
    double *Un[3];
    double *pn;
};

enum { GK_ARRAY = 0, GK_OLD = 1, GK_SKIP = 2 };

struct GhostArgs {
    int nghost;
    int nlevels;
    const int *level_start;  // device, nlevels+1
    const int *cell;         // padded index of each ghost (level-sorted)
    const int *ref;          // [8*g+e]: padded index (GK_ARRAY) or ghost id (GK_OLD)
    const int8_t *kind;      // [8*g+e]
    const double *w;         // [8*g+e] normalised weights (0 where skipped)
    const double *wself;     // weight of the ghost cell in its own stencil
    double *old;             // [4*g]: snapshot of u1,u2,u3,p
    const int *hlevel_start; // host copy of level_start (launch sizes; not read on the device)
};

void launch_conv_rhs(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                     const BCSet &bc, const uint8_t *flag, const ConvArgs &a, double dt, const double f[3],
                     int les);
void launch_smagorinsky(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                        const uint8_t *flag, const double *lvset, const double *const u[3], const TauArgs &t,
                        double cs);
void launch_ustar_prhs(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                       const BCSet &bc, const uint8_t *flag, const UstarArgs &a, double dt, double Re);
// when: 0 fills with the values at the step's start time, 1 at its end
// time (the two differ only for VAL_FUNC faces).
void launch_fill_outer(cudaStream_t s, const Grid &g, const BCSet &bc, double *const u[3], double *p, int when);
// x[l n + P] = u[l][P] (NaN, as on solid cells, becomes 0): the initial
// guess of the momentum solve.
void launch_velocity_guess(cudaStream_t s, const Grid &g, double *const u[3], double *x);
void launch_interp_stag(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                        const double *const u[3], double *const U[3]);
void launch_ghost_update(cudaStream_t s, const GhostArgs &a, double *const u[3], double *p);
void launch_solid_nan(cudaStream_t s, const Grid &g, const uint8_t *flag, double *const u[3], double *p);

struct IRScal;
template <typename T>
struct OpT;
void launch_conv_rhs32(cudaStream_t s, const Grid &g, const AxisF axf[3], const OpT<float> &A, const BCSet &bc,
                       const uint8_t *flag, const Conv32Args &a, double dt, const double f[3], int les,
                       double *partials, unsigned int *counter, IRScal *out);
// update_next over tiles of 32 (k) x 8 (j) columns marching over planes of
// i: each face of U^{n+1} is computed once (x faces carried along i, y
// faces exchanged in shared memory, z faces by warp shuffle).  a32: the
// increment form of IBM3D_MIXED32, else the FP64 step (a64).
void launch_update_next_tiled(cudaStream_t s, const Grid &g, const Axis ax64[3], const DtAxis dta[3],
                              const AxisF axf[3], const BCSet &bc, const uint8_t *flag, const NextArgs *a64,
                              const Next32Args *a32, double dt, double *partials, unsigned int *counter,
                              double *maxdiv_out);
// calc_u_tilde into ut (3 x ncell floats), then U* and the Poisson
// right-hand side over tiles, then the outer rows (outer: padded indices of
// the nout outer cells).
void launch_ustar_prhs32_tiled(cudaStream_t s, const Grid &g, const AxisF axf[3], const Axis ax64[3],
                               const BCSet &bc, const uint8_t *flag, const Ustar32Args &a, float *ut, double dt,
                               double Re, const int *outer, int nout);
void launch_widen_f32(cudaStream_t s, long long n, const float *x, double *y);
void launch_ustar_from_increment(cudaStream_t s, long long n, const double *u, const float *e, double *y);
// Compares d2f_int / f2d_int with the hardware conversions on n host
// values; returns 0 and the mismatch count, or -1 on a CUDA error.
int conversion_check(long long n, const double *x_host, unsigned long long *mismatches);

// Warm-started pressure solve: pp <- 2 pp - prev once two increments are
// known (hist >= 2), prev <- the old pp; then hist advances (up to 2).
void launch_pressure_guess(cudaStream_t s, long long n, double *pp, double *prev, int *hist);

// Register-only FMA throughput in TFLOP/s: which 0 FP64, 1 FP32.
double fma_rate(int which);

// Result export: float u, v, w, p, vorticity, Q, each (nx+4)(ny+4)(nz+4)
// values in [z][y][x] order, into out (6 such arrays).  ny + 4 <= 65535.
void launch_export_fields(cudaStream_t s, const Grid &g, const Axis &ax, const Axis &ay, const Axis &az,
                          const double *const u[3], const double *p, float *out);

}  // namespace ibm
