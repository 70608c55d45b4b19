// IBMSolver C ABI on one GB300: host orchestration of the fractional step.
//
// Entry points mirror src/ibm3d_setup.c, src/ibm3d_init.c,
// src/ibm3d_fracstep.c, src/ibm3d_turb.c and src/ibm3d_export.c (cited per
// function).  All per-step work runs on the GPU; the host only sequences
// kernels, reads Krylov convergence scalars, and prints the reference's
// per-step table.
#include <cmath>
#include <ctime>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <functional>
#include <string>
#include <vector>

#include "../../include/ibm3d.h"
#include "../../include/ibm3d_gb300.h"
#include "common.cuh"
#include "geo3d.h"
#include "kernels.h"
#include "krylov.h"
#include "multigrid.h"
#include "ncfile.h"
#include "prof.h"
#include "setup.h"

using namespace ibm;

#include <atomic>

namespace ibm {
static std::atomic<long long> g_launches{0};
// While a step is being recorded into a graph, launches are counted into
// the recording instead (they run only when the graph does).
static thread_local long long *g_redirect = nullptr;
void note_launches(int n) {
    if (g_redirect) *g_redirect += n;
    else g_launches += n;
}
}  // namespace ibm

// One recorded time step (CUDA graph): the step's kernels with both
// linear solves as device-side while loops, the outer-layer fill, the
// ghost update and the read-back of the step's scalars.  The field
// pointers alternate between steps, so a graph is keyed by them.
struct StepGraph {
    const void *key[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaGraphExec_t exec = nullptr;
    int fixed = 0;                          // kernels outside solver loops
    int mom_iter = 0, mom_outer = 0;        // per momentum iteration / refinement cycle
    int p_iter = 0, p_outer = 0;
};

// Host parameters baked into recorded graphs.
struct GraphSig {
    int precision, les, use_mg, max_outer, solver, gm_restart, warm, p_guess, pvec;
    double tol, divtol, Re, dt, f[3], cs, inner_tol[2];
    bool operator==(const GraphSig &o) const { return memcmp(this, &o, sizeof *this) == 0; }
};

struct ibm3d_device {
    cudaStream_t s = nullptr;
    Grid g{};
    int dev_id = 0;
    char dev_name[288] = "";  // the device name (up to 256) and its " (sm_XY)"
    // Per-axis 1-D tables: 9 arrays of n+4 doubles each.
    double *tab[3] = {nullptr, nullptr, nullptr};
    Axis ax[3];
    // FP32 copies (wm, wp, rd, rdc, rdcc, km, kp) for the FP32 explicit stages.
    float *tabf[3] = {nullptr, nullptr, nullptr};
    AxisF axf[3];
    // dt x rdc and dt x rdcc per axis (FP64).
    double *dtab[3] = {nullptr, nullptr, nullptr};
    DtAxis dta[3];
    BCSet bc{};
    // Fields.
    double *fields = nullptr;
    size_t nfields = 0;
    double *u[3], *un[3], *ustar, *U[3], *Un[3], *Us[3], *p, *pn, *pp, *N[3], *Np[3], *tau[6], *b, *lvset, *dinv;
    uint8_t *flag = nullptr;
    int *gid = nullptr;
    // Pressure-guess extrapolation (IBMSolver_set_pressure_guess): the
    // increment before the last one, and how many increments are known.
    double *pp_prev = nullptr;
    int *pp_hist = nullptr;
    int p_guess = 1;   // warm-started (mixed) pressure solves start from the extrapolation
    // IBM3D_MIXED32: N and N_prev in FP32 (6 arrays of ncell floats).
    float *f32 = nullptr;
    float *N32[3], *Np32[3];
    float *ut32 = nullptr;   // u~ (3 x ncell floats)
    // Ghost cells.
    int nghost = 0, nlevels = 0;
    std::vector<int> ghost_level_start;   // host copy of the ghosts' level starts (launch sizes)
    int *g_mem = nullptr;
    double *g_dmem = nullptr;
    int8_t *g_kind = nullptr;
    GhostArgs gargs{};
    int *g_gidx = nullptr;
    double *g_gw = nullptr, *g_gwself = nullptr;
    std::vector<GhostStencil> gst;   // lexicographic order
    std::vector<int> gcell_lex;      // padded index, lexicographic order
    // Operator tables of the matrix-free solves: FP64 ks per axis; FP32
    // km, kp, ks, d per axis, then dinv, wdiv (n each), ghost weights.
    double *op64 = nullptr;
    float *op32 = nullptr;
    dfloat *opdf = nullptr;       // the FP64 tables as double-floats: km, kp, ks, d per axis, dinv, ghost weights
    int *sweep_outer = nullptr;   // outer cells of the padded grid (sweep launches)
    OpT<double> A64{};
    OpT<float> A32{};
    OpT<dfloat> Adf{};
    // Solvers: FP64 BiCGSTAB (plain path) and FP64 refinement around FP32
    // BiCGSTAB (mixed path), each with its multigrid preconditioner.
    KrylovWork<double> kmom, kpres;
    IRWork irmom, irpres;
    GMG<double> *mg = nullptr;
    GMG<float> *mg32 = nullptr;
    WidenedPreconditioner pc64;   // FP32 multigrid under an FP64 Krylov solve
    // IBM3D_MIXED32 pressure solve on double-float vectors: a view of
    // kpres's buffers, the solution vector and the FP32 multigrid behind it.
    KrylovWork<dfloat> kpres_df;
    dfloat *pp_df = nullptr;
    DFloatPreconditioner pcdf;
    int pvec = IBM3D_PVEC_DFLOAT;
    GmresWork gm;                 // SOLVER_GMRES pressure solves
    int gm_restart = 10;          // restart length (the reference's KDim, src/ibm3d_setup.c:1474)
    double *red_partials = nullptr;
    unsigned int *red_counter = nullptr;
    double *maxdiv_d = nullptr;
    double *maxdiv_h = nullptr;
    // VAL_FUNC boundary values and body force, sampled on the host each
    // step: per sampled face a block of 2 x 4 x nt values (start-time
    // values, then end-time values; see BCFace), and 3 x ncell force values.
    double *smp_d = nullptr, *smp_h = nullptr;
    size_t smp_n = 0;
    size_t smp_off[6] = {0, 0, 0, 0, 0, 0};
    bool smp_face[6] = {false, false, false, false, false, false};
    double smp_t[2] = {0, 0}, smp_dev_t[2] = {0, 0};
    bool smp_valid = false, smp_dev_valid = false;
    double *force_d = nullptr, *force_h = nullptr;
    double force_t = 0, force_dev_t = 0;
    bool force_valid = false, force_dev_valid = false;
    // Settings.
    double divtol = 0.0;
    int precision = IBM3D_FP64;
    int les = 0;
    int cpt_fallback = 0;
    bool abort_on_error = true;
    size_t dev_bytes = 0;   // device memory taken by assembly (free-memory difference)
    // Recorded steps.
    bool use_graphs = true;
    int mg_sweeps[5] = {3, 3, 2, 2, 16};  // multigrid sweeps: fine pre/post, coarse pre/post, coarsest
    double mg_omega = 1.0;               // over-relaxation of the fine-grid smoother
    int mg_coarsening = IBM3D_COARSEN_SPACING;
    int warm_start = 1;                  // mixed modes: momentum solve from the current velocity
    int maxit_mom = 200, maxit_p = 1000; // Krylov iteration caps (src/ibm3d_setup.c:1411-1432, 1435-1563)
    double mg_width_ratio = 1.5;
    // Mixed path: relative tolerance of each FP32 inner solve (momentum,
    // pressure) and the refinement-cycle cap.
    // FP32 inner solves of the refinement cycles: momentum to 5e-7 (one
    // cycle then meets the usual 1e-6 momentum tolerance: FP32 BiCGSTAB's
    // recursive residual keeps falling below the FP32 rounding of the
    // true one, and the FP64 check decides), pressure to 1e-5.
    double inner_tol[2] = {5e-7, 1e-5};
    int max_outer = 12;
    cudaStream_t aux[2] = {nullptr, nullptr};
    std::vector<StepGraph> graphs;
    GraphSig gsig{};
    // Last-step statistics.
    SolveReport rep_mom, rep_p;
    double max_div = 0.0;
    // Totals since assembly (IBMSolverStats).
    long long steps_total = 0, iters_u_total[3] = {0, 0, 0}, iters_p_total = 0, outer_p_total = 0;
    double max_div_max = 0.0;
    int status = IBM3D_OK;
    char message[512] = {0};  // text of the last error
    bool assembled = false;
    Prof prof;
};

namespace {

// A batched step runs one graph branch per member; with CUDA's default of 8
// hardware work queues most branches wait for a queue.  Ask for the maximum
// (32) when the library is loaded, unless the host already chose a value;
// it applies to CUDA contexts created after this point.
__attribute__((constructor)) void ibm3d_queues() { setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0); }

constexpr double kNaN = __builtin_nan("");

int ncell_of(const IBMSolver *s) { return (s->Nx + 4) * (s->Ny + 4) * (s->Nz + 4); }

void set_status(IBMSolver *s, int code, const char *fmt, ...) {
    char text[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(text, sizeof text, fmt, ap);
    va_end(ap);
    if (s && s->dev) {
        s->dev->status = code;
        memcpy(s->dev->message, text, sizeof text);
    }
    fprintf(stderr, "error: %s\n", text);
    if (s && s->dev && s->dev->abort_on_error && code != IBM3D_ENOCONV) std::exit(255);
}

bool cuda_check(IBMSolver *s, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_status(s, IBM3D_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    return false;
}

bool isperiodic(IBMSolverBCType t) { return t == BC_ALL_PERIODIC || t == BC_VELOCITY_PERIODIC; }

double *c1(double *a, int i) { return &a[i + 2]; }

// Outer-layer coefficients of one face (see BCFace).
void make_bcface(const IBMSolver *sv, int f, BCFace &F) {
    const IBMSolverBC &B = sv->bc[f];
    switch (B.type) {
    case BC_VELOCITY_COMPONENT:
    case BC_STATIONARY_WALL: F.type = BCT_VELOCITY; break;
    case BC_PRESSURE: F.type = BCT_PRESSURE; break;
    case BC_FREE_SLIP_WALL:
    case BC_SYMMETRIC: F.type = BCT_SLIP; break;
    case BC_ALL_PERIODIC: F.type = BCT_PERIODIC; break;
    case BC_VELOCITY_PERIODIC: F.type = BCT_VELPERIODIC; break;
    }
    F.val[0] = B.const_u1;
    F.val[1] = B.const_u2;
    F.val[2] = B.const_u3;
    F.pval = B.const_p;
    const int axis = face_axis(f);
    const bool low = face_low(f);
    const double *d = axis == 0 ? sv->dx : axis == 1 ? sv->dy : sv->dz;
    const double *c = axis == 0 ? sv->xc : axis == 1 ? sv->yc : sv->zc;
    const int N = axis == 0 ? sv->Nx : axis == 1 ? sv->Ny : sv->Nz;
    auto D = [&](int i) { return d[i + 2]; };
    auto C = [&](int i) { return c[i + 2]; };
    // Pressure-Dirichlet fill widths: the reference's down face reads dx here
    // (src/ibm3d_fracstep.c:1792-1800); every other face its own axis.
    const double *dp = (f == F_D) ? sv->dx : d;
    auto DP = [&](int i) { return dp[i + 2]; };
    for (int L = 1; L <= 2; L++) {
        double a, b, ap, bp, ea, eb;
        if (low) {
            if (L == 1) {
                a = D(-1) / 2; b = D(0) / 2;
                ap = DP(-1) / 2; bp = DP(0) / 2;
                ea = C(0) - C(-1); eb = C(1) - C(0);
            } else {
                a = D(-2) / 2 + D(-1); b = D(0) + D(1) / 2;
                ap = DP(-2) / 2 + DP(-1); bp = DP(0) + DP(1) / 2;
                ea = C(-1) - C(-2); eb = C(0) - C(-1);
            }
            F.dir_o[L - 1] = b / (a + b);
            F.dir_m[L - 1] = a / (a + b);
            F.fv_a[L - 1] = (a + b) / b;
            F.fv_b[L - 1] = a / b;
            F.fp_a[L - 1] = (ap + bp) / bp;
            F.fp_b[L - 1] = ap / bp;
            F.ext_o[L - 1] = eb / (ea + eb);
            F.ext_2[L - 1] = ea / (ea + eb);
            F.fe_a[L - 1] = (ea + eb) / eb;
            F.fe_b[L - 1] = ea / eb;
        } else {
            if (L == 1) {
                a = D(N - 1) / 2; b = D(N) / 2;
                ap = DP(N - 1) / 2; bp = DP(N) / 2;
                ea = C(N - 1) - C(N - 2); eb = C(N) - C(N - 1);
            } else {
                a = D(N - 2) / 2 + D(N - 1); b = D(N) + D(N + 1) / 2;
                ap = DP(N - 2) / 2 + DP(N - 1); bp = DP(N) + DP(N + 1) / 2;
                ea = C(N) - C(N - 1); eb = C(N + 1) - C(N);
            }
            F.dir_o[L - 1] = a / (a + b);
            F.dir_m[L - 1] = b / (a + b);
            F.fv_a[L - 1] = (a + b) / a;
            F.fv_b[L - 1] = b / a;
            F.fp_a[L - 1] = (ap + bp) / ap;
            F.fp_b[L - 1] = bp / ap;
            F.ext_o[L - 1] = ea / (ea + eb);
            F.ext_2[L - 1] = eb / (ea + eb);
            F.fe_a[L - 1] = (ea + eb) / ea;
            F.fe_b[L - 1] = eb / ea;
        }
    }
}

template <typename T>
void dfree(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}

void drop_graphs(ibm3d_device *d) {
    for (auto &G : d->graphs)
        if (G.exec) cudaGraphExecDestroy(G.exec);
    d->graphs.clear();
}

void release_device(ibm3d_device *d) {
    if (!d) return;
    delete d->mg;
    d->mg = nullptr;
    delete d->mg32;
    d->mg32 = nullptr;
    d->pc64.release();
    d->gm.release();
    d->kmom.release();
    d->kpres.release();
    d->kpres_df.release();
    dfree(d->pp_df);
    d->irmom.release();
    d->irpres.release();
    dfree(d->op64);
    dfree(d->op32);
    dfree(d->opdf);
    dfree(d->sweep_outer);
    d->A64 = OpT<double>{};
    d->A32 = OpT<float>{};
    d->Adf = OpT<dfloat>{};
    for (int a = 0; a < 3; a++) {
        dfree(d->tab[a]);
        dfree(d->tabf[a]);
        dfree(d->dtab[a]);
    }
    dfree(d->fields);
    dfree(d->f32);
    dfree(d->pp_prev);
    dfree(d->pp_hist);
    dfree(d->flag);
    dfree(d->gid);
    dfree(d->g_mem);
    dfree(d->g_dmem);
    dfree(d->g_kind);
    dfree(d->red_partials);
    dfree(d->red_counter);
    dfree(d->maxdiv_d);
    if (d->maxdiv_h) cudaFreeHost(d->maxdiv_h);
    d->maxdiv_h = nullptr;
    dfree(d->smp_d);
    dfree(d->force_d);
    if (d->smp_h) cudaFreeHost(d->smp_h);
    if (d->force_h) cudaFreeHost(d->force_h);
    d->smp_h = d->force_h = nullptr;
    d->smp_n = 0;
    d->smp_valid = d->smp_dev_valid = d->force_valid = d->force_dev_valid = false;
    d->nghost = d->nlevels = 0;
    d->gargs = GhostArgs{};
    d->g_gidx = nullptr;
    d->g_gw = d->g_gwself = nullptr;
    d->assembled = false;
    drop_graphs(d);
    for (auto &a : d->aux) {
        if (a) cudaStreamDestroy(a);
        a = nullptr;
    }
    if (d->s) cudaStreamDestroy(d->s);
    d->s = nullptr;
}

template <typename T>
T *dmalloc(IBMSolver *sv, size_t n, const char *what) {
    void *p = nullptr;
    if (!cuda_check(sv, cudaMalloc(&p, n * sizeof(T) + 16), what)) return nullptr;
    cudaMemsetAsync(p, 0, n * sizeof(T) + 16, sv->dev->s);
    return (T *)p;
}

// Grid extension (src/ibm3d_setup.c:535-618) and the Crank-Nicolson
// coefficients (src/ibm3d_setup.c:620-632) on the host arrays.
void host_metrics(IBMSolver *s) {
    auto ext = [](double *d, double *c, int N, bool plo, bool phi) {
        *c1(d, -1) = plo ? *c1(d, N - 1) : *c1(d, 0);
        *c1(d, -2) = plo ? *c1(d, N - 2) : *c1(d, 1);
        *c1(d, N) = phi ? *c1(d, 0) : *c1(d, N - 1);
        *c1(d, N + 1) = phi ? *c1(d, 1) : *c1(d, N - 2);
        *c1(c, -1) = *c1(c, 0) - (*c1(d, -1) + *c1(d, 0)) / 2;
        *c1(c, -2) = *c1(c, -1) - (*c1(d, -2) + *c1(d, -1)) / 2;
        *c1(c, N) = *c1(c, N - 1) + (*c1(d, N - 1) + *c1(d, N)) / 2;
        *c1(c, N + 1) = *c1(c, N) + (*c1(d, N) + *c1(d, N + 1)) / 2;
    };
    ext(s->dx, s->xc, s->Nx, isperiodic(s->bc[3].type), isperiodic(s->bc[1].type));
    ext(s->dy, s->yc, s->Ny, isperiodic(s->bc[2].type), isperiodic(s->bc[0].type));
    ext(s->dz, s->zc, s->Nz, isperiodic(s->bc[4].type), isperiodic(s->bc[5].type));
    auto kco = [&](double *km, double *kp, const double *d, const double *c, int N) {
        for (int i = 0; i < N; i++) {
            km[i + 2] = s->dt / (2 * s->Re * (c[i + 2] - c[i + 1]) * d[i + 2]);
            kp[i + 2] = s->dt / (2 * s->Re * (c[i + 3] - c[i + 2]) * d[i + 2]);
        }
    };
    kco(s->kx_W, s->kx_E, s->dx, s->xc, s->Nx);
    kco(s->ky_S, s->ky_N, s->dy, s->yc, s->Ny);
    kco(s->kz_D, s->kz_U, s->dz, s->zc, s->Nz);
}

bool upload_axes(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    const double *D[3] = {sv->dx, sv->dy, sv->dz}, *Cc[3] = {sv->xc, sv->yc, sv->zc};
    const double *KM[3] = {sv->kx_W, sv->ky_S, sv->kz_D}, *KP[3] = {sv->kx_E, sv->ky_N, sv->kz_U};
    const int Ns[3] = {sv->Nx, sv->Ny, sv->Nz};
    for (int a = 0; a < 3; a++) {
        const int n = Ns[a] + 4;
        std::vector<double> h(9 * (size_t)n, 0.0);
        double *dd = &h[0], *cc = &h[n], *wm = &h[2 * n], *wp = &h[3 * n], *rd = &h[4 * n], *rdc = &h[5 * n],
               *rdcc = &h[6 * n], *km = &h[7 * n], *kp = &h[8 * n];
        for (int q = 0; q < n; q++) {
            dd[q] = D[a][q];
            cc[q] = Cc[a][q];
            rd[q] = 1.0 / D[a][q];
            km[q] = KM[a][q];
            kp[q] = KP[a][q];
            if (q >= 1) {
                wm[q] = D[a][q] / (D[a][q - 1] + D[a][q]);
                wp[q] = D[a][q - 1] / (D[a][q - 1] + D[a][q]);
                rdc[q] = 1.0 / (Cc[a][q] - Cc[a][q - 1]);
            }
            if (q >= 1 && q + 1 < n) rdcc[q] = 1.0 / (Cc[a][q + 1] - Cc[a][q - 1]);
        }
        d->tab[a] = dmalloc<double>(sv, h.size(), "axis tables");
        if (!d->tab[a]) return false;
        cudaMemcpyAsync(d->tab[a], h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, d->s);
        double *t = d->tab[a];
        d->ax[a] = Axis{t, t + n, t + 2 * n, t + 3 * n, t + 4 * n, t + 5 * n, t + 6 * n, t + 7 * n, t + 8 * n};
        // FP32 copies of wm, wp, rd, rdc, rdcc, km, kp (rows 2..8).
        std::vector<float> hf(7 * (size_t)n);
        for (size_t q = 0; q < hf.size(); q++) hf[q] = (float)h[2 * (size_t)n + q];
        d->tabf[a] = dmalloc<float>(sv, hf.size(), "FP32 axis tables");
        if (!d->tabf[a]) return false;
        cudaMemcpyAsync(d->tabf[a], hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice, d->s);
        float *f = d->tabf[a];
        d->axf[a] = AxisF{f, f + n, f + 2 * n, f + 3 * n, f + 4 * n, f + 5 * n, f + 6 * n};
        std::vector<double> hd(2 * (size_t)n);
        for (int q = 0; q < n; q++) {
            hd[q] = sv->dt * rdc[q];
            hd[n + q] = sv->dt * rdcc[q];
        }
        d->dtab[a] = dmalloc<double>(sv, hd.size(), "dt axis tables");
        if (!d->dtab[a]) return false;
        cudaMemcpyAsync(d->dtab[a], hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice, d->s);
        d->dta[a] = DtAxis{d->dtab[a], d->dtab[a] + n};
    }
    return true;
}

bool alloc_fields(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    const long long n = d->g.ncell;
    // u, un, ustar(3), U, Un, Us, p, pn, pp, N, Np, tau(6), b(3), lvset, dinv
    d->nfields = 3 + 3 + 3 + 3 + 3 + 3 + 1 + 1 + 1 + 3 + 3 + 6 + 3 + 1 + 1;
    d->fields = dmalloc<double>(sv, d->nfields * (size_t)n, "field arrays");
    if (!d->fields) return false;
    double *q = d->fields;
    auto take = [&](int k) {
        double *r = q;
        q += (size_t)k * n;
        return r;
    };
    for (int l = 0; l < 3; l++) d->u[l] = take(1);
    for (int l = 0; l < 3; l++) d->un[l] = take(1);
    d->ustar = take(3);
    for (int l = 0; l < 3; l++) d->U[l] = take(1);
    for (int l = 0; l < 3; l++) d->Un[l] = take(1);
    for (int l = 0; l < 3; l++) d->Us[l] = take(1);
    d->p = take(1);
    d->pn = take(1);
    d->pp = take(1);
    for (int l = 0; l < 3; l++) d->N[l] = take(1);
    for (int l = 0; l < 3; l++) d->Np[l] = take(1);
    for (int l = 0; l < 6; l++) d->tau[l] = take(1);
    d->b = take(3);
    d->lvset = take(1);
    d->dinv = take(1);
    d->f32 = dmalloc<float>(sv, 9 * (size_t)n, "FP32 convection terms and u~");
    if (!d->f32) return false;
    d->ut32 = d->f32 + 6 * (size_t)n;
    d->pp_prev = dmalloc<double>(sv, n, "pressure increment history");
    d->pp_hist = dmalloc<int>(sv, 1, "pressure increment count");
    if (!d->pp_prev || !d->pp_hist) return false;
    for (int l = 0; l < 3; l++) {
        d->N32[l] = d->f32 + (size_t)l * n;
        d->Np32[l] = d->f32 + (size_t)(3 + l) * n;
    }
    d->flag = dmalloc<uint8_t>(sv, n, "flags");
    d->gid = dmalloc<int>(sv, n, "ghost map");
    // Partials of the fused reductions: up to 8 values per block of the
    // largest reducing launch (tiles at most one plane deep, plus blocks
    // over the outer cells).
    const long long tiles = (long long)((d->g.nz + 31) / 32) * ((d->g.ny + 7) / 8) * d->g.nx;
    d->red_partials = dmalloc<double>(sv, 8 * (size_t)(tiles + n / 256 + 4096), "reduction partials");
    d->red_counter = dmalloc<unsigned int>(sv, 1, "reduction counter");
    d->maxdiv_d = dmalloc<double>(sv, 1, "max div");
    if (!d->flag || !d->gid || !d->red_partials || !d->red_counter || !d->maxdiv_d) return false;
    if (!cuda_check(sv, cudaMallocHost(&d->maxdiv_h, sizeof(double)), "pinned scalar")) return false;
    return true;
}

// Level set and flags (src/ibm3d_setup.c:1081-1254) on the GPU.
bool build_levelset(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    const long long n = d->g.ncell;
    if (!sv->poly) {
        std::vector<double> h(n, 0.5);
        cudaMemcpyAsync(d->lvset, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, d->s);
        std::vector<uint8_t> f(n, FLUID);
        cudaMemcpyAsync(d->flag, f.data(), n, cudaMemcpyHostToDevice, d->s);
        cudaStreamSynchronize(d->s);
        return true;
    }
    CptModel m;
    build_cpt_model(sv->poly, 15, m);
    int nfb = 0;
    if (gpu_cpt(d->s, m, sv->Nx + 4, sv->Ny + 4, sv->Nz + 4, d->ax[0].c, d->ax[1].c, d->ax[2].c, d->lvset, 15, &nfb) != 0) {
        set_status(sv, IBM3D_ECUDA, "level-set kernels failed");
        return false;
    }
    d->cpt_fallback = nfb;
    gpu_flags(d->s, d->g, d->lvset, d->flag);
    return cuda_check(sv, cudaStreamSynchronize(d->s), "flags");
}

// Ghost stencils (GPU), dependency levels and operator tables (host).
bool build_ghosts(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    const Grid &g = d->g;
    const long long n = g.ncell;
    std::vector<uint8_t> fl(n);
    cudaMemcpyAsync(fl.data(), d->flag, n, cudaMemcpyDeviceToHost, d->s);
    cudaStreamSynchronize(d->s);
    d->gcell_lex.clear();
    for (int i = 0; i < sv->Nx; i++)
        for (int j = 0; j < sv->Ny; j++)
            for (int k = 0; k < sv->Nz; k++) {
                const long long P = cidx(g, i, j, k);
                if (fl[P] == GHOST) d->gcell_lex.push_back((int)P);
            }
    const int ng = (int)d->gcell_lex.size();
    d->nghost = ng;
    d->gst.assign(ng, GhostStencil{});
    std::vector<int> hgid(n, -1);
    if (ng > 0) {
        int *gc = nullptr;
        GhostStencil *gs = nullptr;
        cudaMalloc(&gc, sizeof(int) * ng);
        cudaMalloc(&gs, sizeof(GhostStencil) * ng);
        cudaMemcpyAsync(gc, d->gcell_lex.data(), sizeof(int) * ng, cudaMemcpyHostToDevice, d->s);
        const int rc = gpu_ghost_stencils(d->s, g, d->ax[0].c, d->ax[1].c, d->ax[2].c, d->lvset, d->flag, gc, ng, gs);
        cudaMemcpyAsync(d->gst.data(), gs, sizeof(GhostStencil) * ng, cudaMemcpyDeviceToHost, d->s);
        cudaStreamSynchronize(d->s);
        cudaFree(gc);
        cudaFree(gs);
        if (rc != 0) {
            set_status(sv, IBM3D_ECUDA, "ghost stencil kernel failed");
            return false;
        }
        for (int q = 0; q < ng; q++)
            if (!d->gst[q].ok) {
                int i, j, k;
                cijk(g, d->gcell_lex[q], i, j, k);
                set_status(sv, IBM3D_EGEOM, "mirror point of ghost cell (%d,%d,%d) lies outside the grid", i, j, k);
                return false;
            }
        // Lexicographic ghost id of each ghost cell.
        std::vector<int> lexid(n, -1);
        for (int q = 0; q < ng; q++) lexid[d->gcell_lex[q]] = q;
        // Dependency level: 1 + max level of lower-index ghosts in the stencil.
        std::vector<int> level(ng, 0);
        int nlev = 1;
        for (int q = 0; q < ng; q++) {
            int lv = 0;
            for (int e = 0; e < 8; e++) {
                const int c = d->gst[q].cell[e];
                if (c < 0) continue;
                const int h = lexid[c];
                if (h >= 0 && h < q) lv = std::max(lv, level[h] + 1);
            }
            level[q] = lv;
            nlev = std::max(nlev, lv + 1);
        }
        // Level-major order.
        std::vector<int> order(ng);
        for (int q = 0; q < ng; q++) order[q] = q;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return level[a] < level[b]; });
        std::vector<int> newid(ng);
        for (int q = 0; q < ng; q++) newid[order[q]] = q;
        std::vector<int> lstart(nlev + 1, 0);
        for (int q = 0; q < ng; q++) lstart[level[q] + 1]++;
        for (int l = 0; l < nlev; l++) lstart[l + 1] += lstart[l];
        std::vector<int> cell(ng), ref(8 * ng), gidx(8 * ng);
        std::vector<int8_t> kind(8 * ng);
        std::vector<double> w(8 * ng), wself(ng);
        for (int t = 0; t < ng; t++) {
            const int q = order[t];
            const GhostStencil &st = d->gst[q];
            cell[t] = d->gcell_lex[q];
            wself[t] = st.wself;
            hgid[cell[t]] = t;
            for (int e = 0; e < 8; e++) {
                const int c = st.cell[e];
                w[8 * t + e] = st.w[e];
                gidx[8 * t + e] = c;
                if (c < 0) {
                    kind[8 * t + e] = GK_SKIP;
                    ref[8 * t + e] = 0;
                } else if (lexid[c] > q) {
                    kind[8 * t + e] = GK_OLD;
                    ref[8 * t + e] = newid[lexid[c]];
                } else {
                    kind[8 * t + e] = GK_ARRAY;
                    ref[8 * t + e] = c;
                }
            }
        }
        d->nlevels = nlev;
        // Device copies: ints [cell | ref | gidx | level_start], doubles [w | wself | old(4*ng) | gw].
        d->g_mem = dmalloc<int>(sv, (size_t)ng * 17 + nlev + 1, "ghost tables");
        d->g_dmem = dmalloc<double>(sv, (size_t)ng * (8 + 1 + 4), "ghost weights");
        d->g_kind = dmalloc<int8_t>(sv, (size_t)ng * 8, "ghost kinds");
        if (!d->g_mem || !d->g_dmem || !d->g_kind) return false;
        int *im = d->g_mem;
        cudaMemcpyAsync(im, cell.data(), sizeof(int) * ng, cudaMemcpyHostToDevice, d->s);
        cudaMemcpyAsync(im + ng, ref.data(), sizeof(int) * 8 * ng, cudaMemcpyHostToDevice, d->s);
        cudaMemcpyAsync(im + 9 * ng, gidx.data(), sizeof(int) * 8 * ng, cudaMemcpyHostToDevice, d->s);
        cudaMemcpyAsync(im + 17 * ng, lstart.data(), sizeof(int) * (nlev + 1), cudaMemcpyHostToDevice, d->s);
        double *dm = d->g_dmem;
        cudaMemcpyAsync(dm, w.data(), sizeof(double) * 8 * ng, cudaMemcpyHostToDevice, d->s);
        cudaMemcpyAsync(dm + 8 * ng, wself.data(), sizeof(double) * ng, cudaMemcpyHostToDevice, d->s);
        cudaMemcpyAsync(d->g_kind, kind.data(), 8 * ng, cudaMemcpyHostToDevice, d->s);
        d->ghost_level_start = lstart;
        d->gargs = GhostArgs{ng, nlev, im + 17 * ng, im, im + ng, d->g_kind, dm, dm + 8 * ng, dm + 9 * ng,
                             d->ghost_level_start.data()};
        d->g_gidx = im + 9 * ng;
        d->g_gw = dm;
        d->g_gwself = dm + 8 * ng;
    }
    cudaMemcpyAsync(d->gid, hgid.data(), sizeof(int) * n, cudaMemcpyHostToDevice, d->s);
    return cuda_check(sv, cudaStreamSynchronize(d->s), "ghost tables");
}

// 1/coeffsum of fluid rows and the host p_coeffsum (src/ibm3d_setup.c:1641-1649).
void build_coeffsum(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    const long long n = d->g.ncell;
    std::vector<uint8_t> fl(n);
    cudaMemcpyAsync(fl.data(), d->flag, n, cudaMemcpyDeviceToHost, d->s);
    cudaStreamSynchronize(d->s);
    std::vector<double> dinv(n, 0.0);
    std::fill(sv->p_coeffsum, sv->p_coeffsum + n, 0.0);
    bool singular = true;
    for (int f = 0; f < 6; f++)
        if (sv->bc[f].type == BC_PRESSURE || sv->bc[f].type == BC_VELOCITY_PERIODIC) singular = false;
    for (int i = 0; i < sv->Nx; i++)
        for (int j = 0; j < sv->Ny; j++)
            for (int k = 0; k < sv->Nz; k++) {
                const long long P = cidx(d->g, i, j, k);
                if (singular && i == 0 && j == 0 && k == 0) continue;
                if (fl[P] != FLUID) continue;
                const double cs = sv->ky_N[j + 2] + sv->kx_E[i + 2] + sv->ky_S[j + 2] + sv->kx_W[i + 2] +
                                  sv->kz_D[k + 2] + sv->kz_U[k + 2];
                sv->p_coeffsum[P] = cs;
                dinv[P] = 1.0 / cs;
            }
    for (long long P = 0; P < n; P++) sv->flag[P] = fl[P];
    cudaMemcpyAsync(d->dinv, dinv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, d->s);
    cudaStreamSynchronize(d->s);
}

// Operator tables of both precisions and the two OpT views of them.
bool build_ops(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    const Grid &g = d->g;
    const long long n = g.ncell;
    const int ng = d->nghost;
    const int Ns[3] = {sv->Nx, sv->Ny, sv->Nz};
    const double *KM[3] = {sv->kx_W, sv->ky_S, sv->kz_D}, *KP[3] = {sv->kx_E, sv->ky_N, sv->kz_U};
    const double *D[3] = {sv->dx, sv->dy, sv->dz};
    size_t n64 = 0, n32 = 0;
    for (int a = 0; a < 3; a++) {
        n64 += Ns[a] + 4;
        n32 += 4 * (size_t)(Ns[a] + 4);
    }
    n32 += 2 * (size_t)n + 9 * (size_t)ng;
    std::vector<double> h64(n64, 0.0);
    std::vector<float> h32(n32, 0.0f);
    // Double-float tables: the FP64 values of km, kp, ks, d per axis, then
    // dinv (n) and the ghost weights (9 per ghost), each split in two words.
    const size_t ndf = n32 - (size_t)n;
    std::vector<dfloat> hdf(ndf, dfloat(0));
    d->op64 = dmalloc<double>(sv, n64, "operator tables");
    d->op32 = dmalloc<float>(sv, n32, "operator tables");
    d->opdf = dmalloc<dfloat>(sv, ndf, "operator tables");
    if (!d->op64 || !d->op32 || !d->opdf) return false;
    OpT<double> &A = d->A64;
    OpT<float> &B = d->A32;
    OpT<dfloat> &C = d->Adf;
    A = OpT<double>{};
    B = OpT<float>{};
    C = OpT<dfloat>{};
    size_t o64 = 0, o32 = 0;
    for (int a = 0; a < 3; a++) {
        const int m = Ns[a] + 4;
        double *ks = &h64[o64];
        float *km = &h32[o32], *kp = km + m, *ks32 = km + 2 * m, *dd = km + 3 * m;
        dfloat *kmd = &hdf[o32], *kpd = kmd + m, *ksd = kmd + 2 * m, *ddd = kmd + 3 * m;
        for (int q = 0; q < m; q++) {
            ks[q] = KM[a][q] + KP[a][q];
            km[q] = (float)KM[a][q];
            kp[q] = (float)KP[a][q];
            ks32[q] = (float)ks[q];
            dd[q] = (float)D[a][q];
            kmd[q] = dfloat(KM[a][q]);
            kpd[q] = dfloat(KP[a][q]);
            ksd[q] = dfloat(ks[q]);
            ddd[q] = dfloat(D[a][q]);
        }
        A.km[a] = d->ax[a].km;
        A.kp[a] = d->ax[a].kp;
        A.d[a] = d->ax[a].d;
        A.ks[a] = d->op64 + o64;
        B.km[a] = d->op32 + o32;
        B.kp[a] = d->op32 + o32 + m;
        B.ks[a] = d->op32 + o32 + 2 * m;
        B.d[a] = d->op32 + o32 + 3 * m;
        C.km[a] = d->opdf + o32;
        C.kp[a] = d->opdf + o32 + m;
        C.ks[a] = d->opdf + o32 + 2 * m;
        C.d[a] = d->opdf + o32 + 3 * m;
        o64 += m;
        o32 += 4 * (size_t)m;
    }
    // FP32 dinv and the divergence weights 2 Re coeffsum.
    std::vector<double> dinv(n);
    cudaMemcpyAsync(dinv.data(), d->dinv, sizeof(double) * n, cudaMemcpyDeviceToHost, d->s);
    std::vector<double> gw(8 * (size_t)ng), gws(ng);
    if (ng > 0) {
        cudaMemcpyAsync(gw.data(), d->g_gw, sizeof(double) * 8 * ng, cudaMemcpyDeviceToHost, d->s);
        cudaMemcpyAsync(gws.data(), d->g_gwself, sizeof(double) * ng, cudaMemcpyDeviceToHost, d->s);
    }
    if (!cuda_check(sv, cudaStreamSynchronize(d->s), "operator tables")) return false;
    float *dinv32 = &h32[o32], *wdiv = dinv32 + n, *gw32 = wdiv + n, *gws32 = gw32 + 8 * (size_t)ng;
    for (long long P = 0; P < n; P++) {
        dinv32[P] = (float)dinv[P];
        wdiv[P] = (float)(2.0 * sv->Re * sv->p_coeffsum[P]);
    }
    for (size_t q = 0; q < gw.size(); q++) gw32[q] = (float)gw[q];
    for (int q = 0; q < ng; q++) gws32[q] = (float)gws[q];
    dfloat *dinvd = &hdf[o32], *gwd = dinvd + n, *gwsd = gwd + 8 * (size_t)ng;
    for (long long P = 0; P < n; P++) dinvd[P] = dfloat(dinv[P]);
    for (size_t q = 0; q < gw.size(); q++) gwd[q] = dfloat(gw[q]);
    for (int q = 0; q < ng; q++) gwsd[q] = dfloat(gws[q]);
    cudaMemcpyAsync(d->opdf, hdf.data(), sizeof(dfloat) * ndf, cudaMemcpyHostToDevice, d->s);
    cudaMemcpyAsync(d->op64, h64.data(), sizeof(double) * n64, cudaMemcpyHostToDevice, d->s);
    cudaMemcpyAsync(d->op32, h32.data(), sizeof(float) * n32, cudaMemcpyHostToDevice, d->s);
    float *f32 = d->op32 + o32;
    for (int f = 0; f < 6; f++) {
        const BCFace &F = d->bc.f[f];
        A.bc[f].type = B.bc[f].type = C.bc[f].type = F.type;
        for (int L = 0; L < 2; L++) {
            C.bc[f].dir_o[L] = dfloat(F.dir_o[L]);
            C.bc[f].dir_m[L] = dfloat(F.dir_m[L]);
            C.bc[f].ext_o[L] = dfloat(F.ext_o[L]);
            C.bc[f].ext_2[L] = dfloat(F.ext_2[L]);
            A.bc[f].dir_o[L] = F.dir_o[L];
            A.bc[f].dir_m[L] = F.dir_m[L];
            A.bc[f].ext_o[L] = F.ext_o[L];
            A.bc[f].ext_2[L] = F.ext_2[L];
            B.bc[f].dir_o[L] = (float)F.dir_o[L];
            B.bc[f].dir_m[L] = (float)F.dir_m[L];
            B.bc[f].ext_o[L] = (float)F.ext_o[L];
            B.bc[f].ext_2[L] = (float)F.ext_2[L];
        }
    }
    // Sweep geometry: interior tiles of SW_TK x SW_TJ columns by `pi` planes,
    // with `pi` lowered on small grids so that the interior alone fills the
    // GPU; then the outer cells in index order.
    SweepGeom sw{};
    sw.tk = (g.nz + SW_TK - 1) / SW_TK;
    sw.tj = (g.ny + SW_TJ - 1) / SW_TJ;
    sw.pi = 8;
    while (sw.pi > 1 && (long long)sw.tk * sw.tj * ((g.nx + sw.pi - 1) / sw.pi) < 1216) sw.pi /= 2;
    sw.ti = (g.nx + sw.pi - 1) / sw.pi;
    sw.nint = sw.tk * sw.tj * sw.ti;
    std::vector<int> outer;
    outer.reserve((size_t)(n - (long long)g.nx * g.ny * g.nz));
    for (long long P = 0; P < n; P++) {
        int i, j, k;
        cijk(g, P, i, j, k);
        if (i < 0 || i >= g.nx || j < 0 || j >= g.ny || k < 0 || k >= g.nz) outer.push_back((int)P);
    }
    sw.nout = (int)outer.size();
    sw.nblocks = sw.nint + (sw.nout + SW_THREADS - 1) / SW_THREADS;
    d->sweep_outer = dmalloc<int>(sv, std::max<size_t>(1, outer.size()), "sweep tables");
    if (!d->sweep_outer) return false;
    cudaMemcpyAsync(d->sweep_outer, outer.data(), sizeof(int) * outer.size(), cudaMemcpyHostToDevice, d->s);
    sw.outer = d->sweep_outer;
    A.sw = B.sw = sw;
    const FastDiv fdx = make_fastdiv((unsigned)g.sx), fdy = make_fastdiv((unsigned)g.sy);
    A.g = B.g = g;
    A.fdx = B.fdx = fdx;
    A.fdy = B.fdy = fdy;
    A.p_singular = B.p_singular = d->bc.p_singular;
    A.pinned = B.pinned = cidx(g, 0, 0, 0);
    A.flag = B.flag = d->flag;
    A.gid = B.gid = d->gid;
    A.gidx = B.gidx = d->g_gidx;
    A.gw = d->g_gw;
    A.gwself = d->g_gwself;
    A.dinv = d->dinv;
    B.dinv = f32;
    A.wdiv = B.wdiv = f32 + n;
    B.gw = ng ? f32 + 2 * n : nullptr;
    B.gwself = ng ? f32 + 2 * n + 8 * (size_t)ng : nullptr;
    // The double-float operator: the FP64 operator's index tables, its
    // values split in two words.
    C.g = g;
    C.fdx = fdx;
    C.fdy = fdy;
    C.sw = sw;
    C.p_singular = A.p_singular;
    C.pinned = A.pinned;
    C.flag = A.flag;
    C.gid = A.gid;
    C.gidx = A.gidx;
    C.wdiv = A.wdiv;
    C.dinv = d->opdf + o32;
    C.gw = ng ? d->opdf + o32 + n : nullptr;
    C.gwself = ng ? d->opdf + o32 + n + 8 * (size_t)ng : nullptr;
    return cuda_check(sv, cudaStreamSynchronize(d->s), "operator tables");
}

void swap3(double *a[3], double *b[3]) {
    for (int l = 0; l < 3; l++) std::swap(a[l], b[l]);
}

ConvArgs conv_args(ibm3d_device *d) {
    ConvArgs a{};
    for (int l = 0; l < 3; l++) {
        a.u[l] = d->u[l];
        a.U[l] = d->U[l];
        a.Np[l] = d->Np[l];
        a.N[l] = d->N[l];
        a.b[l] = d->b + l * d->g.ncell;
    }
    for (int t = 0; t < 6; t++) a.tau[t] = d->tau[t];
    a.p = d->p;
    a.force = d->force_d;
    return a;
}

Conv32Args conv32_args(ibm3d_device *d) {
    Conv32Args a{};
    for (int l = 0; l < 3; l++) {
        a.u[l] = d->u[l];
        a.U[l] = d->U[l];
        a.Np[l] = d->Np32[l];
        a.N[l] = d->N32[l];
    }
    for (int t = 0; t < 6; t++) a.tau[t] = d->tau[t];
    a.p = d->p;
    a.force = d->force_d;
    a.c = d->irmom.b32;
    return a;
}

void calc_tau(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    if (!d->les) return;
    TauArgs t{};
    for (int q = 0; q < 6; q++) t.tau[q] = d->tau[q];
    const double *u[3] = {d->u[0], d->u[1], d->u[2]};
    launch_smagorinsky(d->s, d->g, d->ax[0], d->ax[1], d->ax[2], d->flag, d->lvset, u, t, sv->turb_model.Cs);
}

// when: 0 at the step's start time (iterate prologue), 1 at its end.
void fill_outer(IBMSolver *sv, int when) {
    ibm3d_device *d = sv->dev;
    launch_fill_outer(d->s, d->g, d->bc, d->u, d->p, when);
}

// ------------------------------------------------- VAL_FUNC sampling ---
// The reference evaluates VAL_FUNC callbacks inside its loops
// (src/ibm3d_fracstep.c:1978-2035): boundary values at the face centre of
// each outer line at the current time (momentum right-hand side and outer
// fills) and at time + dt (pressure-correction right-hand side), the body
// force at every cell centre at the current time.  Here the host samples
// them once per step into pinned buffers that are copied to the device
// before the step's kernels; the kernels read the samples where they would
// read the constant values.
bool sampled_face(const IBMSolver *sv, int f) {
    const IBMSolverBC &B = sv->bc[f];
    return B.val_type == VAL_FUNC && (B.type == BC_VELOCITY_COMPONENT || B.type == BC_PRESSURE ||
                                      B.type == BC_VELOCITY_PERIODIC);
}

bool alloc_samples(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    size_t n = 0;
    for (int f = 0; f < 6; f++) {
        d->smp_face[f] = sampled_face(sv, f);
        d->bc.f[f].scur = d->bc.f[f].snxt = nullptr;
        d->bc.f[f].nt = face_lines(d->g, f);
        d->smp_off[f] = n;
        if (d->smp_face[f]) n += 8 * (size_t)d->bc.f[f].nt;
    }
    d->smp_n = n;
    if (n) {
        d->smp_d = dmalloc<double>(sv, n, "boundary samples");
        if (!d->smp_d || !cuda_check(sv, cudaMallocHost(&d->smp_h, n * sizeof(double)), "boundary samples")) return false;
        memset(d->smp_h, 0, n * sizeof(double));
        for (int f = 0; f < 6; f++)
            if (d->smp_face[f]) {
                d->bc.f[f].scur = d->smp_d + d->smp_off[f];
                d->bc.f[f].snxt = d->smp_d + d->smp_off[f] + 4 * (size_t)d->bc.f[f].nt;
            }
    }
    if (sv->ext_force.val_type == VAL_FUNC) {
        const size_t m = 3 * (size_t)d->g.ncell;
        d->force_d = dmalloc<double>(sv, m, "force samples");
        if (!d->force_d || !cuda_check(sv, cudaMallocHost(&d->force_h, m * sizeof(double)), "force samples"))
            return false;
        memset(d->force_h, 0, m * sizeof(double));
    }
    return true;
}

// Values of face f at time t into dst (4 x nt: u1, u2, u3, p).
void sample_face(const IBMSolver *sv, int f, double t, double *dst) {
    const IBMSolverBC &B = sv->bc[f];
    const Grid &g = sv->dev->g;
    const int nt = face_lines(g, f), ax = face_axis(f);
    const bool low = face_low(f);
    const bool vel = B.type == BC_VELOCITY_COMPONENT;
    const int na = ax == 0 ? g.ny + 4 : g.nx + 4, nb = ax == 2 ? g.ny + 4 : g.nz + 4;
    for (int a = 0; a < na; a++)
        for (int b = 0; b < nb; b++) {
            double x, y, z;
            if (ax == 0) { x = low ? sv->xmin : sv->xmax; y = sv->yc[a]; z = sv->zc[b]; }
            else if (ax == 1) { x = sv->xc[a]; y = low ? sv->ymin : sv->ymax; z = sv->zc[b]; }
            else { x = sv->xc[a]; y = sv->yc[b]; z = low ? sv->zmin : sv->zmax; }
            const int line = a * nb + b;
            dst[line] = vel ? B.func_u1(t, x, y, z) : 0.0;
            dst[nt + line] = vel ? B.func_u2(t, x, y, z) : 0.0;
            dst[2 * nt + line] = vel ? B.func_u3(t, x, y, z) : 0.0;
            dst[3 * nt + line] = vel ? 0.0 : B.func_p(t, x, y, z);
        }
}

// Samples for a step from time t0 to t1 (the iterate prologue passes its
// start time and the first step's end time), copied on stream st.
void prepare_samples(IBMSolver *sv, cudaStream_t st, double t0, double t1) {
    ibm3d_device *d = sv->dev;
    if (d->smp_n) {
        const bool have0 = d->smp_valid && d->smp_t[0] == t0, have1 = d->smp_valid && d->smp_t[1] == t1;
        if (!(have0 && have1)) {
            const bool rotate = d->smp_valid && d->smp_t[1] == t0;
            for (int f = 0; f < 6; f++) {
                if (!d->smp_face[f]) continue;
                const size_t m = 4 * (size_t)d->bc.f[f].nt;
                double *cur = d->smp_h + d->smp_off[f], *nxt = cur + m;
                if (!have0) {
                    if (rotate) memcpy(cur, nxt, m * sizeof(double));
                    else sample_face(sv, f, t0, cur);
                }
                if (!have1) sample_face(sv, f, t1, nxt);
            }
            d->smp_t[0] = t0;
            d->smp_t[1] = t1;
            d->smp_valid = true;
        }
        if (!(d->smp_dev_valid && d->smp_dev_t[0] == t0 && d->smp_dev_t[1] == t1)) {
            cudaMemcpyAsync(d->smp_d, d->smp_h, d->smp_n * sizeof(double), cudaMemcpyHostToDevice, st);
            d->smp_dev_t[0] = t0;
            d->smp_dev_t[1] = t1;
            d->smp_dev_valid = true;
        }
    }
    if (d->force_d) {
        if (!(d->force_valid && d->force_t == t0)) {
            const Grid &g = d->g;
            const IBMSolverForceFunc fn[3] = {sv->ext_force.func_f1, sv->ext_force.func_f2, sv->ext_force.func_f3};
            for (int i = 0; i < g.nx; i++)
                for (int j = 0; j < g.ny; j++)
                    for (int k = 0; k < g.nz; k++) {
                        const long long P = cidx(g, i, j, k);
                        const double x = sv->xc[i + 2], y = sv->yc[j + 2], z = sv->zc[k + 2];
                        for (int l = 0; l < 3; l++) d->force_h[l * g.ncell + P] = fn[l](t0, x, y, z);
                    }
            d->force_t = t0;
            d->force_valid = true;
        }
        if (!(d->force_dev_valid && d->force_dev_t == t0)) {
            cudaMemcpyAsync(d->force_d, d->force_h, 3 * d->g.ncell * sizeof(double), cudaMemcpyHostToDevice, st);
            d->force_dev_t = t0;
            d->force_dev_valid = true;
        }
    }
}

void ghost_update(IBMSolver *sv, bool solids) {
    ibm3d_device *d = sv->dev;
    if (solids) launch_solid_nan(d->s, d->g, d->flag, d->u, d->p);
    launch_ghost_update(d->s, d->gargs, d->u, d->p);
}

// --------------------------------------------------------- time step ---
// Stages of one fractional step (src/ibm3d_fracstep.c:60-74).
bool mom_ir(const ibm3d_device *d);

SolveParams mom_params(IBMSolver *sv) {
    SolveParams pm;
    pm.tol = sv->tol;
    pm.maxit = sv->dev->maxit_mom;
    pm.inner_tol = sv->dev->inner_tol[0];
    pm.max_outer = sv->dev->max_outer;
    pm.prof = &sv->dev->prof;
    pm.x_given = mom_ir(sv->dev) && sv->dev->warm_start;
    return pm;
}

// The momentum unknown u* starts from the current velocity u^n (u* - u^n
// is O(dt)) when the solve takes an initial guess.
void momentum_guess(IBMSolver *sv, const SolveParams &pm) {
    ibm3d_device *d = sv->dev;
    if (pm.x_given) launch_velocity_guess(d->s, d->g, d->u, d->ustar);
}

bool pres_gmres(const IBMSolver *sv);

SolveParams pres_params(IBMSolver *sv) {
    SolveParams pp = mom_params(sv);
    // The mixed modes start from the last step's pressure increment.
    pp.x_given = sv->dev->precision != IBM3D_FP64 && sv->dev->warm_start && !pres_gmres(sv);
    pp.inner_tol = sv->dev->inner_tol[1];
    pp.maxit = sv->dev->maxit_p;
    pp.divtol = sv->dev->divtol;
    if (pp.divtol > 0) pp.tol = 0.0;  // the divergence rule replaces the relative-residual rule
    return pp;
}

// With IBMSolver_set_pressure_guess(s, 1) a warm-started pressure solve
// starts from the linear extrapolation of the last two increments.
void pressure_guess(IBMSolver *sv, const SolveParams &pp) {
    ibm3d_device *d = sv->dev;
    if (pp.x_given && d->p_guess == 1) launch_pressure_guess(d->s, d->g.ncell, d->pp, d->pp_prev, d->pp_hist);
}

bool use_mg(const IBMSolver *sv) { return sv->precond_type == PRECOND_AMG || sv->linear_solver_type == SOLVER_AMG; }

// Pressure solves with SOLVER_GMRES: flexible GMRES in FP64 (any precision
// mode; the mixed modes precondition it with the FP32 multigrid).
bool pres_gmres(const IBMSolver *sv) { return sv->linear_solver_type == SOLVER_GMRES; }

// Which solve runs as FP64 refinement around FP32 BiCGSTAB, and which step
// has the FP32 explicit stages and the FP32 increment momentum solve.
bool mom_ir(const ibm3d_device *d) { return d->precision == IBM3D_MIXED || d->precision == IBM3D_MIXED_MG; }
bool step32(const ibm3d_device *d) { return d->precision == IBM3D_MIXED32 || d->precision == IBM3D_MIXED32_IR; }
bool pres_ir(const IBMSolver *sv) {
    return (sv->dev->precision == IBM3D_MIXED || sv->dev->precision == IBM3D_MIXED32_IR) && !pres_gmres(sv);
}

// The IBM3D_MIXED32 pressure BiCGSTAB on double-float vectors
// (IBMSolver_set_pressure_vectors; with the FP32 multigrid, whose FP32
// output the double-float solve stores as it comes), and its
// preconditioner.
bool pres_df(const IBMSolver *sv) {
    const ibm3d_device *d = sv->dev;
    return d->precision == IBM3D_MIXED32 && d->pvec == IBM3D_PVEC_DFLOAT && !pres_gmres(sv) && use_mg(sv);
}
Preconditioner<dfloat> *pres_pcdf(IBMSolver *sv) { return &sv->dev->pcdf; }

// Preconditioner of an FP64 pressure Krylov solve.
Preconditioner<double> *pres_pc64(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    if (!use_mg(sv)) return nullptr;
    return d->precision != IBM3D_FP64 ? (Preconditioner<double> *)&d->pc64 : (Preconditioner<double> *)d->mg;
}

void stage_rhs(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    Prof &pf = d->prof;
    const double f[3] = {sv->ext_force.const_f1, sv->ext_force.const_f2, sv->ext_force.const_f3};
    int t = pf.begin("tau");
    calc_tau(sv);
    pf.end(t);
    t = pf.begin("conv_rhs");
    if (step32(d))
        launch_conv_rhs32(d->s, d->g, d->axf, d->A32, d->bc, d->flag, conv32_args(d), sv->dt, f, d->les,
                          d->red_partials, d->red_counter, d->irmom.scal);
    else
        launch_conv_rhs(d->s, d->g, d->ax[0], d->ax[1], d->ax[2], d->bc, d->flag, conv_args(d), sv->dt, f, d->les);
    pf.end(t);
}

void stage_ustar(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    if (step32(d)) {
        Ustar32Args ua{};
        for (int l = 0; l < 3; l++) {
            ua.u[l] = d->u[l];
            ua.e[l] = d->irmom.e32 + l * d->g.ncell;
            ua.Us[l] = d->Us[l];
        }
        ua.p = d->p;
        ua.dinv = d->dinv;
        ua.b = d->b;
        const int t = d->prof.begin("ustar_prhs");
        launch_ustar_prhs32_tiled(d->s, d->g, d->axf, d->ax, d->bc, d->flag, ua, d->ut32, sv->dt, sv->Re,
                                  d->A32.sw.outer, d->A32.sw.nout);
        d->prof.end(t);
        return;
    }
    UstarArgs ua{};
    for (int l = 0; l < 3; l++) {
        ua.us[l] = d->ustar + l * d->g.ncell;
        ua.Us[l] = d->Us[l];
    }
    ua.p = d->p;
    ua.b = d->b;
    const int t = d->prof.begin("ustar_prhs");
    launch_ustar_prhs(d->s, d->g, d->ax[0], d->ax[1], d->ax[2], d->bc, d->flag, ua, sv->dt, sv->Re);
    d->prof.end(t);
}

void stage_next(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    if (step32(d)) {
        Next32Args na{};
        for (int l = 0; l < 3; l++) {
            na.u[l] = d->u[l];
            na.e[l] = d->irmom.e32 + l * d->g.ncell;
            na.Us[l] = d->Us[l];
            na.un[l] = d->un[l];
            na.Un[l] = d->Un[l];
        }
        na.p = d->p;
        na.pp = d->pp;
        na.pn = d->pn;
        const int t = d->prof.begin("update_next");
        launch_update_next_tiled(d->s, d->g, d->ax, d->dta, d->axf, d->bc, d->flag, nullptr, &na, sv->dt,
                                 d->red_partials, d->red_counter, d->maxdiv_d);
        d->prof.end(t);
        return;
    }
    NextArgs na{};
    for (int l = 0; l < 3; l++) {
        na.us[l] = d->ustar + l * d->g.ncell;
        na.Us[l] = d->Us[l];
        na.un[l] = d->un[l];
        na.Un[l] = d->Un[l];
    }
    na.p = d->p;
    na.pp = d->pp;
    na.pn = d->pn;
    const int t = d->prof.begin("update_next");
    launch_update_next_tiled(d->s, d->g, d->ax, d->dta, d->axf, d->bc, d->flag, &na, nullptr, sv->dt,
                             d->red_partials, d->red_counter, d->maxdiv_d);
    d->prof.end(t);
}

void swap_fields(ibm3d_device *d) {
    swap3(d->u, d->un);
    swap3(d->U, d->Un);
    std::swap(d->p, d->pn);
    swap3(d->N, d->Np);
    for (int l = 0; l < 3; l++) std::swap(d->N32[l], d->Np32[l]);
}

// Non-finite residuals mean NaN or Inf reached the solve (the initial
// state, boundary values or force, or a run that diverged): the reference
// would carry them on silently; here they end the iterate call with a
// status.  Non-convergence warns and continues, as in the reference
// (src/ibm3d_fracstep.c:363-369, 673-679, the same messages).
void check_mom(IBMSolver *sv, int rc) {
    for (int l = 0; l < 3; l++)
        if (!std::isfinite(sv->dev->rep_mom.relres[l])) {
            set_status(sv, IBM3D_ENONFINITE,
                       "non-finite residual in the u%d_star solve at step %d: NaN or Inf in the state, boundary "
                       "data or force",
                       l, sv->iter + 1);
            return;
        }
    if (rc == 1) {
        for (int l = 0; l < 3; l++)
            if (sv->dev->rep_mom.relres[l] >= sv->tol) fprintf(stderr, "warning: u%d_star did not converge\n", l);
    } else if (rc == 2) {
        set_status(sv, IBM3D_EBREAKDOWN, "breakdown in the momentum solve");
    }
}

void check_pres(IBMSolver *sv, int rc) {
    if (!std::isfinite(sv->dev->rep_p.relres[0])) {
        set_status(sv, IBM3D_ENONFINITE,
                   "non-finite residual in the p_prime solve at step %d: NaN or Inf in the state, boundary data or "
                   "force",
                   sv->iter + 1);
        return;
    }
    if (rc == 1) fprintf(stderr, "warning: p_prime did not converge\n");
    else if (rc == 2) set_status(sv, IBM3D_EBREAKDOWN, "breakdown in the pressure solve");
}

// One fractional step, host-sequenced (used while stage profiling is on).
void one_step(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    Prof &pf = d->prof;
    stage_rhs(sv);
    const SolveParams pm = mom_params(sv);
    int t = pf.begin("mom_solve");
    momentum_guess(sv, pm);
    int rc = step32(d)  ? solve_inc(d->s, d->A32, OP_MOM, d->irmom, pm, d->rep_mom)
             : mom_ir(d) ? solve_ir(d->s, d->A64, d->A32, OP_MOM, d->irmom, d->b, d->ustar, pm, nullptr, d->rep_mom)
                         : bicgstab<double>(d->s, d->A64, OP_MOM, d->kmom, d->b, d->ustar, pm, nullptr, d->rep_mom);
    pf.end(t);
    check_mom(sv, rc);
    stage_ustar(sv);
    const SolveParams pp = pres_params(sv);
    pressure_guess(sv, pp);
    t = pf.begin("p_solve");
    if (pres_gmres(sv))
        rc = gmres(d->s, d->A64, OP_PRES, d->gm, d->b, d->pp, pp, pres_pc64(sv), d->rep_p);
    else if (pres_ir(sv))
        rc = solve_ir(d->s, d->A64, d->A32, OP_PRES, d->irpres, d->b, d->pp, pp, use_mg(sv) ? d->mg32 : nullptr,
                      d->rep_p);
    else if (pres_df(sv))
        rc = bicgstab_df(d->s, d->Adf, OP_PRES, d->kpres_df, d->pp_df, d->b, d->pp, pp, pres_pcdf(sv), d->rep_p);
    else
        rc = bicgstab<double>(d->s, d->A64, OP_PRES, d->kpres, d->b, d->pp, pp, pres_pc64(sv), d->rep_p);
    pf.end(t);
    check_pres(sv, rc);
    stage_next(sv);
    swap_fields(d);
}

GraphSig graph_sig(const IBMSolver *sv) {
    GraphSig g;
    memset(&g, 0, sizeof g);
    g.precision = sv->dev->precision;
    g.warm = sv->dev->warm_start;
    g.les = sv->dev->les;
    g.use_mg = use_mg(sv);
    g.tol = sv->tol;
    g.divtol = sv->dev->divtol;
    g.Re = sv->Re;
    g.dt = sv->dt;
    g.f[0] = sv->ext_force.const_f1;
    g.f[1] = sv->ext_force.const_f2;
    g.f[2] = sv->ext_force.const_f3;
    g.cs = sv->turb_model.Cs;
    g.inner_tol[0] = sv->dev->inner_tol[0];
    g.inner_tol[1] = sv->dev->inner_tol[1];
    g.max_outer = sv->dev->max_outer;
    g.solver = sv->linear_solver_type;
    g.gm_restart = sv->dev->gm_restart;
    g.p_guess = sv->dev->p_guess;
    g.pvec = sv->dev->pvec;
    return g;
}

// Records one step (everything one_step + fill_outer + ghost_update do)
// into a graph; the field pointers are left as they were.
// Records one step onto d->s, which must be capturing (its own graph or a
// batch graph it joined); fills G's keys and launch accounting.
bool record_step_into(IBMSolver *sv, StepGraph &G) {
    ibm3d_device *d = sv->dev;
    long long count = 0;
    g_redirect = &count;
    bool ok = true;
    int mf = 0, mo = 0, mi = 0, pf = 0, po = 0, pi = 0;
    if (ok) {
        stage_rhs(sv);
        SolveParams pm = mom_params(sv);
        pm.prof = nullptr;
        momentum_guess(sv, pm);
        if (step32(d))
            ok = record_inc(d->s, d->aux, d->A32, OP_MOM, d->irmom, pm, &mf, &mi) == 0;
        else if (mom_ir(d))
            ok = record_ir(d->s, d->aux, d->A64, d->A32, OP_MOM, d->irmom, d->b, d->ustar, pm, nullptr, &mf, &mo,
                           &mi) == 0;
        else
            ok = record_bicgstab<double>(d->s, d->aux, d->A64, OP_MOM, d->kmom, d->b, d->ustar, pm, nullptr, &mf,
                                         &mi) == 0;
    }
    if (ok) {
        stage_ustar(sv);
        SolveParams pp = pres_params(sv);
        pp.prof = nullptr;
        pressure_guess(sv, pp);
        if (pres_gmres(sv))
            ok = record_gmres(d->s, d->aux, d->A64, OP_PRES, d->gm, d->b, d->pp, pp, pres_pc64(sv), &pf, &po,
                              &pi) == 0;
        else if (pres_ir(sv))
            ok = record_ir(d->s, d->aux, d->A64, d->A32, OP_PRES, d->irpres, d->b, d->pp, pp,
                           use_mg(sv) ? d->mg32 : nullptr, &pf, &po, &pi) == 0;
        else if (pres_df(sv))
            ok = record_bicgstab_df(d->s, d->aux, d->Adf, OP_PRES, d->kpres_df, d->pp_df, d->b, d->pp, pp,
                                    pres_pcdf(sv), &pf, &pi) == 0;
        else
            ok = record_bicgstab<double>(d->s, d->aux, d->A64, OP_PRES, d->kpres, d->b, d->pp, pp, pres_pc64(sv),
                                         &pf, &pi) == 0;
    }
    if (ok) {
        stage_next(sv);
        swap_fields(d);
        fill_outer(sv, 1);
        ghost_update(sv, false);
        cudaMemcpyAsync(d->maxdiv_h, d->maxdiv_d, sizeof(double), cudaMemcpyDeviceToHost, d->s);
        swap_fields(d);
    }
    g_redirect = nullptr;
    if (!ok) return false;
    G.key[0] = d->u[0];
    G.key[1] = d->U[0];
    G.key[2] = d->p;
    G.key[3] = d->N[0];
    G.mom_iter = mi;
    G.mom_outer = mo;
    G.p_iter = pi;
    G.p_outer = po;
    // Loop bodies were recorded once each; the rest runs once per step.
    G.fixed = (int)(count - mi - mo - pi - po);
    return true;
}

// Ends any capture still open on the solver's aux streams (left by a
// recording that failed half-way) and discards what it captured.
void close_open_captures(ibm3d_device *d) {
    for (cudaStream_t a : d->aux) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (a && cudaStreamIsCapturing(a, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(a, &g);
        }
    }
    cudaGetLastError();
}

bool record_step(IBMSolver *sv, StepGraph &G) {
    ibm3d_device *d = sv->dev;
    bool ok = cudaStreamBeginCapture(d->s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) ok = record_step_into(sv, G);
    close_open_captures(d);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(d->s, &graph);
    ok = ok && ec == cudaSuccess && graph;
    if (ok) ok = cudaGraphInstantiate(&G.exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return ok;
}

bool has_key(const StepGraph &g, const ibm3d_device *d) {
    return g.key[0] == d->u[0] && g.key[1] == d->U[0] && g.key[2] == d->p && g.key[3] == d->N[0];
}

// After a recorded step ran and its stream is synchronised: the solve
// reports, warnings, launch count and the pointer swaps.
void finish_step(IBMSolver *sv, const StepGraph &G) {
    ibm3d_device *d = sv->dev;
    long long launches = G.fixed;
    int rc;
    if (step32(d)) {
        rc = report_inc(d->irmom, sv->tol, d->rep_mom);
    } else if (mom_ir(d)) {
        rc = report(d->irmom, d->rep_mom);
        launches += (long long)d->rep_mom.outer * G.mom_outer;
    } else {
        rc = report(d->kmom, d->rep_mom);
    }
    launches += (long long)std::max({d->rep_mom.iters[0], d->rep_mom.iters[1], d->rep_mom.iters[2]}) * G.mom_iter;
    check_mom(sv, rc);
    if (pres_gmres(sv)) {
        rc = report(d->gm, d->rep_p);
        launches += (long long)d->rep_p.outer * G.p_outer;
    } else if (pres_ir(sv)) {
        rc = report(d->irpres, d->rep_p);
        launches += (long long)d->rep_p.outer * G.p_outer;
    } else {
        rc = report(d->kpres, d->rep_p);
    }
    launches += (long long)d->rep_p.iters[0] * G.p_iter;
    check_pres(sv, rc);
    note_launches((int)launches);
    swap_fields(d);
}

// One step through its recorded graph.  Returns false when recording
// failed (the caller then runs the step host-sequenced).
// The recorded step for the solver's current field buffers (recorded on
// first use); null when recording failed.
StepGraph *step_graph(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    const GraphSig sig = graph_sig(sv);
    if (!(sig == d->gsig)) {
        drop_graphs(d);
        d->gsig = sig;
    }
    for (auto &g : d->graphs)
        if (has_key(g, d)) return &g;
    StepGraph ng;
    if (!record_step(sv, ng)) return nullptr;
    d->graphs.push_back(ng);
    return &d->graphs.back();
}

bool graph_step(IBMSolver *sv) {
    ibm3d_device *d = sv->dev;
    StepGraph *G = step_graph(sv);
    if (!G) {
        fprintf(stderr, "warning: CUDA graph recording failed; stepping without graphs\n");
        d->use_graphs = false;
        return false;
    }
    if (!cuda_check(sv, cudaGraphLaunch(G->exec, d->s), "graph launch")) return true;
    if (!cuda_check(sv, cudaStreamSynchronize(d->s), "time step")) return true;
    finish_step(sv, *G);
    return true;
}

void print_row(IBMSolver *sv, int i, long elapsed_ms) {
    ibm3d_device *d = sv->dev;
    // The reference's columns (src/ibm3d_fracstep.c:77-105), then this
    // step's max|div U^{n+1}| over fluid cells, measured by k_update_next.
    if (sv->iter % 10 == 1 || i == 1) {
        printf("\n  iter       u1 res       u2 res       u3 res        p res       time   max|div U|\n");
        printf("----------------------------------------------------------------------------------\n");
    }
    long hour = elapsed_ms / 3600000, min = elapsed_ms / 60000 % 60;
    long sec = elapsed_ms / 1000 % 60 + (elapsed_ms % 1000 > 500);
    if (sec >= 60) { sec -= 60; min += 1; }
    if (min >= 60) { min -= 60; hour += 1; }
    printf("%6d   %10.4e   %10.4e   %10.4e   %10.4e   %02ld:%02ld:%02ld   %10.4e\n", sv->iter, d->rep_mom.relres[0],
           d->rep_mom.relres[1], d->rep_mom.relres[2], d->rep_p.relres[0], hour, min, sec, d->max_div);
}

bool check_ready(IBMSolver *sv, const char *fn) {
    if (!sv || !sv->dev || !sv->dev->assembled) {
        set_status(sv, IBM3D_EARG, "%s called before IBMSolver_assemble", fn);
        return false;
    }
    return true;
}

void upload_state(IBMSolver *sv, const double *u1, const double *u2, const double *u3, const double *p) {
    ibm3d_device *d = sv->dev;
    const size_t b = sizeof(double) * d->g.ncell;
    cudaMemcpyAsync(d->u[0], u1, b, cudaMemcpyHostToDevice, d->s);
    cudaMemcpyAsync(d->u[1], u2, b, cudaMemcpyHostToDevice, d->s);
    cudaMemcpyAsync(d->u[2], u3, b, cudaMemcpyHostToDevice, d->s);
    cudaMemcpyAsync(d->p, p, b, cudaMemcpyHostToDevice, d->s);
    // A new run: the pressure increment, a warm start's initial guess,
    // starts from zero, with no history to extrapolate from.
    cudaMemsetAsync(d->pp, 0, b, d->s);
    cudaMemsetAsync(d->pp_prev, 0, b, d->s);
    cudaMemsetAsync(d->pp_hist, 0, sizeof(int), d->s);
    cuda_check(sv, cudaStreamSynchronize(d->s), "state upload");
    sv->iter = 0;
    sv->time = 0;
}

}  // namespace

extern "C" {

// ------------------------------------------------------------ setup ---
IBMSolver *IBMSolver_new(const int num_process, const int rank, const int Px, const int Py, const int Pz) {
    IBMSolver *s = (IBMSolver *)calloc(1, sizeof(IBMSolver));
    s->dev = new ibm3d_device();
    if (const char *e = getenv("IBM3D_NO_ABORT")) s->dev->abort_on_error = atoi(e) == 0;
    if (rank < 0 || rank > num_process) {
        set_status(s, IBM3D_EARG, "Invalid rank: %d", rank);
        return s;
    }
    s->num_process = num_process;
    s->rank = rank;
    // One GPU holds the whole domain: the decomposition collapses to 1x1x1.
    (void)Px; (void)Py; (void)Pz;
    s->Px = s->Py = s->Pz = 1;
    s->ri = s->rj = s->rk = 0;
    s->ext_force.val_type = VAL_CONST;
    s->turb_model.type = TURBMODEL_NONE;
    s->linear_solver_type = SOLVER_BiCGSTAB;
    s->precond_type = PRECOND_AMG;
    s->tol = 1e-6;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_status(s, IBM3D_ECUDA, "no CUDA device available: the GB300 path has no CPU fallback");
        return s;
    }
    cudaGetDevice(&s->dev->dev_id);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, s->dev->dev_id) == cudaSuccess)
        snprintf(s->dev->dev_name, sizeof s->dev->dev_name, "%s (sm_%d%d)", prop.name, prop.major, prop.minor);
    cuda_check(s, cudaStreamCreateWithFlags(&s->dev->s, cudaStreamNonBlocking), "stream");
    s->dev->prof.s = s->dev->s;
    return s;
}

void IBMSolver_destroy(IBMSolver *s) {
    if (!s) return;
    if (s->dev) {
        release_device(s->dev);
        delete s->dev;
    }
    free(s->dx); free(s->dy); free(s->dz);
    free(s->xc); free(s->yc); free(s->zc);
    free(s->kx_W); free(s->kx_E); free(s->ky_S); free(s->ky_N); free(s->kz_D); free(s->kz_U);
    free(s->flag); free(s->lvset); free(s->p_coeffsum);
    free(s->u1); free(s->u2); free(s->u3); free(s->p);
    free(s);
}

void IBMSolver_set_grid(IBMSolver *s, const int Nx, const int Ny, const int Nz, const double *xf, const double *yf,
                        const double *zf) {
    if (Nx < 2 || Ny < 2 || Nz < 2) {
        set_status(s, IBM3D_EARG, "grid must have at least 2 cells per axis (got %d x %d x %d)", Nx, Ny, Nz);
        return;
    }
    s->Nx_global = s->Nx = Nx;
    s->Ny_global = s->Ny = Ny;
    s->Nz_global = s->Nz = Nz;
    auto alloc1 = [](int n) { return (double *)calloc(n + 4, sizeof(double)); };
    s->dx = alloc1(Nx); s->xc = alloc1(Nx); s->kx_W = alloc1(Nx); s->kx_E = alloc1(Nx);
    s->dy = alloc1(Ny); s->yc = alloc1(Ny); s->ky_S = alloc1(Ny); s->ky_N = alloc1(Ny);
    s->dz = alloc1(Nz); s->zc = alloc1(Nz); s->kz_D = alloc1(Nz); s->kz_U = alloc1(Nz);
    for (int i = 0; i < Nx; i++) {
        s->dx[i + 2] = xf[i + 1] - xf[i];
        s->xc[i + 2] = (xf[i + 1] + xf[i]) / 2;
    }
    for (int j = 0; j < Ny; j++) {
        s->dy[j + 2] = yf[j + 1] - yf[j];
        s->yc[j + 2] = (yf[j + 1] + yf[j]) / 2;
    }
    for (int k = 0; k < Nz; k++) {
        s->dz[k + 2] = zf[k + 1] - zf[k];
        s->zc[k + 2] = (zf[k + 1] + zf[k]) / 2;
    }
    s->xmin = xf[0]; s->xmax = xf[Nx];
    s->ymin = yf[0]; s->ymax = yf[Ny];
    s->zmin = zf[0]; s->zmax = zf[Nz];
    const size_t n = (size_t)ncell_of(s);
    s->flag = (int *)calloc(n, sizeof(int));
    s->lvset = (double *)calloc(n, sizeof(double));
    s->p_coeffsum = (double *)calloc(n, sizeof(double));
    s->u1 = (double *)calloc(n, sizeof(double));
    s->u2 = (double *)calloc(n, sizeof(double));
    s->u3 = (double *)calloc(n, sizeof(double));
    s->p = (double *)calloc(n, sizeof(double));
}

void IBMSolver_set_params(IBMSolver *s, const double Re, const double dt) {
    s->Re = Re;
    s->dt = dt;
}

void IBMSolver_set_ext_force(IBMSolver *s, IBMSolverValType val_type, ...) {
    va_list ap;
    va_start(ap, val_type);
    s->ext_force.val_type = val_type;
    if (val_type == VAL_CONST) {
        s->ext_force.const_f1 = va_arg(ap, double);
        s->ext_force.const_f2 = va_arg(ap, double);
        s->ext_force.const_f3 = va_arg(ap, double);
    } else {
        s->ext_force.func_f1 = va_arg(ap, IBMSolverForceFunc);
        s->ext_force.func_f2 = va_arg(ap, IBMSolverForceFunc);
        s->ext_force.func_f3 = va_arg(ap, IBMSolverForceFunc);
    }
    va_end(ap);
}

void IBMSolver_set_turb_model(IBMSolver *s, IBMSolverTurbModelType type, ...) {
    va_list ap;
    va_start(ap, type);
    s->turb_model.type = type;
    if (type == TURBMODEL_SMAGORINSKY) s->turb_model.Cs = va_arg(ap, double);
    else if (type != TURBMODEL_NONE) set_status(s, IBM3D_EUNSUPPORTED, "turbulence model %d is not implemented", (int)type);
    va_end(ap);
}

static void set_bc_impl(IBMSolver *s, int direction, IBMSolverBCType type, IBMSolverValType vt, double u1, double u2,
                        double u3, double pv, IBMSolverBCValFunc f1, IBMSolverBCValFunc f2, IBMSolverBCValFunc f3,
                        IBMSolverBCValFunc fp) {
    for (int i = 0; i < 6; i++) {
        if (!(direction & (1 << i))) continue;
        s->bc[i].type = type;
        s->bc[i].val_type = vt;
        if (vt == VAL_CONST) {
            s->bc[i].const_u1 = u1;
            s->bc[i].const_u2 = u2;
            s->bc[i].const_u3 = u3;
            s->bc[i].const_p = pv;
        } else {
            s->bc[i].func_u1 = f1;
            s->bc[i].func_u2 = f2;
            s->bc[i].func_u3 = f3;
            s->bc[i].func_p = fp;
        }
    }
}

void IBMSolver_set_bc(IBMSolver *s, IBMSolverDirection direction, IBMSolverBCType type, ...) {
    IBMSolverValType vt = VAL_CONST;
    double u1 = kNaN, u2 = kNaN, u3 = kNaN, pv = kNaN;
    IBMSolverBCValFunc f1 = nullptr, f2 = nullptr, f3 = nullptr, fp = nullptr;
    va_list ap;
    va_start(ap, type);
    switch (type) {
    case BC_VELOCITY_COMPONENT:
        vt = (IBMSolverValType)va_arg(ap, int);
        if (vt == VAL_CONST) {
            u1 = va_arg(ap, double);
            u2 = va_arg(ap, double);
            u3 = va_arg(ap, double);
        } else {
            f1 = va_arg(ap, IBMSolverBCValFunc);
            f2 = va_arg(ap, IBMSolverBCValFunc);
            f3 = va_arg(ap, IBMSolverBCValFunc);
        }
        break;
    case BC_PRESSURE:
    case BC_VELOCITY_PERIODIC:
        vt = (IBMSolverValType)va_arg(ap, int);
        if (vt == VAL_CONST) pv = va_arg(ap, double);
        else fp = va_arg(ap, IBMSolverBCValFunc);
        break;
    case BC_STATIONARY_WALL:
        type = BC_VELOCITY_COMPONENT;
        u1 = u2 = u3 = 0;
        break;
    case BC_SYMMETRIC:
        type = BC_FREE_SLIP_WALL;
        break;
    default:;
    }
    va_end(ap);
    set_bc_impl(s, direction, type, vt, u1, u2, u3, pv, f1, f2, f3, fp);
}

void IBMSolver_set_obstacle(IBMSolver *s, Polyhedron *poly) { s->poly = poly; }

void IBMSolver_set_linear_solver(IBMSolver *s, IBMSolverLinearSolverType type, IBMSolverPrecondType precond,
                                 const double tol) {
    if (type == SOLVER_AMG && precond != PRECOND_NONE) {
        set_status(s, IBM3D_EARG, "Cannot use preconditioner with BoomerAMG solver");
        return;
    }
    s->linear_solver_type = type;
    s->precond_type = precond;
    s->tol = tol;
    ibm3d_device *d = s->dev;
    if (d && d->assembled && type == SOLVER_GMRES && !d->gm.base &&
        d->gm.allocate(d->g.ncell, d->gm_restart, d->A64.sw.nblocks) != 0)
        set_status(s, IBM3D_ECUDA, "GMRES workspace allocation failed");
}

void IBMSolver_set_autosave(IBMSolver *s, const char *filename, int period) {
    s->autosave_filename = filename;
    s->autosave_period = period;
}

// src/ibm3d_setup.c:499-639
void IBMSolver_assemble(IBMSolver *s) {
    ibm3d_device *d = s->dev;
    if (!d || !d->s) {
        set_status(s, IBM3D_ECUDA, "no GPU stream: the solver was not created on a CUDA device");
        return;
    }
    if (!s->dx) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_grid must be called before IBMSolver_assemble");
        return;
    }
    if (isperiodic(s->bc[0].type) != isperiodic(s->bc[2].type) || isperiodic(s->bc[1].type) != isperiodic(s->bc[3].type) ||
        isperiodic(s->bc[4].type) != isperiodic(s->bc[5].type)) {
        set_status(s, IBM3D_EARG, "Inconsistent periodic boundary condition");
        return;
    }
    for (int f = 0; f < 6; f++)
        if (sampled_face(s, f) &&
            (s->bc[f].type == BC_VELOCITY_COMPONENT ? !(s->bc[f].func_u1 && s->bc[f].func_u2 && s->bc[f].func_u3)
                                                    : !s->bc[f].func_p)) {
            set_status(s, IBM3D_EARG, "VAL_FUNC boundary condition without a function");
            return;
        }
    if (s->ext_force.val_type == VAL_FUNC &&
        !(s->ext_force.func_f1 && s->ext_force.func_f2 && s->ext_force.func_f3)) {
        set_status(s, IBM3D_EARG, "VAL_FUNC body force without a function");
        return;
    }
    if (s->turb_model.type != TURBMODEL_NONE && s->turb_model.type != TURBMODEL_SMAGORINSKY) {
        set_status(s, IBM3D_EUNSUPPORTED, "turbulence model %d is not implemented", (int)s->turb_model.type);
        return;
    }
    host_metrics(s);
    size_t free0 = 0, total0 = 0;
    cudaMemGetInfo(&free0, &total0);
    Grid &g = d->g;
    g.nx = s->Nx;
    g.ny = s->Ny;
    g.nz = s->Nz;
    g.sy = s->Nz + 4;
    g.sx = (long long)(s->Ny + 4) * g.sy;
    g.ncell = (long long)(s->Nx + 4) * g.sx;
    set_grid_dividers(g);
    release_device(d);
    d->s = nullptr;
    cuda_check(s, cudaStreamCreateWithFlags(&d->s, cudaStreamNonBlocking), "stream");
    for (auto &a : d->aux) cuda_check(s, cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking), "stream");
    d->prof.s = d->s;
    for (int f = 0; f < 6; f++) make_bcface(s, f, d->bc.f[f]);
    d->bc.p_singular = 1;
    for (int f = 0; f < 6; f++)
        if (s->bc[f].type == BC_PRESSURE || s->bc[f].type == BC_VELOCITY_PERIODIC) d->bc.p_singular = 0;
    d->les = s->turb_model.type == TURBMODEL_SMAGORINSKY;
    if (!upload_axes(s) || !alloc_fields(s) || !alloc_samples(s)) return;
    if (!build_levelset(s)) return;
    if (!build_ghosts(s)) return;
    build_coeffsum(s);
    cudaMemcpyAsync(s->lvset, d->lvset, sizeof(double) * g.ncell, cudaMemcpyDeviceToHost, d->s);
    if (!build_ops(s)) return;
    const int mb = d->A64.sw.nblocks;
    if (d->kmom.allocate(g.ncell, 3, false, mb) != 0 || d->kpres.allocate(g.ncell, 1, true, mb) != 0 ||
        d->irmom.allocate(g.ncell, 3, false, mb) != 0 || d->irpres.allocate(g.ncell, 1, true, mb) != 0) {
        set_status(s, IBM3D_ECUDA, "Krylov workspace allocation failed");
        return;
    }
    d->kpres_df = dfloat_view(d->kpres);
    d->pp_df = dmalloc<dfloat>(s, g.ncell, "Krylov workspace");
    if (!d->pp_df) return;
    MGGeometry geom;
    const double *D[3] = {s->dx, s->dy, s->dz};
    const int Ns[3] = {s->Nx, s->Ny, s->Nz};
    for (int a = 0; a < 3; a++) {
        geom.f[a].assign(Ns[a] + 1, 0.0);
        for (int i = 0; i < Ns[a]; i++) geom.f[a][i + 1] = geom.f[a][i] + D[a][i + 2];
    }
    GMGConfig mc;
    mc.nu_pre = d->mg_sweeps[0];
    mc.nu_post = d->mg_sweeps[1];
    mc.nuc_pre = d->mg_sweeps[2];
    mc.nuc_post = d->mg_sweeps[3];
    mc.coarse_sweeps = d->mg_sweeps[4];
    mc.omega = d->mg_omega;
    mc.coarsening = d->mg_coarsening == IBM3D_COARSEN_HALVE ? MG_COARSEN_HALVE : MG_COARSEN_SPACING;
    mc.width_ratio = d->mg_width_ratio;
    const int *gcell = d->nghost ? d->gargs.cell : nullptr;
    d->mg = new GMG<double>();
    d->mg32 = new GMG<float>();
    if (d->mg->setup(d->s, d->A64, d->A64, gcell, d->nghost, geom, mc) != 0 ||
        d->mg32->setup(d->s, d->A64, d->A32, gcell, d->nghost, geom, mc) != 0) {
        set_status(s, IBM3D_ECUDA, "multigrid setup failed");
        return;
    }
    d->mg->set_prof(&d->prof);
    d->mg32->set_prof(&d->prof);
    if (d->pc64.allocate(g.ncell, d->mg32) != 0) {
        set_status(s, IBM3D_ECUDA, "preconditioner workspace allocation failed");
        return;
    }
    d->pcdf.attach(d->pc64);
    if (pres_gmres(s) && d->gm.allocate(g.ncell, d->gm_restart, mb) != 0) {
        set_status(s, IBM3D_ECUDA, "GMRES workspace allocation failed");
        return;
    }
    if (!cuda_check(s, cudaStreamSynchronize(d->s), "assemble")) return;
    size_t free1 = 0, total1 = 0;
    cudaMemGetInfo(&free1, &total1);
    d->dev_bytes = free0 > free1 ? free0 - free1 : 0;
    d->assembled = true;
    d->status = IBM3D_OK;
}

// src/utils.c:111-171, on the host from the assembled level set.
void IBMSolver_ghost_interp(IBMSolver *s, const int i, const int j, const int k, int idx[][3], double coeff[]) {
    const int Ny = s->Ny, Nz = s->Nz;
    auto L = [&](int a, int b, int c) { return s->lvset[(long long)(Ny + 4) * (Nz + 4) * (a + 2) + (Nz + 4) * (b + 2) + c + 2]; };
    const double *xc = s->xc, *yc = s->yc, *zc = s->zc;
    const double nx = (L(i + 1, j, k) - L(i - 1, j, k)) / (xc[i + 3] - xc[i + 1]);
    const double ny = (L(i, j + 1, k) - L(i, j - 1, k)) / (yc[j + 3] - yc[j + 1]);
    const double nz = (L(i, j, k + 1) - L(i, j, k - 1)) / (zc[k + 3] - zc[k + 1]);
    const double c = -2 * L(i, j, k);
    const Vector m = Vector_lincom(1, Vector{xc[i + 2], yc[j + 2], zc[k + 2]}, c, Vector{nx, ny, nz});
    auto ub = [](int len, const double *arr, double val) {
        int l = 0, h = len;
        while (l < h) {
            const int mid = l + (h - l) / 2;
            if (val >= arr[mid]) l = mid + 1;
            else h = mid;
        }
        return l;
    };
    const int im = ub(s->Nx + 4, xc, m.x) - 3, jm = ub(s->Ny + 4, yc, m.y) - 3, km = ub(s->Nz + 4, zc, m.z) - 3;
    for (int l = 0; l < 8; l++) {
        idx[l][0] = im + !!(l & 4);
        idx[l][1] = jm + !!(l & 2);
        idx[l][2] = km + !!(l & 1);
    }
    const double xl = xc[im + 2], xu = xc[im + 3], yl = yc[jm + 2], yu = yc[jm + 3], zl = zc[km + 2], zu = zc[km + 3];
    const double vol = (xu - xl) * (yu - yl) * (zu - zl);
    coeff[0] = (xu - m.x) * (yu - m.y) * (zu - m.z) / vol;
    coeff[1] = (xu - m.x) * (yu - m.y) * (m.z - zl) / vol;
    coeff[2] = (xu - m.x) * (m.y - yl) * (zu - m.z) / vol;
    coeff[3] = (xu - m.x) * (m.y - yl) * (m.z - zl) / vol;
    coeff[4] = (m.x - xl) * (yu - m.y) * (zu - m.z) / vol;
    coeff[5] = (m.x - xl) * (yu - m.y) * (m.z - zl) / vol;
    coeff[6] = (m.x - xl) * (m.y - yl) * (zu - m.z) / vol;
    coeff[7] = (m.x - xl) * (m.y - yl) * (m.z - zl) / vol;
}

// ------------------------------------------------------------- init ---
// src/ibm3d_init.c:15-37
void IBMSolver_init_flow_const(IBMSolver *s, const double u1, const double u2, const double u3, const double p) {
    if (!check_ready(s, "IBMSolver_init_flow_const")) return;
    const size_t n = (size_t)ncell_of(s);
    std::fill(s->u1, s->u1 + n, u1);
    std::fill(s->u2, s->u2 + n, u2);
    std::fill(s->u3, s->u3 + n, u3);
    std::fill(s->p, s->p + n, p);
    upload_state(s, s->u1, s->u2, s->u3, s->p);
}

// src/ibm3d_init.c:237-262
void IBMSolver_init_flow_func(IBMSolver *s, IBMSolverInitFunc f1, IBMSolverInitFunc f2, IBMSolverInitFunc f3,
                              IBMSolverInitFunc fp) {
    if (!check_ready(s, "IBMSolver_init_flow_func")) return;
    for (int i = -2; i < s->Nx + 2; i++)
        for (int j = -2; j < s->Ny + 2; j++)
            for (int k = -2; k < s->Nz + 2; k++) {
                const long long P = cidx(s->dev->g, i, j, k);
                const double x = s->xc[i + 2], y = s->yc[j + 2], z = s->zc[k + 2];
                s->u1[P] = f1(x, y, z);
                s->u2[P] = f2(x, y, z);
                s->u3[P] = f3(x, y, z);
                s->p[P] = fp(x, y, z);
            }
    upload_state(s, s->u1, s->u2, s->u3, s->p);
}

void IBMSolver_init_flow_array(IBMSolver *s, const double *u1, const double *u2, const double *u3, const double *p) {
    if (!check_ready(s, "IBMSolver_init_flow_array")) return;
    upload_state(s, u1, u2, u3, p);
}

// ----------------------------------------------------------- export ---
// Exact-resume state: header, then every device field a later
// IBMSolver_iterate call can read, in role order, as padded FP64 arrays.
// u and p alone do not suffice: the reference double-buffers u, U, p and N
// (src/ibm3d_fracstep.c:795-804) and update_next writes only fluid cells
// of u_next, so after each swap the ghost cells and padding corners hold
// the values of two steps back, which update_ghost reads for ghosts later
// in its sweep (src/ibm3d_fracstep.c:1915-1976).  The reference's own
// restart from its float file cannot reproduce those; this file does.
struct StateHeader {
    char magic[8];
    int nx, ny, nz, iter;
    double time;
    int nfields;
    int pp_hist;   // pressure increments known to the guess extrapolation (0..2)
};

namespace {

constexpr int kStateFields = 28;

// Device arrays of the state, in file order.
void state_fields(ibm3d_device *d, double *f[kStateFields]) {
    int q = 0;
    for (int l = 0; l < 3; l++) f[q++] = d->u[l];
    for (int l = 0; l < 3; l++) f[q++] = d->un[l];
    for (int l = 0; l < 3; l++) f[q++] = d->U[l];
    for (int l = 0; l < 3; l++) f[q++] = d->Un[l];
    f[q++] = d->p;
    f[q++] = d->pn;
    for (int l = 0; l < 3; l++) f[q++] = d->N[l];
    for (int l = 0; l < 3; l++) f[q++] = d->Np[l];
    for (int l = 0; l < 6; l++) f[q++] = d->tau[l];
    f[q++] = d->pp;       // the last pressure increment: the next solve's initial guess
    f[q++] = d->pp_prev;  // the one before (guess extrapolation)
}

bool write_state(IBMSolver *s, const std::string &path) {
    ibm3d_device *d = s->dev;
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    StateHeader h{};
    memcpy(h.magic, "IBM3DST4", 8);
    h.nx = s->Nx; h.ny = s->Ny; h.nz = s->Nz; h.iter = s->iter; h.time = s->time;
    h.nfields = kStateFields;
    cudaMemcpy(&h.pp_hist, d->pp_hist, sizeof(int), cudaMemcpyDeviceToHost);
    const size_t n = (size_t)d->g.ncell;
    bool ok = fwrite(&h, sizeof h, 1, f) == 1;
    double *fld[kStateFields];
    state_fields(d, fld);
    std::vector<double> buf(n);
    for (int q = 0; q < kStateFields && ok; q++) {
        ok = cuda_check(s, cudaMemcpy(buf.data(), fld[q], n * sizeof(double), cudaMemcpyDeviceToHost), "state read");
        ok = ok && fwrite(buf.data(), sizeof(double), n, f) == n;
    }
    return fclose(f) == 0 && ok;
}

// 1: read into the device fields (and u, p into the host mirrors); 0: no
// such file; -1: a file that is not a state of this grid (nothing changed).
int read_state(IBMSolver *s, const std::string &path) {
    ibm3d_device *d = s->dev;
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return 0;
    StateHeader h{};
    const size_t n = (size_t)d->g.ncell;
    bool ok = fread(&h, sizeof h, 1, f) == 1 && memcmp(h.magic, "IBM3DST4", 8) == 0 && h.nx == s->Nx &&
              h.ny == s->Ny && h.nz == s->Nz && h.nfields == kStateFields;
    std::vector<double> buf(ok ? kStateFields * n : 0);
    ok = ok && fread(buf.data(), sizeof(double), buf.size(), f) == buf.size();
    fclose(f);
    if (!ok) return -1;
    double *fld[kStateFields];
    state_fields(d, fld);
    for (int q = 0; q < kStateFields; q++)
        cudaMemcpyAsync(fld[q], buf.data() + q * n, n * sizeof(double), cudaMemcpyHostToDevice, d->s);
    const int hist = h.pp_hist < 0 ? 0 : h.pp_hist > 2 ? 2 : h.pp_hist;
    cudaMemcpyAsync(d->pp_hist, &hist, sizeof(int), cudaMemcpyHostToDevice, d->s);
    if (!cuda_check(s, cudaStreamSynchronize(d->s), "state upload")) return 1;
    double *host[4] = {s->u1, s->u2, s->u3, s->p};
    const int role[4] = {0, 1, 2, 12};
    for (int q = 0; q < 4; q++) std::copy(buf.begin() + role[q] * n, buf.begin() + (role[q] + 1) * n, host[q]);
    s->iter = h.iter;
    s->time = h.time;
    return 1;
}

// The reference's result file (src/ibm3d_export.c:143-196): dimensions
// time(1), x, y, z (padded sizes); time, x, y, z as double with axis and
// units attributes; iter as a scalar int; u, v, w, p, vorticity, Q as
// float [time][z][y][x].  The fields and vorticity/Q come from the GPU.
bool write_result_nc(IBMSolver *s, const std::string &path) {
    ibm3d_device *d = s->dev;
    const long long plane = (long long)(s->Nx + 4) * (s->Ny + 4) * (s->Nz + 4);
    if (s->Ny + 4 > 65535) {
        set_status(s, IBM3D_EARG, "export: Ny + 4 = %d exceeds 65535", s->Ny + 4);
        return false;
    }
    float *dbuf = nullptr;
    if (!cuda_check(s, cudaMalloc(&dbuf, sizeof(float) * 6 * plane), "export buffer")) return false;
    std::vector<float> h((size_t)(6 * plane));
    launch_export_fields(d->s, d->g, d->ax[0], d->ax[1], d->ax[2], d->u, d->p, dbuf);
    cudaMemcpyAsync(h.data(), dbuf, sizeof(float) * 6 * plane, cudaMemcpyDeviceToHost, d->s);
    const bool dev_ok = cuda_check(s, cudaStreamSynchronize(d->s), "export");
    cudaFree(dbuf);
    if (!dev_ok) return false;

    NcFile f;
    f.dims = {{"time", 1}, {"x", s->Nx + 4}, {"y", s->Ny + 4}, {"z", s->Nz + 4}};
    const double tval = s->time;
    const int ival = s->iter;
    f.vars.push_back({"time", NCT_DOUBLE, {0}, {{"axis", "T"}, {"units", "seconds"}}, &tval});
    f.vars.push_back({"x", NCT_DOUBLE, {1}, {{"axis", "X"}, {"units", "meters"}}, s->xc});
    f.vars.push_back({"y", NCT_DOUBLE, {2}, {{"axis", "Y"}, {"units", "meters"}}, s->yc});
    f.vars.push_back({"z", NCT_DOUBLE, {3}, {{"axis", "Z"}, {"units", "meters"}}, s->zc});
    f.vars.push_back({"iter", NCT_INT, {}, {}, &ival});
    const char *names[6] = {"u", "v", "w", "p", "vorticity", "Q"};
    const char *units[6] = {"m/s", "m/s", "m/s", "m/s", "1/s", "1/s^2"};
    for (int q = 0; q < 6; q++)
        f.vars.push_back({names[q], NCT_FLOAT, {0, 3, 2, 1}, {{"units", units[q]}}, h.data() + q * plane});
    return nc_write(path, f);
}

// src/ibm3d_init.c:84-140: time, iter and the float u, v, w, p of a
// result file, over the padded grid.  Same return codes as read_state.
int read_result_nc(IBMSolver *s, const std::string &path) {
    NcFile f;
    FILE *probe = fopen(path.c_str(), "rb");
    if (!probe) return 0;
    fclose(probe);
    if (!nc_read_header(path, f)) return -1;
    auto dim = [&](const char *nm) -> long long {
        for (auto &x : f.dims)
            if (x.first == nm) return x.second;
        return -1;
    };
    if (dim("x") != s->Nx + 4 || dim("y") != s->Ny + 4 || dim("z") != s->Nz + 4) return -1;
    std::vector<double> tv, iv, fv[4];
    const char *names[4] = {"u", "v", "w", "p"};
    bool ok = nc_read_var(path, f, "time", tv) && nc_read_var(path, f, "iter", iv) && !tv.empty() && !iv.empty();
    for (int q = 0; q < 4 && ok; q++) ok = nc_read_var(path, f, names[q], fv[q]);
    const long long plane = (long long)(s->Nx + 4) * (s->Ny + 4) * (s->Nz + 4);
    for (int q = 0; q < 4 && ok; q++) ok = (long long)fv[q].size() == plane;
    if (!ok) return -1;
    double *dst[4] = {s->u1, s->u2, s->u3, s->p};
    const Grid &g = s->dev->g;
    for (int k = -2; k < s->Nz + 2; k++)
        for (int j = -2; j < s->Ny + 2; j++)
            for (int i = -2; i < s->Nx + 2; i++) {
                const long long o = ((long long)(k + 2) * (s->Ny + 4) + (j + 2)) * (s->Nx + 4) + (i + 2);
                const long long P = cidx(g, i, j, k);
                for (int q = 0; q < 4; q++) dst[q][P] = fv[q][o];
            }
    s->time = tv[0];
    s->iter = (int)iv[0];
    return 1;
}

}  // namespace

// src/ibm3d_export.c:16-253.  Writes "<name>.nc" (the reference's float
// result file) and "<name>.ibm3d" (the FP64 state for exact resume).
void IBMSolver_export_result(IBMSolver *s, const char *name) {
    if (!check_ready(s, "IBMSolver_export_result")) return;
    IBMSolver_sync_host(s);
    const std::string nc = std::string(name) + ".nc", st = std::string(name) + ".ibm3d";
    if (!write_result_nc(s, nc)) {
        if (s->dev->status == IBM3D_OK) set_status(s, IBM3D_EARG, "cannot write file \"%s\"", nc.c_str());
        return;
    }
    if (!write_state(s, st)) set_status(s, IBM3D_EARG, "cannot write file \"%s\"", st.c_str());
}

// src/ibm3d_init.c:45-224.  Reads "<name>.ibm3d" when it exists (the
// exact FP64 state export_result writes beside the result file), else the
// float fields, time and iter of "<name>.nc" as the reference does.
void IBMSolver_init_flow_file(IBMSolver *s, const char *name) {
    if (!check_ready(s, "IBMSolver_init_flow_file")) return;
    const std::string st = std::string(name) + ".ibm3d", nc = std::string(name) + ".nc";
    int r = read_state(s, st);
    const std::string used = r != 0 ? st : nc;
    if (r == 0) r = read_result_nc(s, nc);
    if (r == 0) {
        set_status(s, IBM3D_EARG, "cannot open file \"%s\"", nc.c_str());
        return;
    }
    if (r < 0) {
        set_status(s, IBM3D_EARG, "\"%s\" is not a flow file of this grid", used.c_str());
        return;
    }
    if (used == st) return;  // read_state uploaded every field
    const int iter = s->iter;
    const double time = s->time;
    upload_state(s, s->u1, s->u2, s->u3, s->p);
    s->iter = iter;
    s->time = time;
}

// Padded [i][j][k] cell array (solver layout) -> [k][j][i] (file layout).
extern "C++" {
namespace {
template <typename Src, typename Dst>
void to_file_layout(const IBMSolver *s, const Src *a, Dst *out) {
    const int NX = s->Nx + 4, NY = s->Ny + 4, NZ = s->Nz + 4;
    for (int i = 0; i < NX; i++)
        for (int j = 0; j < NY; j++)
            for (int k = 0; k < NZ; k++)
                out[((size_t)k * NY + j) * NX + i] = (Dst)a[((size_t)i * NY + j) * NZ + k];
}

void coord_vars(IBMSolver *s, NcFile &f, int dx, int dy, int dz) {
    f.vars.push_back({"x", NCT_DOUBLE, {dx}, {{"axis", "X"}, {"units", "meters"}}, s->xc});
    f.vars.push_back({"y", NCT_DOUBLE, {dy}, {{"axis", "Y"}, {"units", "meters"}}, s->yc});
    f.vars.push_back({"z", NCT_DOUBLE, {dz}, {{"axis", "Z"}, {"units", "meters"}}, s->zc});
}
}  // namespace
}

// src/ibm3d_export.c:262-435: "<name>.nc" with x, y, z and the level set
// (float) and flags (int) as [z][y][x] over the padded grid.
void IBMSolver_export_lvset_flag(IBMSolver *s, const char *name) {
    if (!check_ready(s, "IBMSolver_export_lvset_flag")) return;
    const size_t n = (size_t)ncell_of(s);
    std::vector<int> flag(n);
    IBMSolver_get_flag(s, flag.data());
    std::vector<float> lv(n);
    std::vector<int32_t> fl(n);
    to_file_layout(s, s->lvset, lv.data());
    to_file_layout(s, flag.data(), fl.data());
    NcFile f;
    f.dims = {{"x", s->Nx + 4}, {"y", s->Ny + 4}, {"z", s->Nz + 4}};
    coord_vars(s, f, 0, 1, 2);
    f.vars.push_back({"lvset", NCT_FLOAT, {2, 1, 0}, {}, lv.data()});
    f.vars.push_back({"flag", NCT_INT, {2, 1, 0}, {}, fl.data()});
    const std::string path = std::string(name) + ".nc";
    if (!nc_write(path, f)) set_status(s, IBM3D_EARG, "cannot write file \"%s\"", path.c_str());
}

// src/ibm3d_export.c:437-650: "<name>.nc" with time, x, y, z, iter and the
// last step's u*, u~ (per component) and p' as float [time][z][y][x].  u~
// is not kept by the GPU step (it is folded into the face-velocity kernel),
// so it is formed here as the reference's calc_u_tilde does
// (src/ibm3d_fracstep.c:388-412): u* + dt (p(+1) - p(-1)) / (c(+1) - c(-1))
// with the step's starting pressure, on [-1, N] in every axis, 0 elsewhere.
void IBMSolver_export_intermediate(IBMSolver *s, const char *name) {
    if (!check_ready(s, "IBMSolver_export_intermediate")) return;
    ibm3d_device *d = s->dev;
    const size_t n = (size_t)ncell_of(s);
    std::vector<double> us[3], pp(n), p0(n);
    const int which[3] = {IBM3D_F_USTAR1, IBM3D_F_USTAR2, IBM3D_F_USTAR3};
    for (int l = 0; l < 3; l++) {
        us[l].resize(n);
        IBMSolver_get_field(s, which[l], us[l].data());
    }
    IBMSolver_get_field(s, IBM3D_F_PPRIME, pp.data());
    // The step's starting pressure is the second pressure buffer after it.
    cudaMemcpy(p0.data(), d->pn, sizeof(double) * n, cudaMemcpyDeviceToHost);
    std::vector<double> ut[3];
    for (int l = 0; l < 3; l++) ut[l].assign(n, 0.0);
    const Grid &g = d->g;
    const double dt = s->dt;
    for (int i = -1; i < s->Nx + 1; i++)
        for (int j = -1; j < s->Ny + 1; j++)
            for (int k = -1; k < s->Nz + 1; k++) {
                const long long P = cidx(g, i, j, k);
                ut[0][P] = us[0][P] + dt * (p0[P + g.sx] - p0[P - g.sx]) / (s->xc[i + 3] - s->xc[i + 1]);
                ut[1][P] = us[1][P] + dt * (p0[P + g.sy] - p0[P - g.sy]) / (s->yc[j + 3] - s->yc[j + 1]);
                ut[2][P] = us[2][P] + dt * (p0[P + 1] - p0[P - 1]) / (s->zc[k + 3] - s->zc[k + 1]);
            }
    std::vector<float> out[7];
    const std::vector<double> *src[7] = {&us[0], &us[1], &us[2], &ut[0], &ut[1], &ut[2], &pp};
    for (int q = 0; q < 7; q++) {
        out[q].resize(n);
        to_file_layout(s, src[q]->data(), out[q].data());
    }
    NcFile f;
    f.dims = {{"time", 1}, {"x", s->Nx + 4}, {"y", s->Ny + 4}, {"z", s->Nz + 4}};
    const double tval = s->time;
    const int ival = s->iter;
    f.vars.push_back({"time", NCT_DOUBLE, {0}, {{"axis", "T"}, {"units", "seconds"}}, &tval});
    coord_vars(s, f, 1, 2, 3);
    f.vars.push_back({"iter", NCT_INT, {}, {}, &ival});
    const char *names[7] = {"u_star", "v_star", "w_star", "u_tilde", "v_tilde", "w_tilde", "p_prime"};
    for (int q = 0; q < 7; q++)
        f.vars.push_back({names[q], NCT_FLOAT, {0, 3, 2, 1}, {{"units", "m/s"}}, out[q].data()});
    const std::string path = std::string(name) + ".nc";
    if (!nc_write(path, f)) set_status(s, IBM3D_EARG, "cannot write file \"%s\"", path.c_str());
}

// -------------------------------------------------------------- turb ---
void IBMSolver_calc_tau_r(IBMSolver *s) {
    if (!check_ready(s, "IBMSolver_calc_tau_r")) return;
    calc_tau(s);
    cuda_check(s, cudaStreamSynchronize(s->dev->s), "calc_tau_r");
}

// ---------------------------------------------------------- iterate ---
// src/ibm3d_fracstep.c:38-115
namespace {
// What every IBMSolver_iterate call does before its steps
// (src/ibm3d_fracstep.c:40-56): outer fill, face velocities, ghost
// update with solid NaNs, and N^{-1} = N^0 for the AB2 bootstrap.
void iterate_prologue(IBMSolver *s);

// Adds a finished step's counts to the solver's totals.
void account_step(ibm3d_device *d) {
    d->steps_total++;
    for (int l = 0; l < 3; l++) d->iters_u_total[l] += d->rep_mom.iters[l];
    d->iters_p_total += d->rep_p.iters[0];
    d->outer_p_total += d->rep_p.outer;
    if (!(d->max_div <= d->max_div_max)) d->max_div_max = d->max_div;
}

void iterate_prologue(IBMSolver *s) {
    ibm3d_device *d = s->dev;
    d->status = IBM3D_OK;
    prepare_samples(s, d->s, s->time, s->time + s->dt);
    fill_outer(s, 0);
    launch_interp_stag(d->s, d->g, d->ax[0], d->ax[1], d->ax[2], d->u, d->U);
    ghost_update(s, true);
    const double f[3] = {s->ext_force.const_f1, s->ext_force.const_f2, s->ext_force.const_f3};
    if (step32(d)) {
        launch_conv_rhs32(d->s, d->g, d->axf, d->A32, d->bc, d->flag, conv32_args(d), s->dt, f, 0, d->red_partials,
                          d->red_counter, d->irmom.scal);
        // The FP64 N buffers swap with them: recorded steps are keyed by
        // the FP64 buffers' parity, which must follow the FP32 ones.
        for (int l = 0; l < 3; l++) std::swap(d->N32[l], d->Np32[l]);
        swap3(d->N, d->Np);
        return;
    }
    launch_conv_rhs(d->s, d->g, d->ax[0], d->ax[1], d->ax[2], d->bc, d->flag, conv_args(d), s->dt, f, 0);
    swap3(d->N, d->Np);
}
}  // namespace

void IBMSolver_iterate(IBMSolver *s, int num_time_steps, bool verbose) {
    if (!check_ready(s, "IBMSolver_iterate")) return;
    ibm3d_device *d = s->dev;
    const double start_time = s->time;
    iterate_prologue(s);
    struct timespec t0, t1;
    clock_gettime(CLOCK_REALTIME, &t0);
    for (int i = 1; i <= num_time_steps; i++) {
        prepare_samples(s, d->s, s->time, start_time + s->dt * i);
        if (!(d->use_graphs && !d->prof.on && graph_step(s))) {
            one_step(s);
            int t = d->prof.begin("fill_outer");
            fill_outer(s, 1);
            d->prof.end(t);
            t = d->prof.begin("ghost_update");
            ghost_update(s, false);
            d->prof.end(t);
            cudaMemcpyAsync(d->maxdiv_h, d->maxdiv_d, sizeof(double), cudaMemcpyDeviceToHost, d->s);
            if (!cuda_check(s, cudaStreamSynchronize(d->s), "time step")) return;
        }
        if (d->status == IBM3D_ECUDA) return;
        s->iter++;
        s->time = start_time + s->dt * i;
        d->max_div = *d->maxdiv_h;
        account_step(d);
        // NaN anywhere near a fluid cell reaches max|div U| (its reduction
        // keeps NaN) or a solve's residual.
        if (d->status != IBM3D_ENONFINITE && !std::isfinite(d->max_div))
            set_status(s, IBM3D_ENONFINITE,
                       "non-finite max|div U| after step %d: NaN or Inf in the state, boundary data or force",
                       s->iter);
        const bool nonfinite = d->status == IBM3D_ENONFINITE;
        d->prof.flush();
        if (verbose && s->rank == 0) {
            clock_gettime(CLOCK_REALTIME, &t1);
            const long el = (t1.tv_sec * 1000 + t1.tv_nsec / 1000000) - (t0.tv_sec * 1000 + t0.tv_nsec / 1000000);
            print_row(s, i, el);
        }
        if (nonfinite) return;
        if (s->autosave_period > 0 && s->iter % s->autosave_period == 0) {
            if (s->rank == 0) printf("\nAutosave...\n\n");
            char fn[1024];
            snprintf(fn, sizeof fn, "%s-%05d", s->autosave_filename, s->iter);
            IBMSolver_export_result(s, fn);
        }
    }
}

// ------------------------------------------------------- extensions ---
int IBMSolver_last_status(const IBMSolver *s) { return s && s->dev ? s->dev->status : IBM3D_EARG; }

const char *IBMSolver_last_message(const IBMSolver *s) { return s && s->dev ? s->dev->message : ""; }

const char *IBMSolver_status_string(int st) {
    switch (st) {
    case IBM3D_OK: return "ok";
    case IBM3D_ENOCONV: return "Krylov solve did not converge";
    case IBM3D_EBREAKDOWN: return "BiCGSTAB breakdown";
    case IBM3D_ECUDA: return "CUDA error";
    case IBM3D_EARG: return "invalid argument";
    case IBM3D_EGEOM: return "ghost-cell mirror point outside the grid";
    case IBM3D_EUNSUPPORTED: return "unsupported on the GPU path";
    case IBM3D_ENONFINITE: return "non-finite values in the time step";
    }
    return "unknown";
}

void IBMSolver_set_bc_const(IBMSolver *s, IBMSolverDirection dir, IBMSolverBCType type, double u1, double u2,
                            double u3, double p) {
    switch (type) {
    case BC_VELOCITY_COMPONENT:
        set_bc_impl(s, dir, type, VAL_CONST, u1, u2, u3, kNaN, nullptr, nullptr, nullptr, nullptr);
        break;
    case BC_PRESSURE:
    case BC_VELOCITY_PERIODIC:
        set_bc_impl(s, dir, type, VAL_CONST, kNaN, kNaN, kNaN, p, nullptr, nullptr, nullptr, nullptr);
        break;
    case BC_STATIONARY_WALL:
        set_bc_impl(s, dir, BC_VELOCITY_COMPONENT, VAL_CONST, 0, 0, 0, kNaN, nullptr, nullptr, nullptr, nullptr);
        break;
    case BC_SYMMETRIC:
        set_bc_impl(s, dir, BC_FREE_SLIP_WALL, VAL_CONST, kNaN, kNaN, kNaN, kNaN, nullptr, nullptr, nullptr, nullptr);
        break;
    default:
        set_bc_impl(s, dir, type, VAL_CONST, kNaN, kNaN, kNaN, kNaN, nullptr, nullptr, nullptr, nullptr);
    }
}

void IBMSolver_set_ext_force_const(IBMSolver *s, double f1, double f2, double f3) {
    s->ext_force.val_type = VAL_CONST;
    s->ext_force.const_f1 = f1;
    s->ext_force.const_f2 = f2;
    s->ext_force.const_f3 = f3;
}

void IBMSolver_set_bc_func(IBMSolver *s, IBMSolverDirection dir, IBMSolverBCType type, IBMSolverBCValFunc f1,
                           IBMSolverBCValFunc f2, IBMSolverBCValFunc f3, IBMSolverBCValFunc fp) {
    if (type == BC_VELOCITY_COMPONENT)
        set_bc_impl(s, dir, type, VAL_FUNC, kNaN, kNaN, kNaN, kNaN, f1, f2, f3, nullptr);
    else if (type == BC_PRESSURE || type == BC_VELOCITY_PERIODIC)
        set_bc_impl(s, dir, type, VAL_FUNC, kNaN, kNaN, kNaN, kNaN, nullptr, nullptr, nullptr, fp);
    else
        set_status(s, IBM3D_EARG, "IBMSolver_set_bc_func: type %d takes no boundary values", (int)type);
}

void IBMSolver_set_ext_force_func(IBMSolver *s, IBMSolverForceFunc f1, IBMSolverForceFunc f2, IBMSolverForceFunc f3) {
    s->ext_force.val_type = VAL_FUNC;
    s->ext_force.func_f1 = f1;
    s->ext_force.func_f2 = f2;
    s->ext_force.func_f3 = f3;
}

void IBMSolver_set_smagorinsky(IBMSolver *s, double Cs) {
    s->turb_model.type = TURBMODEL_SMAGORINSKY;
    s->turb_model.Cs = Cs;
}

void IBMSolver_set_div_tol(IBMSolver *s, double div_tol) { s->dev->divtol = div_tol; }

void IBMSolver_set_gmres_restart(IBMSolver *s, int restart) {
    ibm3d_device *d = s->dev;
    if (restart < 1 || restart > GM_MAX) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_gmres_restart: restart length in [1, %d]", GM_MAX);
        return;
    }
    d->gm_restart = restart;
    if (d->assembled && pres_gmres(s)) {
        drop_graphs(d);
        if (d->gm.allocate(d->g.ncell, restart, d->A64.sw.nblocks) != 0)
            set_status(s, IBM3D_ECUDA, "GMRES workspace allocation failed");
    }
}

void IBMSolver_set_refinement(IBMSolver *s, double inner_tol_mom, double inner_tol_p, int max_outer) {
    if (!(inner_tol_mom > 0 && inner_tol_mom < 1) || !(inner_tol_p > 0 && inner_tol_p < 1) || max_outer < 1) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_refinement: tolerances in (0, 1) and max_outer >= 1");
        return;
    }
    s->dev->inner_tol[0] = inner_tol_mom;
    s->dev->inner_tol[1] = inner_tol_p;
    s->dev->max_outer = max_outer;
}

void IBMSolver_set_multigrid(IBMSolver *s, int nu_pre, int nu_post, int nuc_pre, int nuc_post, int coarse_sweeps,
                             double omega) {
    ibm3d_device *d = s->dev;
    if (nu_pre < 0 || nu_post < 0 || nuc_pre < 0 || nuc_post < 0 || coarse_sweeps < 1 || nu_pre + nu_post < 1 ||
        !(omega > 0.0 && omega < 2.0)) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_multigrid: invalid sweep counts or relaxation weight");
        return;
    }
    const int v[5] = {nu_pre, nu_post, nuc_pre, nuc_post, coarse_sweeps};
    for (int q = 0; q < 5; q++) d->mg_sweeps[q] = v[q];
    d->mg_omega = omega;
    if (d->mg) {
        d->mg->set_sweeps(nu_pre, nu_post, nuc_pre, nuc_post, coarse_sweeps);
        d->mg->set_omega(omega);
    }
    if (d->mg32) {
        d->mg32->set_sweeps(nu_pre, nu_post, nuc_pre, nuc_post, coarse_sweeps);
        d->mg32->set_omega(omega);
    }
    drop_graphs(d);
}

void IBMSolver_set_warm_start(IBMSolver *s, int on) {
    s->dev->warm_start = on != 0;
    drop_graphs(s->dev);
}

void IBMSolver_set_pressure_guess(IBMSolver *s, int mode) {
    if (!s || !s->dev || mode < 0 || mode > 1) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_pressure_guess: mode %d", mode);
        return;
    }
    s->dev->p_guess = mode;
    drop_graphs(s->dev);
}

void IBMSolver_set_pressure_vectors(IBMSolver *s, int kind) {
    if (!s || !s->dev || (kind != IBM3D_PVEC_FP64 && kind != IBM3D_PVEC_DFLOAT)) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_pressure_vectors: kind %d", kind);
        return;
    }
    s->dev->pvec = kind;
    drop_graphs(s->dev);
}

void IBMSolver_set_max_iters(IBMSolver *s, int max_mom, int max_p) {
    if (!s || !s->dev || max_mom < 1 || max_p < 1) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_max_iters: caps must be >= 1 (%d, %d)", max_mom, max_p);
        return;
    }
    s->dev->maxit_mom = max_mom;
    s->dev->maxit_p = max_p;
    drop_graphs(s->dev);
}

void IBMSolver_set_coarsening(IBMSolver *s, int mode, double width_ratio) {
    if (mode != IBM3D_COARSEN_HALVE && mode != IBM3D_COARSEN_SPACING) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_coarsening: unknown mode %d", mode);
        return;
    }
    if (!(width_ratio == 0.0 || (width_ratio >= 1.0 && width_ratio <= 64.0))) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_coarsening: width ratio %g outside [1, 64]", width_ratio);
        return;
    }
    if (s->dev->mg) {
        set_status(s, IBM3D_EARG, "IBMSolver_set_coarsening: call it before IBMSolver_assemble");
        return;
    }
    s->dev->mg_coarsening = mode;
    s->dev->mg_width_ratio = width_ratio == 0.0 ? 1.5 : width_ratio;
}

void IBMSolver_set_graphs(IBMSolver *s, int on) {
    s->dev->use_graphs = on != 0;
    drop_graphs(s->dev);
}

void IBMSolver_set_precision(IBMSolver *s, int mode) {
    if (mode != IBM3D_FP64 && mode != IBM3D_MIXED && mode != IBM3D_MIXED_MG && mode != IBM3D_MIXED32 &&
        mode != IBM3D_MIXED32_IR) {
        set_status(s, IBM3D_EUNSUPPORTED, "precision mode %d is not available", mode);
        return;
    }
    s->dev->precision = mode;
}

void IBMSolver_get_field(IBMSolver *s, int field, double *out) {
    if (!check_ready(s, "IBMSolver_get_field")) return;
    ibm3d_device *d = s->dev;
    const Grid &g = d->g;
    const size_t n = g.ncell;
    const double *src = nullptr;
    int face = -1;
    if (step32(d)) {
        // The FP32 step keeps N in FP32 and u* as u^n + e (u^n is in the
        // second buffer after the step): both are formed in their FP64
        // arrays for read-back.
        if (field >= IBM3D_F_N1 && field <= IBM3D_F_N3)
            launch_widen_f32(d->s, (long long)n, d->Np32[field - IBM3D_F_N1], d->Np[field - IBM3D_F_N1]);
        if (field >= IBM3D_F_USTAR1 && field <= IBM3D_F_USTAR3) {
            const int l = field - IBM3D_F_USTAR1;
            launch_ustar_from_increment(d->s, (long long)n, d->un[l], d->irmom.e32 + l * n, d->ustar + l * n);
        }
    }
    switch (field) {
    case IBM3D_F_U1: src = d->u[0]; break;
    case IBM3D_F_U2: src = d->u[1]; break;
    case IBM3D_F_U3: src = d->u[2]; break;
    case IBM3D_F_P: src = d->p; break;
    case IBM3D_F_FACE_U1: src = d->U[0]; face = 0; break;
    case IBM3D_F_FACE_U2: src = d->U[1]; face = 1; break;
    case IBM3D_F_FACE_U3: src = d->U[2]; face = 2; break;
    case IBM3D_F_USTAR1: src = d->ustar; break;
    case IBM3D_F_USTAR2: src = d->ustar + n; break;
    case IBM3D_F_USTAR3: src = d->ustar + 2 * n; break;
    case IBM3D_F_FACE_USTAR1: src = d->Us[0]; face = 0; break;
    case IBM3D_F_FACE_USTAR2: src = d->Us[1]; face = 1; break;
    case IBM3D_F_FACE_USTAR3: src = d->Us[2]; face = 2; break;
    case IBM3D_F_PPRIME: src = d->pp; break;
    // After a step N and N_prev are swapped: N_prev holds the last step's N.
    case IBM3D_F_N1: src = d->Np[0]; break;
    case IBM3D_F_N2: src = d->Np[1]; break;
    case IBM3D_F_N3: src = d->Np[2]; break;
    case IBM3D_F_LVSET: src = d->lvset; break;
    case IBM3D_F_COEFFSUM:
        memcpy(out, s->p_coeffsum, sizeof(double) * n);
        return;
    default:
        if (field >= IBM3D_F_TAU11 && field <= IBM3D_F_TAU33) {
            src = d->tau[field - IBM3D_F_TAU11];
            break;
        }
        set_status(s, IBM3D_EARG, "unknown field %d", field);
        return;
    }
    if (face < 0) {
        cudaMemcpyAsync(out, src, sizeof(double) * n, cudaMemcpyDeviceToHost, d->s);
        cuda_check(s, cudaStreamSynchronize(d->s), "get_field");
        return;
    }
    std::vector<double> h(n);
    cudaMemcpyAsync(h.data(), src, sizeof(double) * n, cudaMemcpyDeviceToHost, d->s);
    if (!cuda_check(s, cudaStreamSynchronize(d->s), "get_field")) return;
    const int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz;
    size_t q = 0;
    if (face == 0) {
        for (int i = 0; i <= Nx; i++)
            for (int j = -2; j < Ny + 2; j++)
                for (int k = -2; k < Nz + 2; k++) out[q++] = h[cidx(g, i, j, k)];
    } else if (face == 1) {
        for (int i = -2; i < Nx + 2; i++)
            for (int j = 0; j <= Ny; j++)
                for (int k = -2; k < Nz + 2; k++) out[q++] = h[cidx(g, i, j, k)];
    } else {
        for (int i = -2; i < Nx + 2; i++)
            for (int j = -2; j < Ny + 2; j++)
                for (int k = 0; k <= Nz; k++) out[q++] = h[cidx(g, i, j, k)];
    }
}

void IBMSolver_get_flag(IBMSolver *s, int *out) {
    if (!check_ready(s, "IBMSolver_get_flag")) return;
    memcpy(out, s->flag, sizeof(int) * (size_t)ncell_of(s));
}

void IBMSolver_sync_host(IBMSolver *s) {
    if (!check_ready(s, "IBMSolver_sync_host")) return;
    IBMSolver_get_field(s, IBM3D_F_U1, s->u1);
    IBMSolver_get_field(s, IBM3D_F_U2, s->u2);
    IBMSolver_get_field(s, IBM3D_F_U3, s->u3);
    IBMSolver_get_field(s, IBM3D_F_P, s->p);
}

int IBMSolver_num_ghost(IBMSolver *s) { return s && s->dev ? s->dev->nghost : 0; }

int IBMSolver_num_ghost_levels(IBMSolver *s) { return s && s->dev ? s->dev->nlevels : 0; }

void IBMSolver_get_ghost_stencils(IBMSolver *s, int *ijk, int *idx, double *coeff) {
    if (!check_ready(s, "IBMSolver_get_ghost_stencils")) return;
    ibm3d_device *d = s->dev;
    for (int q = 0; q < d->nghost; q++) {
        int i, j, k;
        cijk(d->g, d->gcell_lex[q], i, j, k);
        ijk[3 * q] = i;
        ijk[3 * q + 1] = j;
        ijk[3 * q + 2] = k;
        const GhostStencil &st = d->gst[q];
        for (int l = 0; l < 8; l++) {
            idx[24 * q + 3 * l] = st.im + !!(l & 4);
            idx[24 * q + 3 * l + 1] = st.jm + !!(l & 2);
            idx[24 * q + 3 * l + 2] = st.km + !!(l & 1);
            coeff[8 * q + l] = st.raw[l];
        }
    }
}

void IBMSolver_get_stats(const IBMSolver *s, IBMSolverStats *out) {
    const ibm3d_device *d = s->dev;
    memset(out, 0, sizeof *out);
    out->iter = s->iter;
    out->time = s->time;
    for (int l = 0; l < 3; l++) {
        out->iters_u[l] = d->rep_mom.iters[l];
        out->res_u[l] = d->rep_mom.relres[l];
    }
    out->iters_p = d->rep_p.iters[0];
    out->res_p = d->rep_p.relres[0];
    out->max_div = d->max_div;
    out->mg_levels = d->mg ? d->mg->nlevels() : 0;
    out->outer_u = d->rep_mom.outer;
    out->outer_p = d->rep_p.outer;
    out->cpt_fallback = d->cpt_fallback;
    out->steps_total = d->steps_total;
    for (int l = 0; l < 3; l++) out->iters_u_total[l] = d->iters_u_total[l];
    out->iters_p_total = d->iters_p_total;
    out->outer_p_total = d->outer_p_total;
    out->max_div_max = d->max_div_max;
}

double IBMSolver_time_iterate(IBMSolver *s, int nsteps) {
    if (!check_ready(s, "IBMSolver_time_iterate")) return -1;
    ibm3d_device *d = s->dev;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaStreamSynchronize(d->s);
    cudaEventRecord(a, d->s);
    IBMSolver_iterate(s, nsteps, false);
    cudaEventRecord(b, d->s);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

// Picks the pressure multigrid's smoother sweeps for this case and
// arithmetic mode by measurement: from the current state, each candidate
// runs `steps` recorded steps (after one untimed step that records its
// graphs) and the fastest wins.  The state (every field a step reads, time
// and iteration count) is restored after each trial and at the end, so the
// run continues exactly as if the tuner had not run.
double IBMSolver_autotune(IBMSolver *s, int steps, int *best_out) {
    if (!check_ready(s, "IBMSolver_autotune")) return -1;
    ibm3d_device *d = s->dev;
    if (steps < 1) steps = 1;
    static const int cand[][5] = {{5, 5, 1, 1, 8},  {4, 4, 1, 1, 8},  {6, 6, 1, 1, 8},  {3, 3, 1, 1, 8},
                                  {4, 4, 2, 2, 8},  {3, 3, 2, 2, 8},  {5, 5, 2, 2, 16}, {2, 2, 2, 2, 8},
                                  {4, 4, 2, 2, 16}, {6, 6, 2, 2, 16}, {3, 3, 2, 2, 16}, {5, 5, 1, 1, 16}};
    const int ncand = (int)(sizeof cand / sizeof cand[0]);
    const size_t n = (size_t)d->g.ncell;
    double *save = nullptr;
    if (!cuda_check(s, cudaMalloc(&save, sizeof(double) * (n * kStateFields + 1)), "autotune state")) return -1;
    // By role (the steps swap the buffers behind the roles).
    auto copy_state = [&](bool out) {
        double *fld[kStateFields];
        state_fields(d, fld);
        for (int q = 0; q < kStateFields; q++)
            cudaMemcpyAsync(out ? save + q * n : fld[q], out ? fld[q] : save + q * n, sizeof(double) * n,
                            cudaMemcpyDeviceToDevice, d->s);
        int *hist_save = (int *)(save + n * kStateFields);
        cudaMemcpyAsync(out ? hist_save : d->pp_hist, out ? d->pp_hist : hist_save, sizeof(int),
                        cudaMemcpyDeviceToDevice, d->s);
    };
    copy_state(true);
    const int iter0 = s->iter;
    const double time0 = s->time;
    const double omega = d->mg_omega;
    int keep[5];
    for (int q = 0; q < 5; q++) keep[q] = d->mg_sweeps[q];
    double best = -1;
    int bi = -1;
    for (int c = 0; c < ncand && d->status != IBM3D_ECUDA; c++) {
        IBMSolver_set_multigrid(s, cand[c][0], cand[c][1], cand[c][2], cand[c][3], cand[c][4], omega);
        copy_state(false);
        s->iter = iter0;
        s->time = time0;
        // Records this configuration's graphs for both buffer parities (the
        // steps alternate the field buffers), so the timed steps record none.
        IBMSolver_iterate(s, 2, false);
        copy_state(false);
        s->iter = iter0;
        s->time = time0;
        const double ms = IBMSolver_time_iterate(s, steps) / steps;
        if (d->status != IBM3D_OK && d->status != IBM3D_ENOCONV) break;
        if (best < 0 || ms < best) {
            best = ms;
            bi = c;
        }
    }
    const int *w = bi >= 0 ? cand[bi] : keep;
    IBMSolver_set_multigrid(s, w[0], w[1], w[2], w[3], w[4], omega);
    copy_state(false);
    s->iter = iter0;
    s->time = time0;
    cuda_check(s, cudaStreamSynchronize(d->s), "autotune");
    cudaFree(save);
    if (best_out)
        for (int q = 0; q < 5; q++) best_out[q] = w[q];
    return best;
}

double IBMSolver_time_kernel(IBMSolver *s, int which, int reps, double *bytes) {
    if (!check_ready(s, "IBMSolver_time_kernel")) return -1;
    ibm3d_device *d = s->dev;
    const bool cold = (which & IBM3D_K_COLD) != 0;
    which &= ~IBM3D_K_COLD;
    const bool mixed = d->precision != IBM3D_FP64;   // FP32 multigrid
    const bool f32 = step32(d);
    const double ncell = (double)d->g.ncell, nint = (double)d->g.nx * d->g.ny * d->g.nz;
    double b = 0;
    std::function<void()> launch;
    switch (which) {
    case IBM3D_K_MG_COLOR:
        // Scratch vectors of the pressure solve of the current precision.
        launch = [&]() {
            double bb;
            if (mixed) d->mg32->time_color(d->s, d->irpres.inner.r, d->irpres.inner.s, 1, &bb, false);
            else d->mg->time_color(d->s, d->kpres.r, d->kpres.s, 1, &bb, false);
            b = bb;
        };
        break;
    case IBM3D_K_SPMV_P:
        launch = [&]() {
            if (pres_ir(s)) apply_operator<float>(d->s, d->A32, OP_PRES, 0, d->irpres.inner.r, d->irpres.inner.s);
            else apply_operator<double>(d->s, d->A64, OP_PRES, 0, d->kpres.r, d->kpres.s);
        };
        b = ncell * (3 * (pres_ir(s) ? 4.0 : 8.0) + 1);
        break;
    case IBM3D_K_CONV_RHS:
        // Reads u, U (3 each), p, N_prev (3), flag; writes N (3), b (3).
        launch = [&]() { stage_rhs(s); };
        b = ncell * (f32 ? 7 * 8.0 + 3 * 4.0 + 1 + 6 * 4.0 : 10 * 8.0 + 1 + 6 * 8.0);
        break;
    case IBM3D_K_USTAR_PRHS:
        // Reads u* (or u^n and the FP32 increment), p, flag; writes U* (3), b.
        launch = [&]() { stage_ustar(s); };
        b = ncell * (f32 ? 3 * 8.0 + 3 * 4.0 + 8 + 1 + 8 + 4 * 8.0 : 4 * 8.0 + 1 + 4 * 8.0);
        break;
    case IBM3D_K_UPDATE_NEXT:
        // Reads u* (or u^n and the increment), U* (3), p, p', flag; writes u, U (3 each), p.
        launch = [&]() { stage_next(s); };
        b = nint * (f32 ? 3 * 8.0 + 3 * 4.0 + 3 * 8.0 + 16 + 1 + 7 * 8.0 : 8 * 8.0 + 1 + 7 * 8.0);
        break;
    default:
        set_status(s, IBM3D_EARG, "IBMSolver_time_kernel: unknown kernel %d", which);
        return -1;
    }
    const bool prof_on = d->prof.on;
    d->prof.on = false;
    cudaStreamSynchronize(d->s);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    void *flush = nullptr;
    const size_t flush_bytes = (size_t)256 << 20;   // twice the 129 MB L2
    if (cold && cudaMalloc(&flush, flush_bytes) != cudaSuccess) flush = nullptr;
    double total = 0;
    if (cold && flush) {
        for (int q = 0; q < reps; q++) {
            cudaMemsetAsync(flush, q & 0xff, flush_bytes, d->s);
            cudaEventRecord(e0, d->s);
            launch();
            cudaEventRecord(e1, d->s);
            cudaEventSynchronize(e1);
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            total += t;
        }
    } else {
        cudaEventRecord(e0, d->s);
        for (int q = 0; q < reps; q++) launch();
        cudaEventRecord(e1, d->s);
        cudaEventSynchronize(e1);
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        total = t;
    }
    d->prof.on = prof_on;
    if (flush) cudaFree(flush);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (bytes) *bytes = b;
    if (!cuda_check(s, cudaGetLastError(), "IBMSolver_time_kernel")) return -1;
    return reps > 0 ? total / reps : 0;
}

double IBMSolver_measure_fma_rate(int which) { return ibm::fma_rate(which == 0 ? 0 : 1); }

void IBMSolver_set_profiling(IBMSolver *s, int on) {
    s->dev->prof.reset();
    s->dev->prof.on = on != 0;
}

int IBMSolver_get_profile(IBMSolver *s, int max, char names[][32], int *launches, double *total_ms) {
    ibm3d_device *d = s->dev;
    d->prof.flush();
    int q = 0;
    for (auto &kv : d->prof.total) {
        if (q >= max) break;
        snprintf(names[q], 32, "%s", kv.first.c_str());
        launches[q] = (int)kv.second.first;
        total_ms[q] = kv.second.second;
        q++;
    }
    return q;
}

long long IBMSolver_kernel_launches(void) { return ibm::g_launches.load(); }

int IBMSolver_check_fp32_conversions(long long n, const double *values, unsigned long long *mismatches) {
    if (n <= 0 || !values || !mismatches) return -1;
    return ibm::conversion_check(n, values, mismatches);
}

int IBMSolver_host_register(void *ptr, size_t bytes) {
    return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? 0 : -1;
}

int IBMSolver_host_unregister(void *ptr) { return cudaHostUnregister(ptr) == cudaSuccess ? 0 : -1; }

const char *IBMSolver_device_name(IBMSolver *s) { return s && s->dev ? s->dev->dev_name : ""; }

// Polyhedron_cpt (src/geo3d.c:436-704) on the GPU for an arbitrary grid.
void Polyhedron_cpt(const Polyhedron *const poly, const int nx, const int ny, const int nz, const double *x,
                    const double *y, const double *z, double *f, const double maxd) {
    CptModel m;
    build_cpt_model(poly, maxd, m);
    double *dx = nullptr, *dy = nullptr, *dz = nullptr, *df = nullptr;
    const size_t n = (size_t)nx * ny * nz;
    cudaStream_t s;
    if (cudaStreamCreate(&s) != cudaSuccess || cudaMalloc(&dx, sizeof(double) * nx) != cudaSuccess ||
        cudaMalloc(&dy, sizeof(double) * ny) != cudaSuccess || cudaMalloc(&dz, sizeof(double) * nz) != cudaSuccess ||
        cudaMalloc(&df, sizeof(double) * n) != cudaSuccess) {
        fprintf(stderr, "error: Polyhedron_cpt needs a CUDA device\n");
        std::exit(255);
    }
    cudaMemcpyAsync(dx, x, sizeof(double) * nx, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dy, y, sizeof(double) * ny, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dz, z, sizeof(double) * nz, cudaMemcpyHostToDevice, s);
    const int rc = gpu_cpt(s, m, nx, ny, nz, dx, dy, dz, df, maxd, nullptr);
    cudaMemcpyAsync(f, df, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFree(dx); cudaFree(dy); cudaFree(dz); cudaFree(df);
    cudaStreamDestroy(s);
    if (rc != 0) {
        fprintf(stderr, "error: Polyhedron_cpt kernels failed\n");
        std::exit(255);
    }
}

}  // extern "C"

// ------------------------------------------------------------- batches ---
// Many independent solvers advanced together: every batched step is ONE
// CUDA graph launch whose parallel branches are the members' recorded steps
// (each with its own device-side Krylov loops), so small cases share the
// GPU instead of running one after another.  A member's batched steps
// since it joined form one run: they compute exactly what one
// IBMSolver_iterate call of that many steps computes for it alone (same
// kernels, same order on its own data); the reference's per-call prologue
// runs when it joins, or again if it was stepped outside the batch.
struct IBMBatch {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<IBMSolver *> members;
    std::vector<cudaEvent_t> join;
    std::vector<int> next_iter;     // member's iter after its last batched step; -1: not started
    std::vector<double> run_start;  // member's time when its run in the batch began
    std::vector<int> run_steps;     // batched steps of that run so far
    struct Rec {
        std::vector<const void *> key;
        cudaGraphExec_t exec = nullptr;
        std::vector<StepGraph> parts;
    };
    std::vector<Rec> cache;
    int combined = 1;  // 1: one graph for all members; 0: each member's own step graph
    int status = IBM3D_OK;
    // A step launched by IBMBatch_launch and not yet finished.
    bool pending = false;
    Rec *pending_rec = nullptr;
    std::vector<StepGraph *> pending_own;
};

namespace {
void batch_drop(IBMBatch *b) {
    for (auto &r : b->cache)
        if (r.exec) cudaGraphExecDestroy(r.exec);
    b->cache.clear();
}

std::vector<const void *> batch_key(IBMBatch *b) {
    std::vector<const void *> k;
    for (IBMSolver *m : b->members) {
        ibm3d_device *d = m->dev;
        const GraphSig sig = graph_sig(m);
        if (!(sig == d->gsig)) {
            drop_graphs(d);
            d->gsig = sig;
        }
        k.push_back(m);
        k.push_back(d->u[0]);
        k.push_back(d->U[0]);
        k.push_back(d->p);
        k.push_back(d->N[0]);
    }
    return k;
}

bool batch_record(IBMBatch *b, IBMBatch::Rec &R) {
    bool ok = cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) ok = cudaEventRecord(b->fork, b->s) == cudaSuccess;
    R.parts.assign(b->members.size(), StepGraph{});
    for (size_t q = 0; ok && q < b->members.size(); q++) {
        ibm3d_device *d = b->members[q]->dev;
        ok = cudaStreamWaitEvent(d->s, b->fork, 0) == cudaSuccess;
        if (ok) ok = record_step_into(b->members[q], R.parts[q]);

        if (ok) ok = cudaEventRecord(b->join[q], d->s) == cudaSuccess;
        if (ok) ok = cudaStreamWaitEvent(b->s, b->join[q], 0) == cudaSuccess;
    }
    // A failed recording can leave a loop-body capture open on an aux
    // stream; close those before the parent capture.
    for (IBMSolver *m : b->members) close_open_captures(m->dev);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->s, &graph);
    ok = ok && ec == cudaSuccess && graph;
    if (ok) ok = cudaGraphInstantiate(&R.exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return ok;
}
}  // namespace

IBMBatch *IBMBatch_new(void) {
    IBMBatch *b = new IBMBatch();
    if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess) {
        fprintf(stderr, "error: IBMBatch_new: no usable GPU\n");
        b->status = IBM3D_ECUDA;
    }
    return b;
}

namespace {
bool batch_finish(IBMBatch *b);
}

void IBMBatch_destroy(IBMBatch *b) {
    if (!b) return;
    batch_finish(b);
    batch_drop(b);
    for (auto e : b->join) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->s) cudaStreamDestroy(b->s);
    delete b;
}

int IBMBatch_add(IBMBatch *b, IBMSolver *s) {
    if (b && b->pending) {
        fprintf(stderr, "error: IBMBatch_add: a launched step has not been waited for\n");
        return -1;
    }
    if (!b || !s || !s->dev || !s->dev->assembled) {
        fprintf(stderr, "error: IBMBatch_add: the solver must be assembled first\n");
        return -1;
    }
    for (IBMSolver *m : b->members)
        if (m == s) return 0;
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return -1;
    b->members.push_back(s);
    b->join.push_back(e);
    b->next_iter.push_back(-1);
    b->run_start.push_back(0.0);
    b->run_steps.push_back(0);
    batch_drop(b);
    return 0;
}

int IBMBatch_remove(IBMBatch *b, IBMSolver *s) {
    if (b->pending) {
        fprintf(stderr, "error: IBMBatch_remove: a launched step has not been waited for\n");
        return -1;
    }
    for (size_t q = 0; q < b->members.size(); q++)
        if (b->members[q] == s) {
            b->members.erase(b->members.begin() + q);
            cudaEventDestroy(b->join[q]);
            b->join.erase(b->join.begin() + q);
            b->next_iter.erase(b->next_iter.begin() + q);
            b->run_start.erase(b->run_start.begin() + q);
            b->run_steps.erase(b->run_steps.begin() + q);
            batch_drop(b);
            return 0;
        }
    return -1;
}

int IBMBatch_size(const IBMBatch *b) { return b ? (int)b->members.size() : 0; }

namespace {

// First half of a batched step: joins new members (their iterate
// prologue), then launches the step of every member - one graph over all
// members, or each member's own step graph on its stream - without
// waiting for it.  Returns false on a recording or launch failure.
bool batch_launch(IBMBatch *b) {
    for (size_t q = 0; q < b->members.size(); q++) {
        IBMSolver *m = b->members[q];
        if (b->next_iter[q] != m->iter) {  // joined, or stepped outside the batch: a new run
            b->run_start[q] = m->time;
            b->run_steps[q] = 0;
            iterate_prologue(m);
            b->next_iter[q] = m->iter;
        }
        m->dev->status = IBM3D_OK;
        cudaEventRecord(b->join[q], m->dev->s);
        cudaStreamWaitEvent(b->s, b->join[q], 0);
    }
    if (!b->combined) {
        // Each member's own recorded step on its own stream, all forked
        // from and joined into the batch stream.
        b->pending_own.assign(b->members.size(), nullptr);
        for (size_t q = 0; q < b->members.size(); q++) {
            b->pending_own[q] = step_graph(b->members[q]);
            if (!b->pending_own[q]) {
                fprintf(stderr, "error: IBMBatch_iterate: recording a member's step failed\n");
                return false;
            }
        }
        cudaEventRecord(b->fork, b->s);
        for (size_t q = 0; q < b->members.size(); q++) {
            IBMSolver *m = b->members[q];
            cudaStreamWaitEvent(m->dev->s, b->fork, 0);
            prepare_samples(m, m->dev->s, m->time, b->run_start[q] + m->dt * (b->run_steps[q] + 1));
            cudaGraphLaunch(b->pending_own[q]->exec, m->dev->s);
            cudaEventRecord(b->join[q], m->dev->s);
            cudaStreamWaitEvent(b->s, b->join[q], 0);
        }
        b->pending = true;
        return true;
    }
    for (size_t q = 0; q < b->members.size(); q++) {
        IBMSolver *m = b->members[q];
        prepare_samples(m, b->s, m->time, b->run_start[q] + m->dt * (b->run_steps[q] + 1));
    }
    const std::vector<const void *> key = batch_key(b);
    IBMBatch::Rec *R = nullptr;
    for (auto &r : b->cache)
        if (r.key == key) R = &r;
    if (!R) {
        if (b->cache.size() >= 4) batch_drop(b);
        IBMBatch::Rec nr;
        nr.key = key;
        if (!batch_record(b, nr)) {
            fprintf(stderr, "error: IBMBatch_iterate: recording the batched step failed\n");
            return false;
        }
        b->cache.push_back(nr);
        R = &b->cache.back();
    }
    if (cudaGraphLaunch(R->exec, b->s) != cudaSuccess) {
        fprintf(stderr, "error: IBMBatch_iterate: %s\n", cudaGetErrorString(cudaGetLastError()));
        return false;
    }
    b->pending_rec = R;
    b->pending = true;
    return true;
}

// Second half: waits for the launched step and books it for every member
// (solve reports, warnings, pointer swaps, iteration count and time).
bool batch_finish(IBMBatch *b) {
    if (!b->pending) return true;
    b->pending = false;
    if (cudaStreamSynchronize(b->s) != cudaSuccess) {
        fprintf(stderr, "error: IBMBatch_iterate: %s\n", cudaGetErrorString(cudaGetLastError()));
        return false;
    }
    for (size_t q = 0; q < b->members.size(); q++) {
        IBMSolver *m = b->members[q];
        finish_step(m, b->combined ? b->pending_rec->parts[q] : *b->pending_own[q]);
        m->iter++;
        b->run_steps[q]++;
        b->next_iter[q] = m->iter;
        m->time = b->run_start[q] + m->dt * b->run_steps[q];
        m->dev->max_div = *m->dev->maxdiv_h;
        account_step(m->dev);
        if (m->dev->status != IBM3D_OK && m->dev->status != IBM3D_ENOCONV) b->status = m->dev->status;
    }
    return true;
}

}  // namespace

double IBMBatch_iterate(IBMBatch *b, int nsteps) {
    if (!b || b->members.empty() || nsteps < 1) return 0.0;
    if (b->pending && !batch_finish(b)) {
        b->status = IBM3D_ECUDA;
        return -1;
    }
    b->status = IBM3D_OK;
    cudaEventRecord(b->t0, b->s);
    for (int i = 1; i <= nsteps; i++) {
        if (!batch_launch(b) || !batch_finish(b)) {
            b->status = IBM3D_ECUDA;
            return -1;
        }
    }
    cudaEventRecord(b->t1, b->s);
    cudaEventSynchronize(b->t1);
    float ms = 0;
    cudaEventElapsedTime(&ms, b->t0, b->t1);
    return ms;
}

int IBMBatch_launch(IBMBatch *b) {
    if (!b || b->members.empty() || b->pending) return -1;
    b->status = IBM3D_OK;
    if (!batch_launch(b)) {
        b->status = IBM3D_ECUDA;
        return -1;
    }
    return 0;
}

int IBMBatch_wait(IBMBatch *b) {
    if (!b) return -1;
    if (!batch_finish(b)) {
        b->status = IBM3D_ECUDA;
        return -1;
    }
    return 0;
}

int IBMBatch_last_status(const IBMBatch *b) { return b ? b->status : IBM3D_EARG; }

void IBMBatch_set_combined(IBMBatch *b, int on) {
    if (!b) return;
    b->combined = on != 0;
    batch_drop(b);
}

size_t IBMSolver_device_bytes(const IBMSolver *s) { return s && s->dev ? s->dev->dev_bytes : 0; }
