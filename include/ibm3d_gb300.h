/*
 * ibm3d-gb300 extensions to the reference C ABI.
 *
 * None of these exist in the reference; they are additive and never change
 * the behaviour of the reference entry points.  They serve callers that
 * cannot use C varargs (FFI layers), expose per-step solver statistics and
 * device timing, and let a host hand fields to the GPU and read them back.
 */
#ifndef IBM3D_GB300_H
#define IBM3D_GB300_H

#include <stddef.h>

#include "ibm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status of the last call on a solver: 0 ok, otherwise an IBM3D_E* code. */
enum {
    IBM3D_OK = 0,
    IBM3D_ENOCONV = 1,      /* a Krylov solve hit its iteration cap (warning, as in the reference) */
    IBM3D_EBREAKDOWN = 2,   /* BiCGSTAB breakdown */
    IBM3D_ECUDA = 3,        /* CUDA error or no usable GPU */
    IBM3D_EARG = 4,         /* invalid argument or call order */
    IBM3D_EGEOM = 5,        /* ghost-cell mirror point outside the grid */
    IBM3D_EUNSUPPORTED = 6, /* feature not available on the GPU path */
    IBM3D_ENONFINITE = 7    /* NaN or Inf in a step: in the initial state, the
                               boundary data or force, or a diverging run; the
                               iterate call stops after that step */
};
int IBMSolver_last_status(const IBMSolver *);
/* Text of the last error set on this solver ("" if none); the reference
   prints such errors and aborts (e.g. src/ibm3d_init.c:88-90). */
const char *IBMSolver_last_message(const IBMSolver *);
const char *IBMSolver_status_string(int status);

/* Non-variadic forms of set_bc / set_ext_force / set_turb_model (same
   semantics as the VAL_CONST variadic calls). */
void IBMSolver_set_bc_const(IBMSolver *, IBMSolverDirection, IBMSolverBCType,
                            double u1, double u2, double u3, double p);
void IBMSolver_set_ext_force_const(IBMSolver *, double f1, double f2, double f3);
/* Non-variadic forms of the VAL_FUNC calls (src/ibm3d_setup.c:306-327,
   365-434): set_bc(dir, BC_VELOCITY_COMPONENT, VAL_FUNC, f1, f2, f3) and
   set_bc(dir, BC_PRESSURE or BC_VELOCITY_PERIODIC, VAL_FUNC, fp) (the
   unused functions may be NULL); set_ext_force(VAL_FUNC, f1, f2, f3).
   The callbacks run on the host: once per step for every outer line of a
   VAL_FUNC face (start and end time of the step) and, for a VAL_FUNC
   force, for every interior cell centre at the step's start time. */
void IBMSolver_set_bc_func(IBMSolver *, IBMSolverDirection, IBMSolverBCType,
                           IBMSolverBCValFunc f1, IBMSolverBCValFunc f2, IBMSolverBCValFunc f3,
                           IBMSolverBCValFunc fp);
void IBMSolver_set_ext_force_func(IBMSolver *, IBMSolverForceFunc f1, IBMSolverForceFunc f2,
                                  IBMSolverForceFunc f3);
void IBMSolver_set_smagorinsky(IBMSolver *, double Cs);

/* Pressure-solve stopping rule.  div_tol > 0: stop once the projected face
   velocity satisfies max|div U^{n+1}| <= div_tol on fluid cells; 0 (the
   default) keeps the reference's ||r||/||b|| < tol rule. */
void IBMSolver_set_div_tol(IBMSolver *, double div_tol);

/* Arithmetic of the linear solves.  IBM3D_FP64 (default): FP64 BiCGSTAB
   with an FP64 multigrid preconditioner, as the reference.  IBM3D_MIXED:
   FP64 iterative refinement (residuals, updates and the stopping test in
   FP64, on the exact FP64 rows) around FP32 BiCGSTAB solves with an FP32
   multigrid preconditioner; it stops on the same FP64 criterion.
   IBM3D_MIXED_MG: momentum as IBM3D_MIXED; the pressure solve is FP64
   BiCGSTAB whose preconditioner is the FP32 multigrid V-cycle (input
   rounded to FP32, output widened to FP64).  In these three modes every
   other part of the step stays FP64.
   IBM3D_MIXED32: the explicit stages in FP32 as well - convection and the
   momentum right-hand side, u~ and U* - and the momentum solve in FP32 on
   the increment e = u* - u^n (right-hand side c = b - A u^n formed in
   FP32 without the O(1) cancellation, stopping test ||c - A e|| <
   tol ||b|| / 2); FP64 for the state updates u^{n+1} = u^n + (e - dt G p'),
   the face projection, p, the Poisson right-hand side (the FP64 divergence
   of U*) and the pressure solve as IBM3D_MIXED_MG.  Its results differ
   from the FP64 step by the FP32 rounding of O(dt) increments (~1e-7
   relative velocity after a few hundred steps); max|div U| is driven to
   the same bound.  IBM3D_MIXED32_IR: the same, with the pressure solved
   as in IBM3D_MIXED (FP64 refinement around FP32 BiCGSTAB with the FP32
   multigrid). */
enum { IBM3D_FP64 = 0, IBM3D_MIXED = 1, IBM3D_MIXED_MG = 2, IBM3D_MIXED32 = 3, IBM3D_MIXED32_IR = 4 };
void IBMSolver_set_precision(IBMSolver *, int mode);

/* Step sequencing.  on (default): each time step runs as one recorded CUDA
   graph whose linear solves iterate on the device (conditional while
   nodes), with one host synchronisation per step; off: the host sequences
   every kernel and reads the Krylov scalars after each half iteration.
   Both give bitwise identical results.  Stage profiling
   (IBMSolver_set_profiling) always uses the host-sequenced form. */
void IBMSolver_set_graphs(IBMSolver *, int on);

/* Pressure multigrid V-cycle: Gauss-Seidel sweeps before and after the
   coarse-grid correction on the fine grid (nu_pre, nu_post) and on the
   coarse levels (nuc_pre, nuc_post), sweeps on the coarsest level, and the
   over-relaxation weight of the fine-grid fluid rows (0 < omega < 2;
   defaults 3, 3, 2, 2, 16, 1.0).  Tuning only: the solve still stops on the
   same residual or divergence test. */
void IBMSolver_set_multigrid(IBMSolver *, int nu_pre, int nu_post, int nuc_pre, int nuc_post, int coarse_sweeps,
                             double omega);

/* Mixed modes: start the momentum solve from the current velocity (on,
   the default) instead of zero.  u* differs from u^n by O(dt), so the
   first FP64 refinement residual is small against ||b|| and the FP32
   inner solve stops sooner; the stopping test (||r|| < tol ||b||) is the
   same.  The plain FP64 step always starts from zero, as the reference. */
void IBMSolver_set_warm_start(IBMSolver *, int on);

/* Self-test of the integer-pipe FP64 <-> FP32 conversions of the
   IBM3D_MIXED32 stages against the hardware conversion instructions on
   the GPU: each of the n values is converted both ways; *mismatches counts
   the results that differ bit for bit (values on an exact rounding tie,
   which these round away from zero and the hardware to even, and FP32
   subnormals, which these flush to zero, are the expected differences).
   Returns 0, or -1 on a CUDA error or bad argument. */
int IBMSolver_check_fp32_conversions(long long n, const double *values, unsigned long long *mismatches);

/* Initial guess of a warm-started pressure solve (the mixed modes):
   0 the last step's increment p'; 1 (default) its linear extrapolation
   2 p'_{n-1} - p'_{n-2} once two increments are known.  The solve stops
   on the same test either way; both increments are part of the
   exact-resume state.  Measured with IBM3D_MIXED32: 3.9 against 4.15
   pressure iterations per step on the sphere (192x128x128), 13.4 against
   16.1 on the LES channel (128x96x128), the same on the 64^3 cavity. */
void IBMSolver_set_pressure_guess(IBMSolver *, int mode);

/* Storage and arithmetic of the IBM3D_MIXED32 pressure BiCGSTAB's vectors:
   IBM3D_PVEC_DFLOAT (default) keeps each entry as a double-float, the
   unevaluated sum of two FP32 words (48-bit significand), and runs the
   vector and operator arithmetic as error-free FP32 transformations;
   IBM3D_PVEC_FP64 keeps FP64 vectors.  Either way the right-hand side,
   the solution p' and the scalars of the iteration (alpha, omega, rho, the
   norms and the combination of the dot products) are FP64, the stopping
   test is the same and max|div U| is checked in FP64 after the
   projection.  GB300 issues FP64 operations at 1/72 of its FP32 rate:
   the FP64 vectors make the solve FP64-bound, the double-float ones bring
   it near the memory bound.  The preconditioned vectors are the FP32
   multigrid's output as it comes (FP32 entries); without the multigrid
   preconditioner (PRECOND_AMG) the vectors stay FP64.  Other precision
   modes ignore the setting. */
enum { IBM3D_PVEC_FP64 = 0, IBM3D_PVEC_DFLOAT = 1 };
void IBMSolver_set_pressure_vectors(IBMSolver *, int kind);

/* Krylov iteration caps of the momentum and pressure solves (defaults
   200 and 1000, the reference's hypre settings, src/ibm3d_setup.c:1411-1563).
   A solve that reaches its cap prints the reference's warning
   ("warning: u0_star did not converge", "warning: p_prime did not
   converge") and the step continues, as in the reference. */
void IBMSolver_set_max_iters(IBMSolver *, int max_mom, int max_p);

/* Coarsening of the pressure multigrid (before IBMSolver_assemble).
   IBM3D_COARSEN_SPACING (default): a coarse level merges neighbouring
   cells along an axis only while their joint width is at most
   width_ratio x 2^(level+1) x the finest width (width_ratio in [1, 64];
   0 = the default 1.5), so the small cells of a stretched grid coarsen
   first and the levels stay near isotropic; each level keeps at most half
   the cells of the one before.  IBM3D_COARSEN_HALVE: every level halves
   every axis (width_ratio unused).  The two coincide on uniform grids.
   Tuning only: the solve stops on the same test. */
enum { IBM3D_COARSEN_HALVE = 0, IBM3D_COARSEN_SPACING = 1 };
void IBMSolver_set_coarsening(IBMSolver *, int mode, double width_ratio);

/* Restart length of SOLVER_GMRES pressure solves (1..32; default 10, the
   reference's KDim).  The GMRES is flexible (it keeps every preconditioned
   vector), so the FP32 multigrid of the mixed modes may precondition it. */
void IBMSolver_set_gmres_restart(IBMSolver *, int restart);

/* Autotuner: times `steps` recorded steps of this case, from its current
   state, under each of a fixed set of multigrid sweep configurations
   (fine pre/post, coarse pre/post, coarsest), keeps the fastest (written
   to best[5] when best is not NULL) and returns its milliseconds per step.
   The solver's state is restored, so the run continues unchanged. */
double IBMSolver_autotune(IBMSolver *, int steps, int *best);

/* Mixed path (IBM3D_MIXED): relative tolerance of each FP32 inner solve of
   the momentum and pressure refinement cycles, and the cycle cap.  The
   outer FP64 stopping rule is unchanged.  Defaults 5e-7, 1e-5, 12. */
void IBMSolver_set_refinement(IBMSolver *, double inner_tol_mom, double inner_tol_p, int max_outer);

/* Initial state from host arrays in the padded (N+4)^3 layout, k fastest
   (u1, u2, u3, p).  Sets iter = 0 and time = 0 like init_flow_const. */
void IBMSolver_init_flow_array(IBMSolver *, const double *u1, const double *u2, const double *u3, const double *p);

/* Field read-back in the reference's layouts.  Cell fields: (Nx+4)(Ny+4)(Nz+4);
   U1: (Nx+1)(Ny+4)(Nz+4); U2: (Nx+4)(Ny+1)(Nz+4); U3: (Nx+4)(Ny+4)(Nz+1). */
enum {
    IBM3D_F_U1 = 0, IBM3D_F_U2, IBM3D_F_U3, IBM3D_F_P,
    IBM3D_F_FACE_U1, IBM3D_F_FACE_U2, IBM3D_F_FACE_U3,
    IBM3D_F_USTAR1, IBM3D_F_USTAR2, IBM3D_F_USTAR3,
    IBM3D_F_FACE_USTAR1, IBM3D_F_FACE_USTAR2, IBM3D_F_FACE_USTAR3,
    IBM3D_F_PPRIME, IBM3D_F_N1, IBM3D_F_N2, IBM3D_F_N3,
    IBM3D_F_LVSET, IBM3D_F_COEFFSUM,
    IBM3D_F_TAU11, IBM3D_F_TAU12, IBM3D_F_TAU13, IBM3D_F_TAU22, IBM3D_F_TAU23, IBM3D_F_TAU33,
    IBM3D_F_COUNT
};
void IBMSolver_get_field(IBMSolver *, int field, double *out);
void IBMSolver_get_flag(IBMSolver *, int *out);
/* Copies u1, u2, u3, p into the struct's host mirrors. */
void IBMSolver_sync_host(IBMSolver *);

/* Ghost cells, in lexicographic (i, j, k) order.  For each ghost: its
   (i, j, k), the 8 stencil cells and raw trilinear weights exactly as
   IBMSolver_ghost_interp returns them (computed on the GPU). */
int IBMSolver_num_ghost(IBMSolver *);
void IBMSolver_get_ghost_stencils(IBMSolver *, int *ijk, int *interp_idx, double *interp_coeff);
/* Dependency levels of the in-place ghost update. */
int IBMSolver_num_ghost_levels(IBMSolver *);

typedef struct {
    int iter;               /* solver->iter after the step */
    double time;
    int iters_u[3];         /* BiCGSTAB iterations, momentum components */
    int iters_p;            /* BiCGSTAB iterations, pressure */
    double res_u[3];        /* final relative residual norms */
    double res_p;
    double max_div;         /* max |div U^{n+1}| over fluid cells (pinned cell excluded) */
    int mg_levels;          /* pressure multigrid levels (incl. the fine grid) */
    int cpt_fallback;       /* level-set points settled by the full extrusion scan */
    int outer_u;            /* refinement cycles of the momentum solve (IBM3D_MIXED) */
    int outer_p;            /* refinement cycles of the pressure solve (IBM3D_MIXED) */
    /* Totals over every step since IBMSolver_assemble (averages over a run
       are differences of two reads). */
    long long steps_total;
    long long iters_u_total[3];
    long long iters_p_total;
    long long outer_p_total;
    double max_div_max;     /* largest per-step max|div U| */
} IBMSolverStats;
void IBMSolver_get_stats(const IBMSolver *, IBMSolverStats *);

/* Device timing: runs IBMSolver_iterate(nsteps) bracketed by CUDA events on
   the solver's stream and returns the elapsed device milliseconds. */
double IBMSolver_time_iterate(IBMSolver *, int nsteps);

/* Device time of one launch of a hot kernel on the solver's current data,
   in the current precision: the average over reps launches between CUDA
   events on the solver's stream (ms), and its algorithmic bytes per launch
   in *bytes (for a roofline).  IBM3D_K_MG_COLOR: one colour pass of the
   pressure multigrid's fine-grid smoother; IBM3D_K_SPMV_P: one pressure
   operator application (both on scratch vectors of the pressure solve).
   IBM3D_K_CONV_RHS, IBM3D_K_USTAR_PRHS, IBM3D_K_UPDATE_NEXT: the step's
   explicit kernels of the current mode (FP64, or the FP32 stages of
   IBM3D_MIXED32), re-run on the last step's inputs; they write only
   buffers the next step overwrites first.  Or IBM3D_K_COLD into which:
   an L2-sized buffer is written before each launch and only the launches
   are timed (cold cache), instead of back-to-back launches. */
enum {
    IBM3D_K_MG_COLOR = 0, IBM3D_K_SPMV_P = 1, IBM3D_K_CONV_RHS = 2, IBM3D_K_USTAR_PRHS = 3,
    IBM3D_K_UPDATE_NEXT = 4, IBM3D_K_COLD = 256
};
double IBMSolver_time_kernel(IBMSolver *, int which, int reps, double *bytes);

/* Register-only FMA throughput of this GPU (TFLOP/s, 2 flops per FMA):
   which 0 FP64, 1 FP32.  A roofline denominator for the kernels that the
   FP64 pipe, not HBM, bounds on this part. */
double IBMSolver_measure_fma_rate(int which);

/* Per-stage device time accumulated while profiling is on (CUDA events
   around each stage of each step).  Stage names: conv_rhs, tau, mom_solve,
   ustar_prhs, p_solve, update_next, fill_outer, ghost_update; plus the
   individual Krylov kernels spmv_mom, spmv_p, mg_vcycle. */
void IBMSolver_set_profiling(IBMSolver *, int on);
int IBMSolver_get_profile(IBMSolver *, int max, char names[][32], int *launches, double *total_ms);

/* Kernels this library has launched since load (all solvers). */
long long IBMSolver_kernel_launches(void);

/* Page-lock / release caller-owned host memory so that the field uploads
   (IBMSolver_init_flow_array) and read-backs (IBMSolver_get_field) it is
   used for run as direct DMA.  0 on success. */
int IBMSolver_host_register(void *ptr, size_t bytes);
int IBMSolver_host_unregister(void *ptr);

/* Device memory the solver's assembly took (bytes; the drop in free device
   memory across IBMSolver_assemble), for admission by HBM footprint. */
size_t IBMSolver_device_bytes(const IBMSolver *);

/* Device name of the solver's GPU (for logs). */
const char *IBMSolver_device_name(IBMSolver *);

/* Batches: independent solvers (any grids, bodies, Re; same GPU) advanced
   together.  Each batched step is one CUDA graph launch whose parallel
   branches are the members' recorded steps, so small cases overlap on the
   GPU.  A member's batched steps since it joined form one run: bitwise the
   results of one IBMSolver_iterate call of that many steps on the same
   solver alone (the reference's per-call prologue runs when the member
   joins, or again after it was stepped outside the batch).  Members must
   be assembled; adding or removing a member re-records the batched step
   at its next use.  IBMBatch_iterate runs nsteps steps of every member and
   returns the device milliseconds (CUDA events on the batch stream), or
   -1 on error. */
typedef struct IBMBatch IBMBatch;
IBMBatch *IBMBatch_new(void);
void IBMBatch_destroy(IBMBatch *);
int IBMBatch_add(IBMBatch *, IBMSolver *);
int IBMBatch_remove(IBMBatch *, IBMSolver *);
int IBMBatch_size(const IBMBatch *);
double IBMBatch_iterate(IBMBatch *, int nsteps);
/* One batched step in two halves: IBMBatch_launch queues the step of every
   member on the GPU and returns at once; IBMBatch_wait waits for it and
   books it (as IBMBatch_iterate(b, 1) does).  Between the two the host is
   free, e.g. to assemble solvers that join at the next step; members may
   not be added or removed then.  Both return 0, or -1 on error. */
int IBMBatch_launch(IBMBatch *);
int IBMBatch_wait(IBMBatch *);
int IBMBatch_last_status(const IBMBatch *);
/* on (default): each batched step is one graph launch over all members,
   re-recorded when the membership changes.  off: each member's own step
   graph is launched on its own stream, forked from and joined into the
   batch stream (one launch per member, nothing re-recorded when members
   come and go: what a server with churning membership wants).  Results
   are the same bit for bit either way. */
void IBMBatch_set_combined(IBMBatch *, int on);

#ifdef __cplusplus
}
#endif

#endif
