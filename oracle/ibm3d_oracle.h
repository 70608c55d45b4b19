/*
 * CPU oracle of the reference's 3D immersed-boundary fractional step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of
 * thecasterian/2020ResearchProject's time step (src/ibm3d_fracstep.c,
 * src/ibm3d_setup.c, src/ibm3d_turb.c, src/utils.c, src/geo3d.c), used by
 * tests/ as the parity checker, by __graft_entry__.smoke() and by bench.py's
 * CPU-baseline leg.  The product (the GPU library) never links or calls it.
 *
 * Parity of this restatement is pinned against the golden fixtures in
 * tests/golden/, which were produced by running the reference's own C
 * sources (see tests/golden/make_golden.py).
 *
 * Arrays use the reference's layouts: cell fields (Nx+4)(Ny+4)(Nz+4) with
 * k fastest; face fields U1 (Nx+1)(Ny+4)(Nz+4), U2 (Nx+4)(Ny+1)(Nz+4),
 * U3 (Nx+4)(Ny+4)(Nz+1).
 */
#ifndef IBM3D_ORACLE_H
#define IBM3D_ORACLE_H

typedef struct {
    int nx, ny, nz;
    const double *xf, *yf, *zf;     /* nx+1, ny+1, nz+1 face coordinates */
    double Re, dt;
    int bc_type[6];                 /* reference BC enum, faces N E S W D U */
    double bc_u[6][3], bc_p[6];
    double force[3];
    double smagorinsky_cs;          /* < 0: no turbulence model */
    double tol;                     /* Krylov relative tolerance */
    double div_tol;                 /* > 0: pressure stops at max|div U| <= div_tol */
    const char *stl_path;           /* NULL: no obstacle */
    const double *lvset_in;         /* optional precomputed level set (padded); skips the CPT */
    int threads;                    /* OpenMP threads, 0 = runtime default */
    /* VAL_FUNC values (src/ibm3d.h:52-80): per face u1, u2, u3, p; NULL
       keeps the constant value.  Callbacks (t, x, y, z). */
    double (*bc_fn[6][4])(double, double, double, double);
    double (*force_fn[3])(double, double, double, double);
} OracleConfig;

typedef struct Oracle Oracle;

Oracle *oracle_create(const OracleConfig *cfg);
void oracle_destroy(Oracle *o);
void oracle_init(Oracle *o, const double *u1, const double *u2, const double *u3, const double *p);
void oracle_iterate(Oracle *o, int nsteps);
/* Field names: u1 u2 u3 p U1 U2 U3 u1star u2star u3star U1star U2star U3star
   pprime N1 N2 N3 lvset coeffsum.  Returns 0, or -1 for an unknown name. */
int oracle_get(Oracle *o, const char *name, double *out);
void oracle_flag(Oracle *o, int *out);
int oracle_num_ghost(Oracle *o);
/* Ghosts in lexicographic order: ijk (n*3), idx (n*8*3), coeff (n*8). */
void oracle_ghost_stencils(Oracle *o, int *ijk, int *idx, double *coeff);
/* Last step: iterations (u1,u2,u3,p), relative residuals, max |div U|. */
void oracle_stats(Oracle *o, int *iters, double *res, double *max_div);

#endif
