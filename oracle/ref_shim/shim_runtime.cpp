// Runtime of the MPI / GLib / netCDF / hypre stand-ins declared under
// include/.  Test infrastructure: linked only into the reference build
// (oracle/_ref), never into the product library.
//
// The hypre part stores each IJ matrix as CSR rows exactly as the reference
// sets them (src/ibm3d_setup.c:1566-2908) and solves every system with an
// ILU(0)-preconditioned BiCGSTAB to ||b-Ax||/||b|| < tol.  The reference's
// BoomerAMG options only change how hypre gets to that answer.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include <algorithm>

#include "include/mpi.h"
#include "include/glib.h"
#include "include/netcdf.h"
#include "include/HYPRE.h"

// ---------------------------------------------------------------- MPI ----
extern "C" {
int MPI_Init(int *, char ***) { return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return 0; }
int MPI_Abort(MPI_Comm, int code) {
    std::fprintf(stderr, "MPI_Abort(%d) called by the reference\n", code);
    std::exit(code == 0 ? 1 : (code & 0xff));
}
int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
    std::fprintf(stderr, "single-rank MPI stand-in: MPI_Send reached\n");
    std::abort();
}
int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
    std::fprintf(stderr, "single-rank MPI stand-in: MPI_Recv reached\n");
    std::abort();
}
}

// --------------------------------------------------------------- GLib ----
struct GTreeCmp {
    GCompareDataFunc f;
    gpointer data;
    bool operator()(gconstpointer a, gconstpointer b) const { return f(a, b, data) < 0; }
};
struct _GTree {
    std::map<gconstpointer, gpointer, GTreeCmp> m;
    GDestroyNotify kd, vd;
    explicit _GTree(GTreeCmp c) : m(c), kd(nullptr), vd(nullptr) {}
};

extern "C" {
void g_free(gpointer mem) { std::free(mem); }
GTree *g_tree_new_full(GCompareDataFunc cmp, gpointer cmp_data, GDestroyNotify kd, GDestroyNotify vd) {
    GTree *t = new _GTree(GTreeCmp{cmp, cmp_data});
    t->kd = kd;
    t->vd = vd;
    return t;
}
gpointer g_tree_lookup(GTree *t, gconstpointer key) {
    auto it = t->m.find(key);
    return it == t->m.end() ? nullptr : it->second;
}
void g_tree_insert(GTree *t, gpointer key, gpointer value) {
    auto it = t->m.find(key);
    if (it != t->m.end()) {
        // GLib semantics: keep the old key (destroying the new one), replace the value.
        if (t->kd) t->kd(key);
        if (t->vd) t->vd(it->second);
        it->second = value;
        return;
    }
    t->m.emplace(key, value);
}
gint g_tree_nnodes(GTree *t) { return (gint)t->m.size(); }
void g_tree_foreach(GTree *t, GTraverseFunc f, gpointer data) {
    for (auto &kv : t->m)
        if (f((gpointer)kv.first, kv.second, data)) break;
}
void g_tree_destroy(GTree *t) {
    for (auto &kv : t->m) {
        if (t->kd) t->kd((gpointer)kv.first);
        if (t->vd) t->vd(kv.second);
    }
    delete t;
}
}

// ------------------------------------------------------------- netCDF ----
// Writers record: with IBM3D_NC_DUMP_DIR set, every nc_put_var_* payload of
// the file being written goes to <dir>/<variable>.bin (raw, little-endian,
// the variable's element type), so the reference's own exports can be
// compared with the GPU library's.  Without it writes are discarded.
// Readers fail (the reference then aborts, src/ibm3d_init.c:223).
namespace {
struct NcState {
    std::vector<size_t> dims;
    std::vector<std::pair<std::string, std::vector<int>>> vars;
};
NcState g_nc;

void nc_record(int varid, const void *data, size_t elem) {
    const char *dir = std::getenv("IBM3D_NC_DUMP_DIR");
    if (!dir || varid < 0 || varid >= (int)g_nc.vars.size()) return;
    size_t count = 1;
    for (int d : g_nc.vars[varid].second) count *= g_nc.dims[d];
    const std::string path = std::string(dir) + "/" + g_nc.vars[varid].first + ".bin";
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return;
    std::fwrite(data, elem, count, f);
    std::fclose(f);
}
}  // namespace

extern "C" {
int nc_create(const char *, int, int *ncidp) {
    g_nc = NcState();
    *ncidp = 1;
    return NC_NOERR;
}
int nc_open(const char *, int, int *) { return NC_ENOTNC; }
int nc_close(int) { return NC_NOERR; }
int nc_enddef(int) { return NC_NOERR; }
int nc_def_dim(int, const char *, size_t len, int *idp) {
    *idp = (int)g_nc.dims.size();
    g_nc.dims.push_back(len);
    return NC_NOERR;
}
int nc_def_var(int, const char *name, nc_type, int ndims, const int *dimidsp, int *varidp) {
    *varidp = (int)g_nc.vars.size();
    g_nc.vars.emplace_back(name, std::vector<int>(dimidsp, dimidsp + ndims));
    return NC_NOERR;
}
int nc_put_att_text(int, int, const char *, size_t, const char *) { return NC_NOERR; }
int nc_put_var_double(int, int varid, const double *op) { nc_record(varid, op, sizeof(double)); return NC_NOERR; }
int nc_put_var_float(int, int varid, const float *op) { nc_record(varid, op, sizeof(float)); return NC_NOERR; }
int nc_put_var_int(int, int varid, const int *op) { nc_record(varid, op, sizeof(int)); return NC_NOERR; }
int nc_inq_varid(int, const char *, int *) { return NC_ENOTNC; }
int nc_get_var_double(int, int, double *) { return NC_ENOTNC; }
int nc_get_var_float(int, int, float *) { return NC_ENOTNC; }
int nc_get_var_int(int, int, int *) { return NC_ENOTNC; }
const char *nc_strerror(int) { return "netCDF is not available in the reference build"; }
}

// -------------------------------------------------------------- hypre ----
struct shim_ij_matrix {
    int lo = 0, hi = -1;
    std::vector<std::map<int, double>> rows;  // building
    std::vector<int> ptr, col;                 // assembled CSR
    std::vector<double> val;
    std::vector<double> ilu;                   // ILU(0) factors, same pattern
    std::vector<int> diag;
    bool assembled = false;
};
struct shim_ij_vector {
    int lo = 0, hi = -1;
    std::vector<double> v;
};
struct shim_solver {
    double tol = 1e-6;
    int maxit = 1000;
    double final_norm = 0;
    int iters = 0;
};

static int g_shim_total_iters = 0;

extern "C" int shim_hypre_total_iterations(void) { return g_shim_total_iters; }

static void csr_assemble(shim_ij_matrix *A) {
    int n = A->hi - A->lo + 1;
    A->ptr.assign(n + 1, 0);
    A->col.clear();
    A->val.clear();
    A->diag.assign(n, -1);
    for (int r = 0; r < n; r++) {
        for (auto &cv : A->rows[r]) {
            if (cv.first == r) A->diag[r] = (int)A->col.size();
            A->col.push_back(cv.first);
            A->val.push_back(cv.second);
        }
        A->ptr[r + 1] = (int)A->col.size();
        if (A->diag[r] < 0) {
            std::fprintf(stderr, "hypre stand-in: row %d has no diagonal entry\n", r + A->lo);
            std::abort();
        }
    }
    // ILU(0) on the same sparsity pattern (IKJ variant).
    A->ilu = A->val;
    std::vector<int> pos(n, -1);
    for (int i = 0; i < n; i++) {
        for (int q = A->ptr[i]; q < A->ptr[i + 1]; q++) pos[A->col[q]] = q;
        for (int q = A->ptr[i]; q < A->ptr[i + 1]; q++) {
            int k = A->col[q];
            if (k >= i) break;
            double lik = A->ilu[q] / A->ilu[A->diag[k]];
            A->ilu[q] = lik;
            for (int s = A->diag[k] + 1; s < A->ptr[k + 1]; s++) {
                int j = A->col[s];
                if (pos[j] >= 0) A->ilu[pos[j]] -= lik * A->ilu[s];
            }
        }
        for (int q = A->ptr[i]; q < A->ptr[i + 1]; q++) pos[A->col[q]] = -1;
    }
    A->rows.clear();
    A->rows.shrink_to_fit();
    A->assembled = true;
}

static void spmv(const shim_ij_matrix *A, const double *x, double *y) {
    int n = (int)A->diag.size();
    for (int r = 0; r < n; r++) {
        double s = 0;
        for (int q = A->ptr[r]; q < A->ptr[r + 1]; q++) s += A->val[q] * x[A->col[q]];
        y[r] = s;
    }
}

static void ilu_apply(const shim_ij_matrix *A, const double *r, double *z) {
    int n = (int)A->diag.size();
    for (int i = 0; i < n; i++) {
        double s = r[i];
        for (int q = A->ptr[i]; q < A->diag[i]; q++) s -= A->ilu[q] * z[A->col[q]];
        z[i] = s;
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = z[i];
        for (int q = A->diag[i] + 1; q < A->ptr[i + 1]; q++) s -= A->ilu[q] * z[A->col[q]];
        z[i] = s / A->ilu[A->diag[i]];
    }
}

static double dot(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
}

// Right-preconditioned BiCGSTAB; returns 0 on convergence, HYPRE_ERROR_CONV otherwise.
static int shim_bicgstab(shim_solver *S, shim_ij_matrix *A, shim_ij_vector *b, shim_ij_vector *x) {
    if (!A->assembled) csr_assemble(A);
    const int n = (int)A->diag.size();
    std::vector<double> r(n), r0(n), p(n), v(n), s(n), t(n), ph(n), sh(n);
    spmv(A, x->v.data(), r.data());
    for (int i = 0; i < n; i++) r[i] = b->v[i] - r[i];
    const double bnorm = std::sqrt(dot(b->v, b->v));
    S->iters = 0;
    if (bnorm == 0.0) {
        std::fill(x->v.begin(), x->v.end(), 0.0);
        S->final_norm = 0;
        return 0;
    }
    double rnorm = std::sqrt(dot(r, r));
    const int maxit = std::max(S->maxit, 20000);
    r0 = r;
    double rho = 1, alpha = 1, omega = 1;
    std::fill(p.begin(), p.end(), 0.0);
    std::fill(v.begin(), v.end(), 0.0);
    int it = 0;
    while (rnorm / bnorm >= S->tol && it < maxit) {
        it++;
        double rho1 = dot(r0, r);
        double beta = (rho1 / rho) * (alpha / omega);
        rho = rho1;
        for (int i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        ilu_apply(A, p.data(), ph.data());
        spmv(A, ph.data(), v.data());
        alpha = rho / dot(r0, v);
        for (int i = 0; i < n; i++) s[i] = r[i] - alpha * v[i];
        double snorm = std::sqrt(dot(s, s));
        if (snorm / bnorm < S->tol) {
            for (int i = 0; i < n; i++) x->v[i] += alpha * ph[i];
            r = s;
            rnorm = snorm;
            break;
        }
        ilu_apply(A, s.data(), sh.data());
        spmv(A, sh.data(), t.data());
        omega = dot(t, s) / dot(t, t);
        for (int i = 0; i < n; i++) {
            x->v[i] += alpha * ph[i] + omega * sh[i];
            r[i] = s[i] - omega * t[i];
        }
        rnorm = std::sqrt(dot(r, r));
    }
    // Report the true residual of the returned iterate.
    spmv(A, x->v.data(), t.data());
    double tr = 0;
    for (int i = 0; i < n; i++) tr += (b->v[i] - t[i]) * (b->v[i] - t[i]);
    S->final_norm = std::sqrt(tr) / bnorm;
    S->iters = it;
    g_shim_total_iters += it;
    return S->final_norm < S->tol ? 0 : HYPRE_ERROR_CONV;
}

extern "C" {
HYPRE_Int HYPRE_Init(void) { return 0; }
HYPRE_Int HYPRE_Finalize(void) { return 0; }
HYPRE_Int HYPRE_CheckError(HYPRE_Int ierr, HYPRE_Int code) { return ierr & code; }

HYPRE_Int HYPRE_IJMatrixCreate(MPI_Comm, HYPRE_BigInt ilo, HYPRE_BigInt ihi, HYPRE_BigInt, HYPRE_BigInt,
                               HYPRE_IJMatrix *m) {
    *m = new shim_ij_matrix;
    (*m)->lo = ilo;
    (*m)->hi = ihi;
    (*m)->rows.resize(ihi - ilo + 1);
    return 0;
}
HYPRE_Int HYPRE_IJMatrixSetObjectType(HYPRE_IJMatrix, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_IJMatrixInitialize(HYPRE_IJMatrix) { return 0; }
HYPRE_Int HYPRE_IJMatrixSetValues(HYPRE_IJMatrix m, HYPRE_Int nrows, HYPRE_Int *ncols, const HYPRE_BigInt *rows,
                                  const HYPRE_BigInt *cols, const HYPRE_Complex *values) {
    int off = 0;
    for (int r = 0; r < nrows; r++) {
        auto &row = m->rows.at(rows[r] - m->lo);
        row.clear();
        for (int c = 0; c < ncols[r]; c++) row[cols[off + c] - m->lo] = values[off + c];
        off += ncols[r];
    }
    return 0;
}
HYPRE_Int HYPRE_IJMatrixAssemble(HYPRE_IJMatrix m) { csr_assemble(m); return 0; }
HYPRE_Int HYPRE_IJMatrixGetObject(HYPRE_IJMatrix m, void **obj) { *obj = m; return 0; }
HYPRE_Int HYPRE_IJMatrixDestroy(HYPRE_IJMatrix m) { delete m; return 0; }

HYPRE_Int HYPRE_IJVectorCreate(MPI_Comm, HYPRE_BigInt lo, HYPRE_BigInt hi, HYPRE_IJVector *v) {
    *v = new shim_ij_vector;
    (*v)->lo = lo;
    (*v)->hi = hi;
    (*v)->v.assign(hi - lo + 1, 0.0);
    return 0;
}
HYPRE_Int HYPRE_IJVectorSetObjectType(HYPRE_IJVector, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_IJVectorInitialize(HYPRE_IJVector) { return 0; }
HYPRE_Int HYPRE_IJVectorSetValues(HYPRE_IJVector v, HYPRE_Int n, const HYPRE_BigInt *idx, const HYPRE_Complex *vals) {
    for (int i = 0; i < n; i++) v->v.at(idx[i] - v->lo) = vals[i];
    return 0;
}
HYPRE_Int HYPRE_IJVectorGetValues(HYPRE_IJVector v, HYPRE_Int n, const HYPRE_BigInt *idx, HYPRE_Complex *vals) {
    for (int i = 0; i < n; i++) vals[i] = v->v.at(idx[i] - v->lo);
    return 0;
}
HYPRE_Int HYPRE_IJVectorAssemble(HYPRE_IJVector) { return 0; }
HYPRE_Int HYPRE_IJVectorGetObject(HYPRE_IJVector v, void **obj) { *obj = v; return 0; }
HYPRE_Int HYPRE_IJVectorDestroy(HYPRE_IJVector v) { delete v; return 0; }

#define SHIM_SOLVER_COMMON(PFX)                                                                   \
    HYPRE_Int PFX##Create(MPI_Comm, HYPRE_Solver *s) { *s = new shim_solver; return 0; }          \
    HYPRE_Int PFX##Destroy(HYPRE_Solver s) { delete s; return 0; }                                \
    HYPRE_Int PFX##SetTol(HYPRE_Solver s, HYPRE_Real tol) { s->tol = tol; return 0; }             \
    HYPRE_Int PFX##SetMaxIter(HYPRE_Solver s, HYPRE_Int it) { s->maxit = it; return 0; }          \
    HYPRE_Int PFX##SetLogging(HYPRE_Solver, HYPRE_Int) { return 0; }                              \
    HYPRE_Int PFX##SetPrintLevel(HYPRE_Solver, HYPRE_Int) { return 0; }                           \
    HYPRE_Int PFX##SetPrecond(HYPRE_Solver, HYPRE_PtrToParSolverFcn, HYPRE_PtrToParSolverFcn,     \
                              HYPRE_Solver) { return 0; }                                         \
    HYPRE_Int PFX##Setup(HYPRE_Solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector, HYPRE_ParVector) {  \
        if (!A->assembled) csr_assemble(A);                                                       \
        return 0;                                                                                 \
    }                                                                                             \
    HYPRE_Int PFX##Solve(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x) { \
        return shim_bicgstab(s, A, b, x);                                                         \
    }                                                                                             \
    HYPRE_Int PFX##GetFinalRelativeResidualNorm(HYPRE_Solver s, HYPRE_Real *n) { *n = s->final_norm; return 0; }

SHIM_SOLVER_COMMON(HYPRE_ParCSRBiCGSTAB)
SHIM_SOLVER_COMMON(HYPRE_ParCSRPCG)
SHIM_SOLVER_COMMON(HYPRE_ParCSRGMRES)
HYPRE_Int HYPRE_ParCSRGMRESSetKDim(HYPRE_Solver, HYPRE_Int) { return 0; }

HYPRE_Int HYPRE_BiCGSTABSetMaxIter(HYPRE_Solver s, HYPRE_Int it) { s->maxit = it; return 0; }
HYPRE_Int HYPRE_BiCGSTABSetTol(HYPRE_Solver s, HYPRE_Real tol) { s->tol = tol; return 0; }
HYPRE_Int HYPRE_BiCGSTABSetLogging(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BiCGSTABSetPrintLevel(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BiCGSTABSetPrecond(HYPRE_Solver, HYPRE_PtrToSolverFcn, HYPRE_PtrToSolverFcn, HYPRE_Solver) { return 0; }

HYPRE_Int HYPRE_BoomerAMGCreate(HYPRE_Solver *s) { *s = new shim_solver; return 0; }
HYPRE_Int HYPRE_BoomerAMGDestroy(HYPRE_Solver s) { delete s; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetup(HYPRE_Solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector, HYPRE_ParVector) {
    if (!A->assembled) csr_assemble(A);
    return 0;
}
HYPRE_Int HYPRE_BoomerAMGSolve(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x) {
    return shim_bicgstab(s, A, b, x);
}
HYPRE_Int HYPRE_BoomerAMGGetFinalRelativeResidualNorm(HYPRE_Solver s, HYPRE_Real *n) { *n = s->final_norm; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetOldDefault(HYPRE_Solver) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetTol(HYPRE_Solver s, HYPRE_Real tol) { s->tol = tol; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetMaxIter(HYPRE_Solver s, HYPRE_Int it) { s->maxit = it; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetMaxRowSum(HYPRE_Solver, HYPRE_Real) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetCoarsenType(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetNonGalerkinTol(HYPRE_Solver, HYPRE_Real) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetLevelNonGalerkinTol(HYPRE_Solver, HYPRE_Real, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetAggNumLevels(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetNumSweeps(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetRelaxType(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetLogging(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetPrintLevel(HYPRE_Solver, HYPRE_Int) { return 0; }
}
