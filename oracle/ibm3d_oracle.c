/*
 * CPU oracle of the reference's 3D immersed-boundary fractional step.
 *
 * TEST INFRASTRUCTURE ONLY (see ibm3d_oracle.h): a plain-C restatement of
 * the reference algorithm, used as the parity checker and as the timed CPU
 * baseline.  Each routine cites the reference lines it restates.  The linear
 * solves follow hypre's BiCGSTAB as the reference configures it (x0 = 0,
 * ||r|| < tol ||b||, momentum unpreconditioned with 200 iterations at most,
 * pressure with up to 1000); the pressure preconditioner is a geometric
 * multigrid V-cycle standing in for BoomerAMG, which changes iteration
 * counts only.  Loops are OpenMP-parallel with static schedules and all
 * reductions add per-thread partials in thread order, so a run with a given
 * thread count is bitwise reproducible.
 *
 * Build: make -C oracle oracle  (gcc, -ffp-contract=off, -fopenmp).
 */
#include "ibm3d_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { BC_VEL = 0, BC_PRES = 1, BC_WALL = 2, BC_SLIP = 3, BC_SYM = 4, BC_PER = 5, BC_VELPER = 6 };
enum { FL = 1, GH = 2, SO = 3 };
enum { FN = 0, FE = 1, FS = 2, FW = 3, FD = 4, FU = 5 };

typedef struct {
    int nx, ny, nz;
    long n;
    int cx, cy, cz;
    double *tx, *ty, *tz, *gx, *gy, *gz, *diag, *r, *z;
} Level;

struct Oracle {
    int nx, ny, nz;
    long sx, sy, nc;
    double Re, dt, time;
    int iter;
    double *dx, *dy, *dz, *xc, *yc, *zc;
    double *kxW, *kxE, *kyS, *kyN, *kzD, *kzU;
    int bct[6];
    double bu[6][3], bp[6];
    double (*bcfn[6][4])(double, double, double, double);
    double (*ffn[3])(double, double, double, double);
    double xmin, xmax, ymin, ymax, zmin, zmax;
    double f[3], cs, tol, divtol;
    int singular, threads;
    int *flag;
    double *lvset, *coeffsum;
    double *u[3], *un[3], *us[3], *ut[3], *U[3], *Un[3], *Us[3];
    double *p, *pn, *pp, *N[3], *Np[3], *tau[6];
    /* ghost stencils, lexicographic */
    int ng;
    int *gcell;
    int (*gidx)[8][3];
    double (*gco)[8];
    int *gid;     /* padded index -> ghost id */
    /* krylov work */
    double *b, *x, *r, *r0, *pv, *v, *s, *t, *ph, *sh;
    /* multigrid */
    int nlev;
    Level lev[24];
    int per[3];
    int iters[4];
    double res[4], maxdiv;
    double *gtmp;
};

/* ------------------------------------------------------------ layout -- */
#define C1(a, i) ((a)[(i) + 2])
static inline long CI(const Oracle *o, int i, int j, int k) { return (long)(i + 2) * o->sx + (long)(j + 2) * o->sy + (k + 2); }
static inline long XI(const Oracle *o, int i, int j, int k) { return (long)i * o->sx + (long)(j + 2) * o->sy + (k + 2); }
static inline long YI(const Oracle *o, int i, int j, int k) {
    return (long)(i + 2) * (o->ny + 1) * (o->nz + 4) + (long)j * (o->nz + 4) + (k + 2);
}
static inline long ZI(const Oracle *o, int i, int j, int k) {
    return (long)(i + 2) * (o->ny + 4) * (o->nz + 1) + (long)(j + 2) * (o->nz + 1) + k;
}
#define C3(a, i, j, k) ((a)[CI(o, i, j, k)])
#define XS(a, i, j, k) ((a)[XI(o, i, j, k)])
#define YS(a, i, j, k) ((a)[YI(o, i, j, k)])
#define ZS(a, i, j, k) ((a)[ZI(o, i, j, k)])

static double *dal(long n) {
    double *p = (double *)calloc((size_t)n, sizeof(double));
    if (!p) {
        fprintf(stderr, "oracle: out of memory\n");
        exit(2);
    }
    return p;
}

static int isper(int t) { return t == BC_PER || t == BC_VELPER; }

/* Deterministic parallel sum of f(i) for i in [0, n). */
#define PSUM(result, n, expr)                                                   \
    do {                                                                        \
        int nt_ = omp_get_max_threads();                                        \
        double part_[256];                                                      \
        if (nt_ > 256) nt_ = 256;                                               \
        _Pragma("omp parallel num_threads(nt_)") {                               \
            int t_ = omp_get_thread_num(), T_ = omp_get_num_threads();          \
            long lo_ = (long)(n) * t_ / T_, hi_ = (long)(n) * (t_ + 1) / T_;    \
            double s_ = 0;                                                      \
            for (long q = lo_; q < hi_; q++) s_ += (expr);                      \
            part_[t_] = s_;                                                     \
            if (t_ == 0)                                                        \
                for (int z_ = T_; z_ < nt_; z_++) part_[z_] = 0;                \
        }                                                                       \
        double s2_ = 0;                                                         \
        for (int z_ = 0; z_ < nt_; z_++) s2_ += part_[z_];                      \
        (result) = s2_;                                                         \
    } while (0)

/* ------------------------------------------------------ ghost stencil -- */
static int upper_bound_(int len, const double *arr, double val) {
    int l = 0, h = len;
    while (l < h) {
        int mid = l + (h - l) / 2;
        if (val >= arr[mid]) l = mid + 1;
        else h = mid;
    }
    return l;
}

/* IBMSolver_ghost_interp (src/utils.c:111-171). */
static void ghost_interp(const Oracle *o, int i, int j, int k, int idx[8][3], double co[8]) {
    const double *lv = o->lvset;
    double nxv = (C3(lv, i + 1, j, k) - C3(lv, i - 1, j, k)) / (C1(o->xc, i + 1) - C1(o->xc, i - 1));
    double nyv = (C3(lv, i, j + 1, k) - C3(lv, i, j - 1, k)) / (C1(o->yc, j + 1) - C1(o->yc, j - 1));
    double nzv = (C3(lv, i, j, k + 1) - C3(lv, i, j, k - 1)) / (C1(o->zc, k + 1) - C1(o->zc, k - 1));
    double c = -2 * C3(lv, i, j, k);
    double mx = 1 * C1(o->xc, i) + c * nxv, my = 1 * C1(o->yc, j) + c * nyv, mz = 1 * C1(o->zc, k) + c * nzv;
    int im = upper_bound_(o->nx + 4, o->xc, mx) - 3;
    int jm = upper_bound_(o->ny + 4, o->yc, my) - 3;
    int km = upper_bound_(o->nz + 4, o->zc, mz) - 3;
    for (int l = 0; l < 8; l++) {
        idx[l][0] = im + !!(l & 4);
        idx[l][1] = jm + !!(l & 2);
        idx[l][2] = km + !!(l & 1);
    }
    double xl = C1(o->xc, im), xu = C1(o->xc, im + 1);
    double yl = C1(o->yc, jm), yu = C1(o->yc, jm + 1);
    double zl = C1(o->zc, km), zu = C1(o->zc, km + 1);
    double vol = (xu - xl) * (yu - yl) * (zu - zl);
    co[0] = (xu - mx) * (yu - my) * (zu - mz) / vol;
    co[1] = (xu - mx) * (yu - my) * (mz - zl) / vol;
    co[2] = (xu - mx) * (my - yl) * (zu - mz) / vol;
    co[3] = (xu - mx) * (my - yl) * (mz - zl) / vol;
    co[4] = (mx - xl) * (yu - my) * (zu - mz) / vol;
    co[5] = (mx - xl) * (yu - my) * (mz - zl) / vol;
    co[6] = (mx - xl) * (my - yl) * (zu - mz) / vol;
    co[7] = (mx - xl) * (my - yl) * (mz - zl) / vol;
}

/* Normalised ghost row: weights of non-solid, non-self entries and the
   self weight (src/ibm3d_setup.c:1653-1698, src/ibm3d_fracstep.c:1935-1962). */
static void ghost_row(const Oracle *o, int g, double w[8], int keep[8], double *wself) {
    double sum = 0;
    const int i = 0;
    (void)i;
    for (int l = 0; l < 8; l++) {
        const int *c = o->gidx[g][l];
        w[l] = C3(o->flag, c[0], c[1], c[2]) == SO ? 0 : o->gco[g][l];
        if (C3(o->flag, c[0], c[1], c[2]) != SO) sum += w[l];
    }
    *wself = 0;
    long P = o->gcell[g];
    for (int l = 0; l < 8; l++) {
        const int *c = o->gidx[g][l];
        w[l] /= sum;
        long q = CI(o, c[0], c[1], c[2]);
        if (q == P) {
            *wself += w[l];
            keep[l] = 0;
        } else {
            keep[l] = C3(o->flag, c[0], c[1], c[2]) != SO;
        }
    }
}

/* ---------------------------------------------------- STL + CPT (setup) -- */
typedef struct { double x, y, z; } V3;
static V3 vsub(V3 a, V3 b) { return (V3){a.x - b.x, a.y - b.y, a.z - b.z}; }
static double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V3 vcrs(V3 a, V3 b) { return (V3){a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static double vnorm(V3 v) { return sqrt(vdot(v, v)); }
static double vangle(V3 a, V3 b) {
    double la = vnorm(a), lb = vnorm(b);
    double c = vdot(a, b) / (la * lb);
    if (c < -1) c = -1;
    else if (c > 1) c = 1;
    return acos(c);
}
static V3 vnormalize(V3 v) {
    double l = vnorm(v);
    return (V3){v.x / l, v.y / l, v.z / l};
}
static V3 vlin(double a, V3 u, double b, V3 v) { return (V3){a * u.x + b * v.x, a * u.y + b * v.y, a * u.z + b * v.z}; }
static V3 vrot(V3 v, V3 axis, double ang) {
    V3 n = vnormalize(axis);
    double c = cos(ang), s = sin(ang);
    V3 r;
    r.x = (c + n.x * n.x * (1 - c)) * v.x + (n.x * n.y * (1 - c) - n.z * s) * v.y + (n.x * n.z * (1 - c) + n.y * s) * v.z;
    r.y = (n.x * n.y * (1 - c) + n.z * s) * v.x + (c + n.y * n.y * (1 - c)) * v.y + (n.y * n.z * (1 - c) - n.x * s) * v.z;
    r.z = (n.x * n.z * (1 - c) - n.y * s) * v.x + (n.y * n.z * (1 - c) + n.x * s) * v.y + (c + n.z * n.z * (1 - c)) * v.z;
    return r;
}

typedef struct {
    int nv, ne, nf;
    V3 *vc;
    int *vnf, **vfaces;
    int (*ev)[2], (*ef)[2];
    int (*fv)[3], (*fe)[3];
    V3 *fn;
} Poly;

/* Open-addressing map from a key of up to 3 doubles to an insertion index. */
typedef struct {
    long cap;
    double *keys;
    int *vals;
} HMap;
static uint64_t hbits(double d) {
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
}
static long hslot(HMap *m, const double *k, int nk) {
    uint64_t h = 1469598103934665603ULL;
    for (int q = 0; q < nk; q++) h = (h ^ hbits(k[q])) * 1099511628211ULL;
    long s = (long)(h % (uint64_t)m->cap);
    while (m->vals[s] >= 0) {
        int eq = 1;
        for (int q = 0; q < nk; q++) eq &= m->keys[s * 3 + q] == k[q];
        if (eq) return s;
        s = (s + 1) % m->cap;
    }
    return s;
}

/* Polyhedron_read_stl (src/geo3d.c:229-368): exact-equality vertex merge in
   first-seen order, unordered edges in first-seen order, vertex face rings. */
static Poly *read_stl(const char *path) {
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        fprintf(stderr, "oracle: cannot open %s\n", path);
        exit(2);
    }
    char hdr[80];
    uint32_t nf;
    if (fread(hdr, 1, 80, fp) != 80 || fread(&nf, 4, 1, fp) != 1) exit(2);
    Poly *P = (Poly *)calloc(1, sizeof(Poly));
    P->nf = (int)nf;
    P->fv = malloc(sizeof(int[3]) * nf);
    P->fe = malloc(sizeof(int[3]) * nf);
    P->fn = malloc(sizeof(V3) * nf);
    HMap vm = {4L * nf + 17, malloc(sizeof(double) * 3 * (4L * nf + 17)), malloc(sizeof(int) * (4L * nf + 17))};
    for (long q = 0; q < vm.cap; q++) vm.vals[q] = -1;
    P->vc = malloc(sizeof(V3) * 3 * nf);
    int *first = malloc(sizeof(int) * 3 * nf), *cnt = calloc(3 * nf, sizeof(int));
    for (uint32_t i = 0; i < nf; i++) {
        float rec[12];
        uint16_t attr;
        if (fread(rec, 4, 12, fp) != 12 || fread(&attr, 2, 1, fp) != 1) exit(2);
        P->fn[i] = (V3){rec[0], rec[1], rec[2]};
        for (int j = 0; j < 3; j++) {
            double key[3] = {rec[3 + 3 * j], rec[4 + 3 * j], rec[5 + 3 * j]};
            long s = hslot(&vm, key, 3);
            if (vm.vals[s] < 0) {
                vm.vals[s] = P->nv;
                memcpy(&vm.keys[s * 3], key, sizeof key);
                P->vc[P->nv] = (V3){key[0], key[1], key[2]};
                first[P->nv] = (int)i;
                P->nv++;
            }
            P->fv[i][j] = vm.vals[s];
            cnt[vm.vals[s]]++;
        }
    }
    fclose(fp);
    P->vnf = cnt;
    P->vfaces = malloc(sizeof(int *) * P->nv);
    for (int v = 0; v < P->nv; v++) {
        P->vfaces[v] = malloc(sizeof(int) * cnt[v]);
        for (int q = 0; q < cnt[v]; q++) P->vfaces[v][q] = -1;
        P->vfaces[v][0] = first[v];
    }
    free(first);
    HMap em = {6L * nf + 17, malloc(sizeof(double) * 3 * (6L * nf + 17)), malloc(sizeof(int) * (6L * nf + 17))};
    for (long q = 0; q < em.cap; q++) em.vals[q] = -1;
    P->ev = malloc(sizeof(int[2]) * 3 * nf);
    P->ef = malloc(sizeof(int[2]) * 3 * nf);
    for (uint32_t i = 0; i < nf; i++)
        for (int j = 0; j < 3; j++) {
            int a = P->fv[i][j], b = P->fv[i][(j + 1) % 3];
            double key[2] = {a < b ? a : b, a < b ? b : a};
            long s = hslot(&em, key, 2);
            if (em.vals[s] < 0) {
                em.vals[s] = P->ne;
                em.keys[s * 3] = key[0];
                em.keys[s * 3 + 1] = key[1];
                P->ev[P->ne][0] = a;
                P->ev[P->ne][1] = b;
                P->ef[P->ne][0] = (int)i;
                P->ef[P->ne][1] = -1;
                P->ne++;
            } else {
                P->ef[em.vals[s]][1] = (int)i;
            }
            P->fe[i][j] = em.vals[s];
        }
    free(vm.keys); free(vm.vals); free(em.keys); free(em.vals);
    for (int v = 0; v < P->nv; v++) {
        int cur = P->vfaces[v][0];
        for (int j = 1; j < P->vnf[v]; j++) {
            int e;
            if (P->fv[cur][0] == v) e = P->fe[cur][2];
            else if (P->fv[cur][1] == v) e = P->fe[cur][0];
            else e = P->fe[cur][1];
            cur = P->ef[e][0] == cur ? P->ef[e][1] : P->ef[e][0];
            if (cur < 0) {
                fprintf(stderr, "oracle: polyhedron is not closed\n");
                exit(2);
            }
            P->vfaces[v][j] = cur;
        }
    }
    return P;
}

static void free_poly(Poly *P) {
    for (int v = 0; v < P->nv; v++) free(P->vfaces[v]);
    free(P->vfaces); free(P->vnf); free(P->vc); free(P->ev); free(P->ef); free(P->fv); free(P->fe); free(P->fn);
    free(P);
}

typedef struct { double a, b, c, d; } Plane;
static Plane plane3(V3 a, V3 b, V3 c) {
    V3 n = vcrs(vsub(b, a), vsub(c, a));
    return (Plane){n.x, n.y, n.z, -vdot(n, a)};
}
static int lower_bound_(int len, const double *arr, double val) {
    int l = 0, h = len;
    while (l < h) {
        int mid = l + (h - l) / 2;
        if (val <= arr[mid]) h = mid;
        else l = mid + 1;
    }
    return l;
}

typedef struct {
    int nx, ny, nz;
    const double *x, *y, *z;
    double *f;
} CptGrid;
#define F3(G, i, j, k) ((G)->f[((long)(i) * (G)->ny + (j)) * (G)->nz + (k)])

static void box_of(const CptGrid *G, const V3 *p, int np, int b[6]) {
    double mx[3] = {-INFINITY, -INFINITY, -INFINITY}, mn[3] = {INFINITY, INFINITY, INFINITY};
    for (int q = 0; q < np; q++) {
        double c[3] = {p[q].x, p[q].y, p[q].z};
        for (int d = 0; d < 3; d++) {
            mx[d] = mx[d] > c[d] ? mx[d] : c[d];
            mn[d] = mn[d] < c[d] ? mn[d] : c[d];
        }
    }
    b[0] = lower_bound_(G->nx, G->x, mn[0]); b[1] = upper_bound_(G->nx, G->x, mx[0]);
    b[2] = lower_bound_(G->ny, G->y, mn[1]); b[3] = upper_bound_(G->ny, G->y, mx[1]);
    b[4] = lower_bound_(G->nz, G->z, mn[2]); b[5] = upper_bound_(G->nz, G->z, mx[2]);
}

static void update_f(CptGrid *G, int i, int j, int k, double dist, int sgn) {
    double *f = &F3(G, i, j, k);
    if (isnan(*f) || dist < fabs(*f)) *f = sgn * dist;
}

/* FaceExtrusion_cpt (src/geo3d.c:871-938). */
static void face_cpt(CptGrid *G, const V3 p[6], int sgn, int ilo, int ihi) {
    int b[6];
    box_of(G, p, 6, b);
    if (b[0] < ilo) b[0] = ilo;
    if (b[1] > ihi) b[1] = ihi;
    Plane pl[5] = {plane3(p[0], p[2], p[1]), plane3(p[3], p[4], p[5]), plane3(p[0], p[1], p[4]),
                   plane3(p[1], p[2], p[5]), plane3(p[0], p[3], p[5])};
    double nn = vnorm((V3){pl[0].a, pl[0].b, pl[0].c});
    for (int i = b[0]; i < b[1]; i++)
        for (int j = b[2]; j < b[3]; j++)
            for (int k = b[4]; k < b[5]; k++) {
                V3 c = {G->x[i], G->y[j], G->z[k]};
                int in = 1;
                for (int l = 0; l < 5; l++)
                    if (pl[l].a * c.x + pl[l].b * c.y + pl[l].c * c.z + pl[l].d > 1e-12) in = 0;
                if (in) update_f(G, i, j, k, fabs(pl[0].a * c.x + pl[0].b * c.y + pl[0].c * c.z + pl[0].d) / nn, sgn);
            }
}

/* EdgeExtrusion_cpt (src/geo3d.c:811-869). */
static void edge_cpt(CptGrid *G, const V3 p[6], int sgn, int ilo, int ihi) {
    int b[6];
    box_of(G, p, 6, b);
    if (b[0] < ilo) b[0] = ilo;
    if (b[1] > ihi) b[1] = ihi;
    Plane pl[5] = {plane3(p[0], p[4], p[2]), plane3(p[1], p[3], p[5]), plane3(p[0], p[2], p[3]),
                   plane3(p[2], p[4], p[5]), plane3(p[0], p[1], p[5])};
    V3 ab = vsub(p[1], p[0]);
    for (int i = b[0]; i < b[1]; i++)
        for (int j = b[2]; j < b[3]; j++)
            for (int k = b[4]; k < b[5]; k++) {
                V3 c = {G->x[i], G->y[j], G->z[k]};
                int in = 1;
                for (int l = 0; l < 5; l++)
                    if (pl[l].a * c.x + pl[l].b * c.y + pl[l].c * c.z + pl[l].d > 1e-12) in = 0;
                if (!in) continue;
                V3 av = vsub(c, p[0]);
                double t = vdot(ab, av) / vdot(ab, ab);
                V3 h = vlin(1 - t, p[0], t, p[1]);
                update_f(G, i, j, k, vnorm(vsub(c, h)), sgn);
            }
}

/* VertexExtrusion_cpt (src/geo3d.c:784-809).  The reference scans the box
   vertex +- radius; points outside the cone's own bounding box (widened by
   a margin far above rounding) fail its angle test, so the scan is limited
   to that box without changing any result.  i is restricted to [ilo, ihi). */
static void vertex_cpt(CptGrid *G, V3 v, V3 axis, double ang, double rad, int sgn, int ilo, int ihi) {
    int b[6] = {lower_bound_(G->nx, G->x, v.x - rad), upper_bound_(G->nx, G->x, v.x + rad),
                lower_bound_(G->ny, G->y, v.y - rad), upper_bound_(G->ny, G->y, v.y + rad),
                lower_bound_(G->nz, G->z, v.z - rad), upper_bound_(G->nz, G->z, v.z + rad)};
    const double la = vnorm(axis), comp[3] = {axis.x / la, axis.y / la, axis.z / la}, vc[3] = {v.x, v.y, v.z};
    const double *ga[3] = {G->x, G->y, G->z};
    const int gn[3] = {G->nx, G->ny, G->nz};
    for (int d = 0; d < 3; d++) {
        double c = comp[d] < -1 ? -1 : comp[d] > 1 ? 1 : comp[d];
        double al = acos(c), th = ang + 1e-6;
        double hi = al - th <= 0 ? 1.0 : cos(al - th), lo = al + th >= 3.141592653589793 ? -1.0 : cos(al + th);
        double m = 1e-6 * (1 + rad);
        double bl = vc[d] + rad * (lo < 0 ? lo : 0) - m, bh = vc[d] + rad * (hi > 0 ? hi : 0) + m;
        int tl = lower_bound_(gn[d], ga[d], bl), th2 = upper_bound_(gn[d], ga[d], bh);
        if (tl > b[2 * d]) b[2 * d] = tl;
        if (th2 < b[2 * d + 1]) b[2 * d + 1] = th2;
    }
    if (b[0] < ilo) b[0] = ilo;
    if (b[1] > ihi) b[1] = ihi;
    for (int i = b[0]; i < b[1]; i++)
        for (int j = b[2]; j < b[3]; j++)
            for (int k = b[4]; k < b[5]; k++) {
                V3 d = vsub((V3){G->x[i], G->y[j], G->z[k]}, v);
                double dist = vnorm(d);
                if (vangle(axis, d) <= ang + 1e-12 && dist <= rad + 1e-12) update_f(G, i, j, k, dist, sgn);
            }
}

/* Polyhedron_cpt (src/geo3d.c:436-704). */
static void cpt(const Poly *P, CptGrid *G, double maxd) {
    const double PI = 3.141592653589793;
    long n = (long)G->nx * G->ny * G->nz;
    for (long q = 0; q < n; q++) G->f[q] = NAN;
    /* Every thread replays the whole extrusion sequence on its own slab of
       i, so each grid point sees the reference's update order. */
#pragma omp parallel
    {
    const int T = omp_get_num_threads(), tid = omp_get_thread_num();
    const int ilo = (int)((long)G->nx * tid / T), ihi = (int)((long)G->nx * (tid + 1) / T);
    for (int i = 0; i < P->nf; i++) {
        V3 p[6];
        for (int j = 0; j < 3; j++) {
            p[j] = P->vc[P->fv[i][j]];
            p[j + 3] = vlin(1, p[j], maxd, P->fn[i]);
        }
        face_cpt(G, p, 1, ilo, ihi);
        for (int j = 0; j < 3; j++) {
            p[j] = P->vc[P->fv[i][(3 - j) % 3]];
            p[j + 3] = vlin(1, p[j], -maxd, P->fn[i]);
        }
        face_cpt(G, p, -1, ilo, ihi);
    }
    for (int i = 0; i < P->ne; i++) {
        V3 p[6];
        p[0] = P->vc[P->ev[i][0]];
        p[1] = P->vc[P->ev[i][1]];
        V3 v = vsub(p[1], p[0]), nl = P->fn[P->ef[i][0]], nr = P->fn[P->ef[i][1]];
        int sgn = vdot(vcrs(v, nl), nr) >= 0 ? 1 : -1;
        double ang = vangle(nl, nr), s = sgn == 1 ? maxd : -maxd;
        V3 wl[3], wr[3];
        int nw;
        if (ang <= PI / 3) {
            nw = 1;
            wl[0] = sgn == 1 ? nl : nr;
            wr[0] = sgn == 1 ? nr : nl;
        } else if (ang <= 2 * PI / 3) {
            V3 nm = vrot(nl, v, ang / 2);
            nw = 2;
            if (sgn == 1) { wl[0] = nl; wr[0] = nm; wl[1] = nm; wr[1] = nr; }
            else { wl[0] = nr; wr[0] = nm; wl[1] = nm; wr[1] = nl; }
        } else {
            nw = 3;
            if (sgn == 1) {
                V3 n1 = vrot(nl, v, ang / 3), n2 = vrot(nl, v, 2 * ang / 3);
                wl[0] = nl; wr[0] = n1; wl[1] = n1; wr[1] = n2; wl[2] = n2; wr[2] = nr;
            } else {
                V3 n1 = vrot(nl, v, -ang / 3), n2 = vrot(nl, v, -2 * ang / 3);
                wl[0] = nr; wr[0] = n2; wl[1] = n2; wr[1] = n1; wl[2] = n1; wr[2] = nl;
            }
        }
        for (int w = 0; w < nw; w++) {
            p[2] = vlin(1, p[0], s, wl[w]);
            p[3] = vlin(1, p[1], s, wl[w]);
            p[4] = vlin(1, p[0], s, wr[w]);
            p[5] = vlin(1, p[1], s, wr[w]);
            edge_cpt(G, p, sgn, ilo, ihi);
        }
    }
    for (int i = 0; i < P->nv; i++) {
        V3 vx = P->vc[i], axis = {0, 0, 0};
        int *adj = malloc(sizeof(int) * P->vnf[i]);
        double adj_angle = 0;
        for (int j = 0; j < P->vnf[i]; j++) {
            int f = P->vfaces[i][j];
            adj[j] = i;
            for (int k = 0; k < 3; k++)
                if (P->fv[f][k] == i) {
                    adj_angle = vangle(vsub(P->vc[P->fv[f][(k + 1) % 3]], vx), vsub(P->vc[P->fv[f][(k + 2) % 3]], vx));
                    adj[j] = P->fv[f][(k + 2) % 3];
                }
            axis = vlin(1, axis, adj_angle, P->fn[f]);
        }
        axis = vnormalize(axis);
        double cone = 0;
        for (int j = 0; j < P->vnf[i]; j++) {
            V3 an = P->fn[P->vfaces[i][j]];
            if (vdot(axis, an) > 0) {
                double a = vangle(axis, an);
                cone = cone > a ? cone : a;
            }
        }
        int convex = 1, concave = 1;
        for (int j = 0; j < P->vnf[i]; j++) {
            double d = vdot(vsub(P->vc[adj[j]], vx), axis);
            if (d > 0) convex = 0;
            if (d < 0) concave = 0;
        }
        free(adj);
        if (!concave) vertex_cpt(G, vx, axis, cone, maxd, 1, ilo, ihi);
        if (!convex) vertex_cpt(G, vx, (V3){-axis.x, -axis.y, -axis.z}, cone, maxd, -1, ilo, ihi);
    }
    }
    /* Fill (src/geo3d.c:643-703). */
    for (int i = 0; i < G->nx; i++)
        for (int j = 0; j < G->ny; j++) {
            for (int k = 1; k < G->nz; k++) {
                double *f = &F3(G, i, j, k), pv = F3(G, i, j, k - 1);
                if (isnan(*f) && pv < 0) *f = -maxd;
                else if (isnan(*f) && pv > 0) *f = maxd;
            }
            for (int k = G->nz - 2; k >= 0; k--) {
                double *f = &F3(G, i, j, k), nv = F3(G, i, j, k + 1);
                if (isnan(*f) && nv < 0) *f = -maxd;
                else if (isnan(*f) && nv > 0) *f = maxd;
            }
        }
    for (int i = 0; i < G->nx; i++)
        for (int k = 0; k < G->nz; k++) {
            for (int j = 1; j < G->ny; j++) {
                double *f = &F3(G, i, j, k), pv = F3(G, i, j - 1, k);
                if (isnan(*f) && pv < 0) *f = -maxd;
                else if (isnan(*f) && pv > 0) *f = maxd;
            }
            for (int j = G->ny - 2; j >= 0; j--) {
                double *f = &F3(G, i, j, k), nv = F3(G, i, j + 1, k);
                if (isnan(*f) && nv < 0) *f = -maxd;
                else if (isnan(*f) && nv > 0) *f = maxd;
            }
        }
    for (int j = 0; j < G->ny; j++)
        for (int k = 0; k < G->nz; k++) {
            for (int i = 1; i < G->nx; i++) {
                double *f = &F3(G, i, j, k), pv = F3(G, i - 1, j, k);
                if (isnan(*f) && pv < 0) *f = -maxd;
                else if (isnan(*f) && pv > 0) *f = maxd;
            }
            for (int i = G->nx - 2; i >= 0; i--) {
                double *f = &F3(G, i, j, k), nv = F3(G, i + 1, j, k);
                if (isnan(*f) && nv < 0) *f = -maxd;
                else if (isnan(*f) && nv > 0) *f = maxd;
            }
        }
}

/* ----------------------------------------------------------- operators -- */
/* Owner face of an outer cell, as the reference's matrix loops split the
   outer shell (src/ibm3d_setup.c:1723-2903); -1 for interior cells. */
static int owner(const Oracle *o, int i, int j, int k, int *L) {
    if (k < 0) { *L = -k; return FD; }
    if (k >= o->nz) { *L = k - o->nz + 1; return FU; }
    if (j < 0) { *L = -j; return FS; }
    if (j >= o->ny) { *L = j - o->ny + 1; return FN; }
    if (i < 0) { *L = -i; return FW; }
    if (i >= o->nx) { *L = i - o->nx + 1; return FE; }
    *L = 0;
    return -1;
}

static int wrap(int i, int n) { return i < 0 ? i + n : i >= n ? i - n : i; }

/* Boundary value q (0-2: u1-u3, 3: p) of face f on the outer line through
   padded cell (i, j, k) at time t: the constant, or the VAL_FUNC callback
   at the face centre of that line, as bc_val_u / bc_val_p evaluate it
   (src/ibm3d_fracstep.c:2001-2035). */
static double bcval(const Oracle *o, int f, int q, double t, int i, int j, int k) {
    if (!o->bcfn[f][q]) return q < 3 ? o->bu[f][q] : o->bp[f];
    double x = C1(o->xc, i), y = C1(o->yc, j), z = C1(o->zc, k);
    if (f == FW) x = o->xmin; else if (f == FE) x = o->xmax;
    else if (f == FS) y = o->ymin; else if (f == FN) y = o->ymax;
    else if (f == FD) z = o->zmin; else z = o->zmax;
    return o->bcfn[f][q](t, x, y, z);
}

/* Row of A_u{type} (type 1..3) or A_p (type 4) applied to x at padded
   (i, j, k); restates create_matrix (src/ibm3d_setup.c:1566-2908). */
static double row(const Oracle *o, int type, const double *x, int i, int j, int k) {
    int L;
    const int f = owner(o, i, j, k, &L);
    const long P = CI(o, i, j, k);
    if (f >= 0) {
        const int axis = (f == FE || f == FW) ? 0 : (f == FN || f == FS) ? 1 : 2;
        const int low = f == FW || f == FS || f == FD;
        const double *d = axis == 0 ? o->dx : axis == 1 ? o->dy : o->dz;
        const double *c = axis == 0 ? o->xc : axis == 1 ? o->yc : o->zc;
        const int N = axis == 0 ? o->nx : axis == 1 ? o->ny : o->nz;
        const long s = axis == 0 ? o->sx : axis == 1 ? o->sy : 1;
        const long in = low ? s : -s;
        const long m = P + (2 * L - 1) * in;
        const int t = o->bct[f];
        int kind; /* 0 Dirichlet interp, 1 Neumann, 2 periodic, 3 extrapolation */
        if (type != 4) {
            if (t == BC_VEL) kind = 0;
            else if (t == BC_PRES) kind = 3;
            else if (t == BC_SLIP) kind = type == axis + 1 ? 0 : 1;
            else kind = 2;
        } else {
            if (t == BC_VEL || t == BC_SLIP) kind = 1;
            else if (t == BC_PRES || t == BC_VELPER) kind = 0;
            else kind = 2;
        }
        double a, b;
        switch (kind) {
        case 0:
            if (low) {
                if (L == 1) { a = C1(d, -1) / 2; b = C1(d, 0) / 2; }
                else { a = C1(d, -2) / 2 + C1(d, -1); b = C1(d, 0) + C1(d, 1) / 2; }
                return b / (a + b) * x[P] + a / (a + b) * x[m];
            }
            if (L == 1) { a = C1(d, N - 1) / 2; b = C1(d, N) / 2; }
            else { a = C1(d, N - 2) / 2 + C1(d, N - 1); b = C1(d, N) + C1(d, N + 1) / 2; }
            return a / (a + b) * x[P] + b / (a + b) * x[m];
        case 1: return x[P] - x[m];
        case 2: return x[P] - x[CI(o, wrap(i, o->nx), wrap(j, o->ny), wrap(k, o->nz))];
        default:
            if (low) {
                if (L == 2) { a = C1(c, -1) - C1(c, -2); b = C1(c, 0) - C1(c, -1); }
                else { a = C1(c, 0) - C1(c, -1); b = C1(c, 1) - C1(c, 0); }
                return b / (a + b) * x[P] - x[P + in] + a / (a + b) * x[P + 2 * in];
            }
            if (L == 1) { a = C1(c, N - 1) - C1(c, N - 2); b = C1(c, N) - C1(c, N - 1); }
            else { a = C1(c, N) - C1(c, N - 1); b = C1(c, N + 1) - C1(c, N); }
            return a / (a + b) * x[P] - x[P + in] + b / (a + b) * x[P + 2 * in];
        }
    }
    if (type == 4 && o->singular && i == 0 && j == 0 && k == 0) return x[P];
    const int fl = o->flag[P];
    if (fl == FL) {
        double v1 = -C1(o->kyN, j), v2 = -C1(o->kxE, i), v3 = -C1(o->kyS, j);
        double v4 = -C1(o->kxW, i), v5 = -C1(o->kzD, k), v6 = -C1(o->kzU, k);
        double v0 = type != 4 ? 1 - v1 - v2 - v3 - v4 - v5 - v6 : -v1 - v2 - v3 - v4 - v5 - v6;
        if (type == 4) {
            v1 /= v0; v2 /= v0; v3 /= v0; v4 /= v0; v5 /= v0; v6 /= v0;
            v0 = 1;
        }
        return v0 * x[P] + v1 * x[P + o->sy] + v2 * x[P + o->sx] + v3 * x[P - o->sy] + v4 * x[P - o->sx] +
               v5 * x[P - 1] + v6 * x[P + 1];
    }
    if (fl == GH) {
        const int g = o->gid[P];
        double w[8], ws;
        int keep[8];
        ghost_row(o, g, w, keep, &ws);
        double y = (type != 4 ? 1 + ws : 1 - ws) * x[P];
        for (int l = 0; l < 8; l++)
            if (keep[l]) y += (type != 4 ? w[l] : -w[l]) * x[CI(o, o->gidx[g][l][0], o->gidx[g][l][1], o->gidx[g][l][2])];
        return y;
    }
    return x[P];
}

static void apply(const Oracle *o, int type, const double *x, double *y) {
#pragma omp parallel for schedule(static)
    for (int i = -2; i < o->nx + 2; i++)
        for (int j = -2; j < o->ny + 2; j++)
            for (int k = -2; k < o->nz + 2; k++) y[CI(o, i, j, k)] = row(o, type, x, i, j, k);
}

/* ------------------------------------------------------------ multigrid -- */
/* Pressure preconditioner: exact fine rows smoothed by colour Gauss-Seidel,
   masked conductance Laplacian on coarser levels, piecewise-constant
   transfers (the GPU library's design, restated serially by colour). */
static int color_of(int i, int j, int k, int nx, int ny, int nz, const int *per) {
    int seam = (per[0] && (nx & 1) && nx > 1 && i == nx - 1) || (per[1] && (ny & 1) && ny > 1 && j == ny - 1) ||
               (per[2] && (nz & 1) && nz > 1 && k == nz - 1);
    return ((i + j + k) & 1) + (seam ? 2 : 0);
}

static int active0(const Oracle *o, int i, int j, int k) {
    return C3(o->flag, i, j, k) == FL && !(o->singular && i == 0 && j == 0 && k == 0);
}

static void mg_setup(Oracle *o) {
    o->per[0] = o->bct[FW] == BC_PER;
    o->per[1] = o->bct[FS] == BC_PER;
    o->per[2] = o->bct[FD] == BC_PER;
    int nx = o->nx, ny = o->ny, nz = o->nz;
    o->nlev = 0;
    while (o->nlev < 24) {
        int cx = nx >= 2, cy = ny >= 2, cz = nz >= 2;
        if (!cx && !cy && !cz) break;
        if ((long)nx * ny * nz <= 64 && o->nlev > 0) break;
        Level *L = &o->lev[o->nlev];
        L->cx = cx; L->cy = cy; L->cz = cz;
        L->nx = cx ? (nx + 1) / 2 : nx;
        L->ny = cy ? (ny + 1) / 2 : ny;
        L->nz = cz ? (nz + 1) / 2 : nz;
        L->n = (long)L->nx * L->ny * L->nz;
        L->tx = dal(L->n); L->ty = dal(L->n); L->tz = dal(L->n);
        L->gx = dal(L->n); L->gy = dal(L->n); L->gz = dal(L->n);
        L->diag = dal(L->n); L->r = dal(L->n); L->z = dal(L->n);
        const double fx = cx ? 0.5 : 1.0, fy = cy ? 0.5 : 1.0, fz = cz ? 0.5 : 1.0;
        for (int I = 0; I < L->nx; I++)
            for (int J = 0; J < L->ny; J++)
                for (int K = 0; K < L->nz; K++) {
                    long q = ((long)I * L->ny + J) * L->nz + K;
                    int i0 = cx ? 2 * I : I, i1 = cx ? (2 * I + 1 < nx ? 2 * I + 1 : nx - 1) : I;
                    int j0 = cy ? 2 * J : J, j1 = cy ? (2 * J + 1 < ny ? 2 * J + 1 : ny - 1) : J;
                    int k0 = cz ? 2 * K : K, k1 = cz ? (2 * K + 1 < nz ? 2 * K + 1 : nz - 1) : K;
                    double tx = 0, ty = 0, tz = 0, gx = 0, gy = 0, gz = 0;
                    for (int i = i0; i <= i1; i++)
                        for (int j = j0; j <= j1; j++)
                            for (int k = k0; k <= k1; k++) {
                                if (o->nlev == 0) {
                                    if (!active0(o, i, j, k)) continue;
                                    double v = C1(o->dx, i) * C1(o->dy, j) * C1(o->dz, k);
                                    if (i == i0) {
                                        if (i > 0) { if (active0(o, i - 1, j, k)) tx += v * C1(o->kxW, i); }
                                        else if (o->per[0] && o->nx > 1 && active0(o, o->nx - 1, j, k)) tx += v * C1(o->kxW, 0);
                                    }
                                    if (j == j0) {
                                        if (j > 0) { if (active0(o, i, j - 1, k)) ty += v * C1(o->kyS, j); }
                                        else if (o->per[1] && o->ny > 1 && active0(o, i, o->ny - 1, k)) ty += v * C1(o->kyS, 0);
                                    }
                                    if (k == k0) {
                                        if (k > 0) { if (active0(o, i, j, k - 1)) tz += v * C1(o->kzD, k); }
                                        else if (o->per[2] && o->nz > 1 && active0(o, i, j, o->nz - 1)) tz += v * C1(o->kzD, 0);
                                    }
                                    /* Pressure-Dirichlet faces folded into the diagonal. */
#define DIRF(t) ((t) == BC_PRES || (t) == BC_VELPER)
                                    if (i == 0 && DIRF(o->bct[FW])) gx += v * C1(o->kxW, 0) * (1 + (C1(o->dx, -1) / 2) / (C1(o->dx, 0) / 2));
                                    if (i == o->nx - 1 && DIRF(o->bct[FE])) gx += v * C1(o->kxE, o->nx - 1) * (1 + (C1(o->dx, o->nx) / 2) / (C1(o->dx, o->nx - 1) / 2));
                                    if (j == 0 && DIRF(o->bct[FS])) gy += v * C1(o->kyS, 0) * (1 + (C1(o->dy, -1) / 2) / (C1(o->dy, 0) / 2));
                                    if (j == o->ny - 1 && DIRF(o->bct[FN])) gy += v * C1(o->kyN, o->ny - 1) * (1 + (C1(o->dy, o->ny) / 2) / (C1(o->dy, o->ny - 1) / 2));
                                    if (k == 0 && DIRF(o->bct[FD])) gz += v * C1(o->kzD, 0) * (1 + (C1(o->dz, -1) / 2) / (C1(o->dz, 0) / 2));
                                    if (k == o->nz - 1 && DIRF(o->bct[FU])) gz += v * C1(o->kzU, o->nz - 1) * (1 + (C1(o->dz, o->nz) / 2) / (C1(o->dz, o->nz - 1) / 2));
                                } else {
                                    Level *F = &o->lev[o->nlev - 1];
                                    long fq = ((long)i * F->ny + j) * F->nz + k;
                                    if (i == i0) tx += F->tx[fq];
                                    if (j == j0) ty += F->ty[fq];
                                    if (k == k0) tz += F->tz[fq];
                                    gx += F->gx[fq];
                                    gy += F->gy[fq];
                                    gz += F->gz[fq];
                                }
                            }
                    L->tx[q] = (I == 0 && L->nx == 1) ? 0 : fx * tx;
                    L->ty[q] = (J == 0 && L->ny == 1) ? 0 : fy * ty;
                    L->tz[q] = (K == 0 && L->nz == 1) ? 0 : fz * tz;
                    L->gx[q] = fx * gx;
                    L->gy[q] = fy * gy;
                    L->gz[q] = fz * gz;
                }
        o->nlev++;
        nx = L->nx; ny = L->ny; nz = L->nz;
        if (L->n <= 64) break;
    }
    for (int l = 0; l < o->nlev; l++) {
        Level *L = &o->lev[l];
        for (int I = 0; I < L->nx; I++)
            for (int J = 0; J < L->ny; J++)
                for (int K = 0; K < L->nz; K++) {
                    long q = ((long)I * L->ny + J) * L->nz + K, sy = L->nz, sx = (long)L->ny * L->nz;
                    double d = L->gx[q] + L->gy[q] + L->gz[q];
                    if (I > 0) d += L->tx[q]; else if (o->per[0] && L->nx > 1) d += L->tx[q];
                    if (I < L->nx - 1) d += L->tx[q + sx]; else if (o->per[0] && L->nx > 1) d += L->tx[q - (long)I * sx];
                    if (J > 0) d += L->ty[q]; else if (o->per[1] && L->ny > 1) d += L->ty[q];
                    if (J < L->ny - 1) d += L->ty[q + sy]; else if (o->per[1] && L->ny > 1) d += L->ty[q - (long)J * sy];
                    if (K > 0) d += L->tz[q]; else if (o->per[2] && L->nz > 1) d += L->tz[q];
                    if (K < L->nz - 1) d += L->tz[q + 1]; else if (o->per[2] && L->nz > 1) d += L->tz[q - K];
                    L->diag[q] = d;
                }
    }
}

static double coarse_off(const Oracle *o, const Level *L, int I, int J, int K) {
    long q = ((long)I * L->ny + J) * L->nz + K, sy = L->nz, sx = (long)L->ny * L->nz;
    double s = 0;
    if (I > 0) s += L->tx[q] * L->z[q - sx]; else if (o->per[0] && L->nx > 1) s += L->tx[q] * L->z[q + (long)(L->nx - 1) * sx];
    if (I < L->nx - 1) s += L->tx[q + sx] * L->z[q + sx]; else if (o->per[0] && L->nx > 1) s += L->tx[q - (long)I * sx] * L->z[q - (long)I * sx];
    if (J > 0) s += L->ty[q] * L->z[q - sy]; else if (o->per[1] && L->ny > 1) s += L->ty[q] * L->z[q + (long)(L->ny - 1) * sy];
    if (J < L->ny - 1) s += L->ty[q + sy] * L->z[q + sy]; else if (o->per[1] && L->ny > 1) s += L->ty[q - (long)J * sy] * L->z[q - (long)J * sy];
    if (K > 0) s += L->tz[q] * L->z[q - 1]; else if (o->per[2] && L->nz > 1) s += L->tz[q] * L->z[q + L->nz - 1];
    if (K < L->nz - 1) s += L->tz[q + 1] * L->z[q + 1]; else if (o->per[2] && L->nz > 1) s += L->tz[q - K] * L->z[q - K];
    return s;
}

static void coarse_smooth(const Oracle *o, Level *L, int sweeps) {
    for (int s = 0; s < sweeps; s++)
        for (int col = 0; col < 4; col++) {
#pragma omp parallel for schedule(static)
            for (int I = 0; I < L->nx; I++)
                for (int J = 0; J < L->ny; J++)
                    for (int K = 0; K < L->nz; K++) {
                        if (color_of(I, J, K, L->nx, L->ny, L->nz, o->per) != col) continue;
                        long q = ((long)I * L->ny + J) * L->nz + K;
                        L->z[q] = L->diag[q] == 0 ? 0 : (L->r[q] + coarse_off(o, L, I, J, K)) / L->diag[q];
                    }
        }
}

static void coarse_restrict(const Oracle *o, Level *F, Level *C) {
#pragma omp parallel for schedule(static)
    for (int I = 0; I < C->nx; I++)
        for (int J = 0; J < C->ny; J++)
            for (int K = 0; K < C->nz; K++) {
                int i0 = C->cx ? 2 * I : I, i1 = C->cx ? (2 * I + 1 < F->nx ? 2 * I + 1 : F->nx - 1) : I;
                int j0 = C->cy ? 2 * J : J, j1 = C->cy ? (2 * J + 1 < F->ny ? 2 * J + 1 : F->ny - 1) : J;
                int k0 = C->cz ? 2 * K : K, k1 = C->cz ? (2 * K + 1 < F->nz ? 2 * K + 1 : F->nz - 1) : K;
                double acc = 0;
                for (int i = i0; i <= i1; i++)
                    for (int j = j0; j <= j1; j++)
                        for (int k = k0; k <= k1; k++) {
                            long q = ((long)i * F->ny + j) * F->nz + k;
                            if (F->diag[q] != 0) acc += F->r[q] - F->diag[q] * F->z[q] + coarse_off(o, F, i, j, k);
                        }
                C->r[((long)I * C->ny + J) * C->nz + K] = acc;
            }
}

static void coarse_prolong(Level *C, Level *F) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < F->nx; i++)
        for (int j = 0; j < F->ny; j++)
            for (int k = 0; k < F->nz; k++) {
                long q = ((long)i * F->ny + j) * F->nz + k;
                if (F->diag[q] == 0) continue;
                F->z[q] += C->z[((long)(C->cx ? i >> 1 : i) * C->ny + (C->cy ? j >> 1 : j)) * C->nz + (C->cz ? k >> 1 : k)];
            }
}

static void coarse_vcycle(Oracle *o, int l) {
    Level *L = &o->lev[l];
    memset(L->z, 0, sizeof(double) * L->n);
    if (l == o->nlev - 1) {
        coarse_smooth(o, L, 40);
        return;
    }
    coarse_smooth(o, L, 2);
    coarse_restrict(o, L, &o->lev[l + 1]);
    coarse_vcycle(o, l + 1);
    coarse_prolong(&o->lev[l + 1], L);
    coarse_smooth(o, L, 2);
}

static void fine_smooth(const Oracle *o, const double *r, double *z, double *gtmp) {
    const int *per = o->per;
    int ncol = ((per[0] && (o->nx & 1)) || (per[1] && (o->ny & 1)) || (per[2] && (o->nz & 1))) ? 4 : 2;
    for (int col = 0; col < ncol; col++) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < o->nx; i++)
            for (int j = 0; j < o->ny; j++)
                for (int k = 0; k < o->nz; k++) {
                    if (color_of(i, j, k, o->nx, o->ny, o->nz, per) != col) continue;
                    long P = CI(o, i, j, k);
                    int fl = o->flag[P];
                    if (fl == GH) continue;
                    if (fl != FL || (o->singular && i == 0 && j == 0 && k == 0)) {
                        z[P] = r[P];
                        continue;
                    }
                    double cs = C1(o->kyN, j) + C1(o->kxE, i) + C1(o->kyS, j) + C1(o->kxW, i) + C1(o->kzD, k) + C1(o->kzU, k);
                    double nb = C1(o->kxW, i) * z[P - o->sx] + C1(o->kxE, i) * z[P + o->sx] + C1(o->kyS, j) * z[P - o->sy] +
                                C1(o->kyN, j) * z[P + o->sy] + C1(o->kzD, k) * z[P - 1] + C1(o->kzU, k) * z[P + 1];
                    z[P] = r[P] + nb / cs;
                }
    }
#pragma omp parallel for schedule(static)
    for (int g = 0; g < o->ng; g++) {
        double w[8], ws, sum = 0;
        int keep[8];
        ghost_row(o, g, w, keep, &ws);
        for (int l = 0; l < 8; l++)
            if (keep[l]) sum += w[l] * z[CI(o, o->gidx[g][l][0], o->gidx[g][l][1], o->gidx[g][l][2])];
        long P = o->gcell[g];
        double d = 1 - ws;
        gtmp[g] = d >= 0.25 ? (r[P] + sum) / d : ws * z[P] + r[P] + sum;
    }
    for (int g = 0; g < o->ng; g++) z[o->gcell[g]] = gtmp[g];
    /* Outer rows solved for the outer value given the interior. */
#pragma omp parallel for schedule(static)
    for (int i = -2; i < o->nx + 2; i++)
        for (int j = -2; j < o->ny + 2; j++)
            for (int k = -2; k < o->nz + 2; k++) {
                int L;
                int f = owner(o, i, j, k, &L);
                if (f < 0) continue;
                long P = CI(o, i, j, k);
                /* row(P) = a*z_P + (rest); a = coefficient of z_P. */
                double zp = z[P];
                z[P] = 0;
                double rest = row(o, 4, z, i, j, k);
                z[P] = 1;
                double a = row(o, 4, z, i, j, k) - rest;
                z[P] = zp;
                (void)zp;
                z[P] = (r[P] - rest) / a;
            }
}

static void mg_apply(Oracle *o, const double *r, double *z) {
    memset(z, 0, sizeof(double) * o->nc);
    double *gtmp = o->gtmp;
    if (o->nlev == 0) {
        for (int s = 0; s < 8; s++) fine_smooth(o, r, z, gtmp);
        return;
    }
    fine_smooth(o, r, z, gtmp);
    fine_smooth(o, r, z, gtmp);
    Level *L1 = &o->lev[0];
#pragma omp parallel for schedule(static)
    for (int I = 0; I < L1->nx; I++)
        for (int J = 0; J < L1->ny; J++)
            for (int K = 0; K < L1->nz; K++) {
                int i0 = L1->cx ? 2 * I : I, i1 = L1->cx ? (2 * I + 1 < o->nx ? 2 * I + 1 : o->nx - 1) : I;
                int j0 = L1->cy ? 2 * J : J, j1 = L1->cy ? (2 * J + 1 < o->ny ? 2 * J + 1 : o->ny - 1) : J;
                int k0 = L1->cz ? 2 * K : K, k1 = L1->cz ? (2 * K + 1 < o->nz ? 2 * K + 1 : o->nz - 1) : K;
                double acc = 0;
                for (int i = i0; i <= i1; i++)
                    for (int j = j0; j <= j1; j++)
                        for (int k = k0; k <= k1; k++) {
                            if (!active0(o, i, j, k)) continue;
                            long P = CI(o, i, j, k);
                            double res = r[P] - row(o, 4, z, i, j, k);
                            double cs = C1(o->kyN, j) + C1(o->kxE, i) + C1(o->kyS, j) + C1(o->kxW, i) + C1(o->kzD, k) + C1(o->kzU, k);
                            acc += C1(o->dx, i) * C1(o->dy, j) * C1(o->dz, k) * cs * res;
                        }
                L1->r[((long)I * L1->ny + J) * L1->nz + K] = acc;
            }
    coarse_vcycle(o, 0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                long P = CI(o, i, j, k);
                int fl = o->flag[P];
                if (fl != FL && fl != GH) continue;
                if (o->singular && i == 0 && j == 0 && k == 0) continue;
                z[P] += L1->z[((long)(L1->cx ? i >> 1 : i) * L1->ny + (L1->cy ? j >> 1 : j)) * L1->nz + (L1->cz ? k >> 1 : k)];
            }
    fine_smooth(o, r, z, gtmp);
    fine_smooth(o, r, z, gtmp);
}

/* --------------------------------------------------------------- Krylov -- */
/* hypre-style right-preconditioned BiCGSTAB from x0 = 0. */
static int bicgstab(Oracle *o, int type, const double *b, double *x, int maxit, int precond, int *iters, double *relres) {
    const long n = o->nc;
    double *r = o->r, *r0 = o->r0, *p = o->pv, *v = o->v, *s = o->s, *t = o->t;
    double *ph = precond ? o->ph : p, *sh = precond ? o->sh : s;
    double bb;
    PSUM(bb, n, b[q] * b[q]);
    for (long q = 0; q < n; q++) {
        x[q] = 0;
        r[q] = b[q];
        r0[q] = b[q];
        p[q] = 0;
        v[q] = 0;
    }
    *iters = 0;
    if (bb == 0) {
        *relres = 0;
        return 0;
    }
    const double bn = sqrt(bb);
    double rho = bb, alpha = 1, omega = 1, beta = 0, rr = bb;
    int it = 0, conv = 0;
    const int divmode = type == 4 && o->divtol > 0;
    while (it < maxit) {
        it++;
#pragma omp parallel for schedule(static)
        for (long q = 0; q < n; q++) p[q] = r[q] + beta * (p[q] - omega * v[q]);
        if (precond) mg_apply(o, p, ph);
        apply(o, type, ph, v);
        double r0v;
        PSUM(r0v, n, r0[q] * v[q]);
        if (r0v == 0) break;
        alpha = rho / r0v;
#pragma omp parallel for schedule(static)
        for (long q = 0; q < n; q++) s[q] = r[q] - alpha * v[q];
        double ss;
        PSUM(ss, n, s[q] * s[q]);
        int half = 0;
        if (divmode) {
            double m = 0;
            for (int i = 0; i < o->nx; i++)
                for (int j = 0; j < o->ny; j++)
                    for (int k = 0; k < o->nz; k++) {
                        long P = CI(o, i, j, k);
                        if (o->coeffsum[P] == 0) continue;
                        double w = 2 * o->Re * o->coeffsum[P] * fabs(s[P]);
                        m = m > w ? m : w;
                    }
            half = m <= o->divtol;
        } else {
            half = sqrt(ss) < o->tol * bn;
        }
        if (half) {
#pragma omp parallel for schedule(static)
            for (long q = 0; q < n; q++) {
                x[q] += alpha * ph[q];
                r[q] = s[q];
            }
            rr = ss;
            conv = 1;
            break;
        }
        if (precond) mg_apply(o, s, sh);
        apply(o, type, sh, t);
        double ts, tt;
        PSUM(ts, n, t[q] * s[q]);
        PSUM(tt, n, t[q] * t[q]);
        if (tt == 0) break;
        omega = ts / tt;
#pragma omp parallel for schedule(static)
        for (long q = 0; q < n; q++) {
            x[q] += alpha * ph[q] + omega * sh[q];
            r[q] = s[q] - omega * t[q];
        }
        double rho1;
        PSUM(rr, n, r[q] * r[q]);
        PSUM(rho1, n, r0[q] * r[q]);
        beta = (rho1 / rho) * (alpha / omega);
        rho = rho1;
        int ok;
        if (divmode) {
            double m = 0;
            for (int i = 0; i < o->nx; i++)
                for (int j = 0; j < o->ny; j++)
                    for (int k = 0; k < o->nz; k++) {
                        long P = CI(o, i, j, k);
                        if (o->coeffsum[P] == 0) continue;
                        double w = 2 * o->Re * o->coeffsum[P] * fabs(r[P]);
                        m = m > w ? m : w;
                    }
            ok = m <= o->divtol;
        } else {
            ok = sqrt(rr) < o->tol * bn;
        }
        if (ok) {
            conv = 1;
            break;
        }
        if (rho1 == 0) break;
    }
    *iters = it;
    *relres = sqrt(rr) / bn;
    return conv ? 0 : 1;
}

/* ------------------------------------------------------------- the step -- */
/* update_outer (src/ibm3d_fracstep.c:855-1906). */
static void update_outer(Oracle *o) {
    double *u1 = o->u[0], *u2 = o->u[1], *u3 = o->u[2], *p = o->p;
    double *u[3] = {u1, u2, u3};
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    /* Axis-generic form of the six face blocks; each block runs after the
       previous ones, as in the reference, so edges see earlier faces. */
    for (int axis = 0; axis < 3; axis++) {
        const double *d = axis == 0 ? o->dx : axis == 1 ? o->dy : o->dz;
        const double *c = axis == 0 ? o->xc : axis == 1 ? o->yc : o->zc;
        const int N = axis == 0 ? nx : axis == 1 ? ny : nz;
        const long s = axis == 0 ? o->sx : axis == 1 ? o->sy : 1;
        const int flo = axis == 0 ? FW : axis == 1 ? FS : FD, fhi = axis == 0 ? FE : axis == 1 ? FN : FU;
        int na, nb;
        if (axis == 0) { na = ny; nb = nz; }
        else if (axis == 1) { na = nx + 4; nb = nz; }
        else { na = nx + 4; nb = ny + 4; }
        for (int side = 0; side < 2; side++) {
            const int f = side == 0 ? flo : fhi, t = o->bct[f];
            const double *dp = (f == FD) ? o->dx : d; /* down face pressure fill reads dx (src/ibm3d_fracstep.c:1792-1800) */
#pragma omp parallel for schedule(static)
            for (int A = 0; A < na; A++)
                for (int B = 0; B < nb; B++) {
                    long base;
                    if (axis == 0) base = CI(o, 0, A, B);
                    else if (axis == 1) base = CI(o, A - 2, 0, B);
                    else base = CI(o, A - 2, B - 2, 0);
                    long c0, c1, o1, o2, i1, i2;
                    double a1, b1, a2, b2, ea1, eb1, ea2, eb2, pa1, pb1, pa2, pb2;
                    if (side == 0) {
                        c0 = base; c1 = base + s; o1 = base - s; o2 = base - 2 * s;
                        i1 = base + (long)(N - 1) * s; i2 = base + (long)(N - 2) * s;
                        a1 = C1(d, -1) / 2; b1 = C1(d, 0) / 2; a2 = C1(d, -2) / 2 + C1(d, -1); b2 = C1(d, 0) + C1(d, 1) / 2;
                        pa1 = C1(dp, -1) / 2; pb1 = C1(dp, 0) / 2; pa2 = C1(dp, -2) / 2 + C1(dp, -1); pb2 = C1(dp, 0) + C1(dp, 1) / 2;
                        ea1 = C1(c, 0) - C1(c, -1); eb1 = C1(c, 1) - C1(c, 0);
                        ea2 = C1(c, -1) - C1(c, -2); eb2 = C1(c, 0) - C1(c, -1);
                    } else {
                        c0 = base + (long)(N - 1) * s; c1 = c0 - s; o1 = c0 + s; o2 = c0 + 2 * s;
                        i1 = base; i2 = base + s;
                        a1 = C1(d, N - 1) / 2; b1 = C1(d, N) / 2; a2 = C1(d, N - 2) / 2 + C1(d, N - 1); b2 = C1(d, N) + C1(d, N + 1) / 2;
                        pa1 = C1(dp, N - 1) / 2; pb1 = C1(dp, N) / 2; pa2 = C1(dp, N - 2) / 2 + C1(dp, N - 1); pb2 = C1(dp, N) + C1(dp, N + 1) / 2;
                        ea1 = C1(c, N - 1) - C1(c, N - 2); eb1 = C1(c, N) - C1(c, N - 1);
                        ea2 = C1(c, N) - C1(c, N - 1); eb2 = C1(c, N + 1) - C1(c, N);
                    }
                    /* padded (i, j, k) of the line's first outer cell, for the face centre */
                    const int li = axis == 0 ? 0 : A - 2, lj = axis == 0 ? A : axis == 1 ? 0 : B - 2;
                    const int lk = axis == 2 ? 0 : B;
                    for (int l = 0; l < 3; l++) {
                        double *w = u[l];
                        double bc = t == BC_VEL ? bcval(o, f, l, o->time, li, lj, lk) : 0.0;
                        switch (t) {
                        case BC_VEL:
                            if (side == 0) {
                                w[o1] = (a1 + b1) / b1 * bc - a1 / b1 * w[c0];
                                w[o2] = (a2 + b2) / b2 * bc - a2 / b2 * w[c1];
                            } else {
                                w[o1] = (a1 + b1) / a1 * bc - b1 / a1 * w[c0];
                                w[o2] = (a2 + b2) / a2 * bc - b2 / a2 * w[c1];
                            }
                            break;
                        case BC_PRES:
                            if (side == 0) {
                                w[o1] = (ea1 + eb1) / eb1 * w[c0] - ea1 / eb1 * w[c1];
                                w[o2] = (ea2 + eb2) / eb2 * w[o1] - ea2 / eb2 * w[c0];
                            } else {
                                w[o1] = (ea1 + eb1) / ea1 * w[c0] - eb1 / ea1 * w[c1];
                                w[o2] = (ea2 + eb2) / ea2 * w[o1] - eb2 / ea2 * w[c0];
                            }
                            break;
                        case BC_SLIP:
                            if (l == axis) {
                                w[o1] = side == 0 ? -a1 / b1 * w[c0] : -b1 / a1 * w[c0];
                                w[o2] = side == 0 ? -a2 / b2 * w[c1] : -b2 / a2 * w[c1];
                            } else {
                                w[o1] = w[c0];
                                w[o2] = w[c1];
                            }
                            break;
                        case BC_PER:
                        case BC_VELPER:
                            w[o1] = w[i1];
                            w[o2] = w[i2];
                            break;
                        }
                    }
                    switch (t) {
                    case BC_VEL:
                    case BC_SLIP:
                        p[o1] = p[c0];
                        p[o2] = p[c1];
                        break;
                    case BC_PRES:
                    case BC_VELPER: {
                        const double pv = bcval(o, f, 3, o->time, li, lj, lk);
                        if (side == 0) {
                            p[o1] = (pa1 + pb1) / pb1 * pv - pa1 / pb1 * p[c0];
                            p[o2] = (pa2 + pb2) / pb2 * pv - pa2 / pb2 * p[c1];
                        } else {
                            p[o1] = (pa1 + pb1) / pa1 * pv - pb1 / pa1 * p[c0];
                            p[o2] = (pa2 + pb2) / pa2 * pv - pb2 / pa2 * p[c1];
                        }
                        break;
                    }
                    case BC_PER:
                        p[o1] = p[i1];
                        p[o2] = p[i2];
                        break;
                    }
                }
        }
    }
}

/* update_ghost (src/ibm3d_fracstep.c:1915-1976): sequential in-place sweep. */
static void update_ghost(Oracle *o) {
    double *u1 = o->u[0], *u2 = o->u[1], *u3 = o->u[2], *p = o->p;
    int g = 0;
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                long P = CI(o, i, j, k);
                if (o->flag[P] == GH) {
                    double w[8], ws;
                    int keep[8];
                    ghost_row(o, g, w, keep, &ws);
                    double s1 = 0, s2 = 0, s3 = 0, sp = 0;
                    for (int l = 0; l < 8; l++) {
                        if (!keep[l]) continue;
                        long q = CI(o, o->gidx[g][l][0], o->gidx[g][l][1], o->gidx[g][l][2]);
                        s1 += w[l] * u1[q];
                        s2 += w[l] * u2[q];
                        s3 += w[l] * u3[q];
                        sp += w[l] * p[q];
                    }
                    double lu = 1 + ws, lp = 1 - ws;
                    u1[P] = -s1 / lu;
                    u2[P] = -s2 / lu;
                    u3[P] = -s3 / lu;
                    if (lp != 0) p[P] = sp / lp;
                    g++;
                } else if (o->flag[P] == SO) {
                    u1[P] = u2[P] = u3[P] = p[P] = NAN;
                }
            }
}

/* interp_stag_vel (src/ibm3d_fracstep.c:807-845). */
static void interp_stag_vel(Oracle *o) {
    const double *dx = o->dx, *dy = o->dy, *dz = o->dz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= o->nx; i++)
        for (int j = -2; j < o->ny + 2; j++)
            for (int k = -2; k < o->nz + 2; k++)
                XS(o->U[0], i, j, k) = (C3(o->u[0], i - 1, j, k) * C1(dx, i) + C3(o->u[0], i, j, k) * C1(dx, i - 1)) / (C1(dx, i - 1) + C1(dx, i));
#pragma omp parallel for schedule(static)
    for (int i = -2; i < o->nx + 2; i++)
        for (int j = 0; j <= o->ny; j++)
            for (int k = -2; k < o->nz + 2; k++)
                YS(o->U[1], i, j, k) = (C3(o->u[1], i, j - 1, k) * C1(dy, j) + C3(o->u[1], i, j, k) * C1(dy, j - 1)) / (C1(dy, j - 1) + C1(dy, j));
#pragma omp parallel for schedule(static)
    for (int i = -2; i < o->nx + 2; i++)
        for (int j = -2; j < o->ny + 2; j++)
            for (int k = 0; k <= o->nz; k++)
                ZS(o->U[2], i, j, k) = (C3(o->u[2], i, j, k - 1) * C1(dz, k) + C3(o->u[2], i, j, k) * C1(dz, k - 1)) / (C1(dz, k - 1) + C1(dz, k));
}

/* calc_N (src/ibm3d_fracstep.c:117-170). */
static void calc_N(Oracle *o) {
    const double *dx = o->dx, *dy = o->dy, *dz = o->dz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (C3(o->flag, i, j, k) == FL) {
                    for (int l = 0; l < 3; l++) {
                        const double *u = o->u[l];
                        double uw = (C3(u, i - 1, j, k) * C1(dx, i) + C3(u, i, j, k) * C1(dx, i - 1)) / (C1(dx, i - 1) + C1(dx, i));
                        double ue = (C3(u, i, j, k) * C1(dx, i + 1) + C3(u, i + 1, j, k) * C1(dx, i)) / (C1(dx, i) + C1(dx, i + 1));
                        double us = (C3(u, i, j - 1, k) * C1(dy, j) + C3(u, i, j, k) * C1(dy, j - 1)) / (C1(dy, j - 1) + C1(dy, j));
                        double un = (C3(u, i, j, k) * C1(dy, j + 1) + C3(u, i, j + 1, k) * C1(dy, j)) / (C1(dy, j) + C1(dy, j + 1));
                        double ud = (C3(u, i, j, k - 1) * C1(dz, k) + C3(u, i, j, k) * C1(dz, k - 1)) / (C1(dz, k - 1) + C1(dz, k));
                        double uu = (C3(u, i, j, k) * C1(dz, k + 1) + C3(u, i, j, k + 1) * C1(dz, k)) / (C1(dz, k) + C1(dz, k + 1));
                        C3(o->N[l], i, j, k) = (XS(o->U[0], i + 1, j, k) * ue - XS(o->U[0], i, j, k) * uw) / C1(dx, i) +
                                              (YS(o->U[1], i, j + 1, k) * un - YS(o->U[1], i, j, k) * us) / C1(dy, j) +
                                              (ZS(o->U[2], i, j, k + 1) * uu - ZS(o->U[2], i, j, k) * ud) / C1(dz, k);
                    }
                } else {
                    for (int l = 0; l < 3; l++) C3(o->N[l], i, j, k) = NAN;
                }
            }
}

/* IBMSolver_calc_tau_r + calc_S (src/ibm3d_turb.c:8-82). */
static void calc_tau(Oracle *o) {
    if (o->cs < 0) return;
    const double *xc = o->xc, *yc = o->yc, *zc = o->zc;
    const double *u1 = o->u[0], *u2 = o->u[1], *u3 = o->u[2];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (C3(o->flag, i, j, k) != FL) continue;
                double S[3][3];
                S[0][0] = (C3(u1, i + 1, j, k) - C3(u1, i - 1, j, k)) / (C1(xc, i + 1) - C1(xc, i - 1));
                S[0][1] = S[1][0] = 0.5 * ((C3(u1, i, j + 1, k) - C3(u1, i, j - 1, k)) / (C1(yc, j + 1) - C1(yc, j - 1)) +
                                           (C3(u2, i + 1, j, k) - C3(u2, i - 1, j, k)) / (C1(xc, i + 1) - C1(xc, i - 1)));
                S[0][2] = S[2][0] = 0.5 * ((C3(u1, i, j, k + 1) - C3(u1, i, j, k - 1)) / (C1(zc, k + 1) - C1(zc, k - 1)) +
                                           (C3(u3, i + 1, j, k) - C3(u3, i - 1, j, k)) / (C1(xc, i + 1) - C1(xc, i - 1)));
                S[1][1] = (C3(u2, i, j + 1, k) - C3(u2, i, j - 1, k)) / (C1(yc, j + 1) - C1(yc, j - 1));
                S[1][2] = S[2][1] = 0.5 * ((C3(u2, i, j, k + 1) - C3(u2, i, j, k - 1)) / (C1(zc, k + 1) - C1(zc, k - 1)) +
                                           (C3(u3, i, j + 1, k) - C3(u3, i, j - 1, k)) / (C1(yc, j + 1) - C1(yc, j - 1)));
                S[2][2] = (C3(u3, i, j, k + 1) - C3(u3, i, j, k - 1)) / (C1(zc, k + 1) - C1(zc, k - 1));
                double delta = 2 * cbrt(C1(o->dx, i) * C1(o->dy, j) * C1(o->dz, k));
                double sm = 0;
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) sm += 2 * (S[a][b] * S[a][b]);
                sm = sqrt(sm);
                double la = o->cs * delta, lb = 0.41 * C3(o->lvset, i, j, k);
                double l = la < lb ? la : lb;
                int t = 0;
                for (int a = 0; a < 3; a++)
                    for (int b = a; b < 3; b++) C3(o->tau[t++], i, j, k) = -2 * (l * l) * sm * S[a][b];
            }
}

static const double *tau_of(const Oracle *o, int a, int b) {
    static const int map[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    return o->tau[map[a][b]];
}

/* calc_u_star (src/ibm3d_fracstep.c:172-386). */
static void calc_u_star(Oracle *o) {
    calc_tau(o);
    const double dt = o->dt;
    for (int l = 0; l < 3; l++) {
        double *b = o->b;
        memset(b, 0, sizeof(double) * o->nc);
        const double *u = o->u[l];
#pragma omp parallel for schedule(static)
        for (int i = 0; i < o->nx; i++)
            for (int j = 0; j < o->ny; j++)
                for (int k = 0; k < o->nz; k++) {
                    if (C3(o->flag, i, j, k) != FL) continue;
                    double dp;
                    if (l == 0) dp = (C3(o->p, i + 1, j, k) - C3(o->p, i - 1, j, k)) / (C1(o->xc, i + 1) - C1(o->xc, i - 1));
                    else if (l == 1) dp = (C3(o->p, i, j + 1, k) - C3(o->p, i, j - 1, k)) / (C1(o->yc, j + 1) - C1(o->yc, j - 1));
                    else dp = (C3(o->p, i, j, k + 1) - C3(o->p, i, j, k - 1)) / (C1(o->zc, k + 1) - C1(o->zc, k - 1));
                    double dtau = 0;
                    if (o->cs >= 0) {
                        const double *t1 = tau_of(o, l, 0), *t2 = tau_of(o, l, 1), *t3 = tau_of(o, l, 2);
                        dtau = (C3(t1, i + 1, j, k) - C3(t1, i - 1, j, k)) / (C1(o->xc, i + 1) - C1(o->xc, i - 1)) +
                               (C3(t2, i, j + 1, k) - C3(t2, i, j - 1, k)) / (C1(o->yc, j + 1) - C1(o->yc, j - 1)) +
                               (C3(t3, i, j, k + 1) - C3(t3, i, j, k - 1)) / (C1(o->zc, k + 1) - C1(o->zc, k - 1));
                    }
                    C3(b, i, j, k) = -dt / 2 * (3 * C3(o->N[l], i, j, k) - C3(o->Np[l], i, j, k)) - dt * dp +
                                     (1 - C1(o->kxW, i) - C1(o->kxE, i) - C1(o->kyS, j) - C1(o->kyN, j) - C1(o->kzD, k) - C1(o->kzU, k)) * C3(u, i, j, k) +
                                     C1(o->kxW, i) * C3(u, i - 1, j, k) + C1(o->kxE, i) * C3(u, i + 1, j, k) +
                                     C1(o->kyS, j) * C3(u, i, j - 1, k) + C1(o->kyN, j) * C3(u, i, j + 1, k) +
                                     C1(o->kzD, k) * C3(u, i, j, k - 1) + C1(o->kzU, k) * C3(u, i, j, k + 1) +
                                     dt * (o->ffn[l] ? o->ffn[l](o->time, C1(o->xc, i), C1(o->yc, j), C1(o->zc, k)) : o->f[l]) -
                                     dt * dtau;
                }
        /* Velocity-BC rows of the outer layers. */
        for (int i = -2; i < o->nx + 2; i++)
            for (int j = -2; j < o->ny + 2; j++)
                for (int k = -2; k < o->nz + 2; k++) {
                    int L, f = owner(o, i, j, k, &L);
                    if (f >= 0 && o->bct[f] == BC_VEL) C3(b, i, j, k) = bcval(o, f, l, o->time, i, j, k);
                }
        bicgstab(o, l + 1, b, o->us[l], 200, 0, &o->iters[l], &o->res[l]);
    }
}

/* calc_u_tilde + calc_U_star (src/ibm3d_fracstep.c:388-487). */
static void calc_U_star(Oracle *o) {
    const double dt = o->dt;
    const double *xc = o->xc, *yc = o->yc, *zc = o->zc, *dx = o->dx, *dy = o->dy, *dz = o->dz;
#pragma omp parallel for schedule(static)
    for (int i = -1; i < o->nx + 1; i++)
        for (int j = -1; j < o->ny + 1; j++)
            for (int k = -1; k < o->nz + 1; k++) {
                C3(o->ut[0], i, j, k) = C3(o->us[0], i, j, k) + dt * (C3(o->p, i + 1, j, k) - C3(o->p, i - 1, j, k)) / (C1(xc, i + 1) - C1(xc, i - 1));
                C3(o->ut[1], i, j, k) = C3(o->us[1], i, j, k) + dt * (C3(o->p, i, j + 1, k) - C3(o->p, i, j - 1, k)) / (C1(yc, j + 1) - C1(yc, j - 1));
                C3(o->ut[2], i, j, k) = C3(o->us[2], i, j, k) + dt * (C3(o->p, i, j, k + 1) - C3(o->p, i, j, k - 1)) / (C1(zc, k + 1) - C1(zc, k - 1));
            }
    const int *fl = o->flag;
#define FG(a, b) (((a) == FL && (b) == GH) || ((a) == GH && (b) == FL))
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (FG(C3(fl, i - 1, j, k), C3(fl, i, j, k)))
                    XS(o->Us[0], i, j, k) = (C3(o->us[0], i - 1, j, k) * C1(dx, i) + C3(o->us[0], i, j, k) * C1(dx, i - 1)) / (C1(dx, i - 1) + C1(dx, i));
                else
                    XS(o->Us[0], i, j, k) = (C3(o->ut[0], i - 1, j, k) * C1(dx, i) + C3(o->ut[0], i, j, k) * C1(dx, i - 1)) / (C1(dx, i - 1) + C1(dx, i)) -
                                            dt * (C3(o->p, i, j, k) - C3(o->p, i - 1, j, k)) / (C1(xc, i) - C1(xc, i - 1));
            }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j <= o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (FG(C3(fl, i, j - 1, k), C3(fl, i, j, k)))
                    YS(o->Us[1], i, j, k) = (C3(o->us[1], i, j - 1, k) * C1(dy, j) + C3(o->us[1], i, j, k) * C1(dy, j - 1)) / (C1(dy, j - 1) + C1(dy, j));
                else
                    YS(o->Us[1], i, j, k) = (C3(o->ut[1], i, j - 1, k) * C1(dy, j) + C3(o->ut[1], i, j, k) * C1(dy, j - 1)) / (C1(dy, j - 1) + C1(dy, j)) -
                                            dt * (C3(o->p, i, j, k) - C3(o->p, i, j - 1, k)) / (C1(yc, j) - C1(yc, j - 1));
            }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k <= o->nz; k++) {
                if (FG(C3(fl, i, j, k - 1), C3(fl, i, j, k)))
                    ZS(o->Us[2], i, j, k) = (C3(o->us[2], i, j, k - 1) * C1(dz, k) + C3(o->us[2], i, j, k) * C1(dz, k - 1)) / (C1(dz, k - 1) + C1(dz, k));
                else
                    ZS(o->Us[2], i, j, k) = (C3(o->ut[2], i, j, k - 1) * C1(dz, k) + C3(o->ut[2], i, j, k) * C1(dz, k - 1)) / (C1(dz, k - 1) + C1(dz, k)) -
                                            dt * (C3(o->p, i, j, k) - C3(o->p, i, j, k - 1)) / (C1(zc, k) - C1(zc, k - 1));
            }
}

/* calc_p_prime (src/ibm3d_fracstep.c:489-707).  Outer rows of pressure
   and velocity-periodic faces hold p_bc(t+dt) - p_bc(t) (:556-645), zero
   for constant values. */
static void calc_p_prime(Oracle *o) {
    double *b = o->b;
    memset(b, 0, sizeof(double) * o->nc);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (o->singular && i == 0 && j == 0 && k == 0) continue;
                if (C3(o->flag, i, j, k) != FL) continue;
                double v = -1 / (2 * o->Re) *
                           ((XS(o->Us[0], i + 1, j, k) - XS(o->Us[0], i, j, k)) / C1(o->dx, i) +
                            (YS(o->Us[1], i, j + 1, k) - YS(o->Us[1], i, j, k)) / C1(o->dy, j) +
                            (ZS(o->Us[2], i, j, k + 1) - ZS(o->Us[2], i, j, k)) / C1(o->dz, k));
                C3(b, i, j, k) = v / C3(o->coeffsum, i, j, k);
            }
    for (int i = -2; i < o->nx + 2; i++)
        for (int j = -2; j < o->ny + 2; j++)
            for (int k = -2; k < o->nz + 2; k++) {
                int L, f = owner(o, i, j, k, &L);
                if (f >= 0 && o->bcfn[f][3] && (o->bct[f] == BC_PRES || o->bct[f] == BC_VELPER))
                    C3(b, i, j, k) = bcval(o, f, 3, o->time + o->dt, i, j, k) - bcval(o, f, 3, o->time, i, j, k);
            }
    bicgstab(o, 4, b, o->pp, 1000, 1, &o->iters[3], &o->res[3]);
}

/* update_next (src/ibm3d_fracstep.c:709-805) plus max|div U^{n+1}|. */
static void update_next(Oracle *o) {
    const double dt = o->dt;
    const int *fl = o->flag;
    double *pp = o->pp;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                int f = C3(fl, i, j, k);
                C3(o->pn, i, j, k) = (f == FL || f == GH) ? C3(o->p, i, j, k) + C3(pp, i, j, k) : NAN;
                if (f == FL) {
                    C3(o->un[0], i, j, k) = C3(o->us[0], i, j, k) - dt * (C3(pp, i + 1, j, k) - C3(pp, i - 1, j, k)) / (C1(o->xc, i + 1) - C1(o->xc, i - 1));
                    C3(o->un[1], i, j, k) = C3(o->us[1], i, j, k) - dt * (C3(pp, i, j + 1, k) - C3(pp, i, j - 1, k)) / (C1(o->yc, j + 1) - C1(o->yc, j - 1));
                    C3(o->un[2], i, j, k) = C3(o->us[2], i, j, k) - dt * (C3(pp, i, j, k + 1) - C3(pp, i, j, k - 1)) / (C1(o->zc, k + 1) - C1(o->zc, k - 1));
                } else if (f == SO) {
                    C3(o->un[0], i, j, k) = C3(o->un[1], i, j, k) = C3(o->un[2], i, j, k) = NAN;
                }
            }
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++)
                XS(o->Un[0], i, j, k) = (C3(fl, i - 1, j, k) != SO && C3(fl, i, j, k) != SO)
                    ? XS(o->Us[0], i, j, k) - dt * (C3(pp, i, j, k) - C3(pp, i - 1, j, k)) / (C1(o->xc, i) - C1(o->xc, i - 1)) : NAN;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j <= o->ny; j++)
            for (int k = 0; k < o->nz; k++)
                YS(o->Un[1], i, j, k) = (C3(fl, i, j - 1, k) != SO && C3(fl, i, j, k) != SO)
                    ? YS(o->Us[1], i, j, k) - dt * (C3(pp, i, j, k) - C3(pp, i, j - 1, k)) / (C1(o->yc, j) - C1(o->yc, j - 1)) : NAN;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k <= o->nz; k++)
                ZS(o->Un[2], i, j, k) = (C3(fl, i, j, k - 1) != SO && C3(fl, i, j, k) != SO)
                    ? ZS(o->Us[2], i, j, k) - dt * (C3(pp, i, j, k) - C3(pp, i, j, k - 1)) / (C1(o->zc, k) - C1(o->zc, k - 1)) : NAN;
    double m = 0;
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (C3(fl, i, j, k) != FL || (o->singular && i == 0 && j == 0 && k == 0)) continue;
                double d = (XS(o->Un[0], i + 1, j, k) - XS(o->Un[0], i, j, k)) / C1(o->dx, i) +
                           (YS(o->Un[1], i, j + 1, k) - YS(o->Un[1], i, j, k)) / C1(o->dy, j) +
                           (ZS(o->Un[2], i, j, k + 1) - ZS(o->Un[2], i, j, k)) / C1(o->dz, k);
                m = m > fabs(d) ? m : fabs(d);
            }
    o->maxdiv = m;
    for (int l = 0; l < 3; l++) {
        double *t;
        t = o->u[l]; o->u[l] = o->un[l]; o->un[l] = t;
        t = o->U[l]; o->U[l] = o->Un[l]; o->Un[l] = t;
        t = o->N[l]; o->N[l] = o->Np[l]; o->Np[l] = t;
    }
    double *t = o->p; o->p = o->pn; o->pn = t;
}

/* IBMSolver_iterate (src/ibm3d_fracstep.c:38-115). */
void oracle_iterate(Oracle *o, int nsteps) {
    if (o->threads > 0) omp_set_num_threads(o->threads);
    double start = o->time;
    update_outer(o);
    interp_stag_vel(o);
    update_ghost(o);
    calc_N(o);
    for (int l = 0; l < 3; l++) {
        double *t = o->N[l];
        o->N[l] = o->Np[l];
        o->Np[l] = t;
    }
    for (int i = 1; i <= nsteps; i++) {
        calc_N(o);
        calc_u_star(o);
        calc_U_star(o);
        calc_p_prime(o);
        update_next(o);
        o->iter++;
        o->time = start + o->dt * i;
        update_outer(o);
        update_ghost(o);
    }
}

/* -------------------------------------------------------------- set-up -- */
Oracle *oracle_create(const OracleConfig *c) {
    Oracle *o = (Oracle *)calloc(1, sizeof(Oracle));
    o->threads = c->threads;
    if (o->threads > 0) omp_set_num_threads(o->threads);
    o->nx = c->nx; o->ny = c->ny; o->nz = c->nz;
    o->sy = c->nz + 4;
    o->sx = (long)(c->ny + 4) * o->sy;
    o->nc = (long)(c->nx + 4) * o->sx;
    o->Re = c->Re; o->dt = c->dt;
    o->cs = c->smagorinsky_cs;
    o->tol = c->tol;
    o->divtol = c->div_tol;
    memcpy(o->f, c->force, sizeof o->f);
    for (int l = 0; l < 3; l++) o->ffn[l] = c->force_fn[l];
    o->xmin = c->xf[0]; o->xmax = c->xf[c->nx];
    o->ymin = c->yf[0]; o->ymax = c->yf[c->ny];
    o->zmin = c->zf[0]; o->zmax = c->zf[c->nz];
    o->singular = 1;
    for (int f = 0; f < 6; f++) {
        int t = c->bc_type[f];
        /* IBMSolver_set_bc rewrites (src/ibm3d_setup.c:403-412). */
        if (t == BC_WALL) t = BC_VEL;
        if (t == BC_SYM) t = BC_SLIP;
        o->bct[f] = t;
        for (int l = 0; l < 3; l++) o->bu[f][l] = c->bc_type[f] == BC_WALL ? 0 : c->bc_u[f][l];
        o->bp[f] = c->bc_p[f];
        for (int q = 0; q < 4; q++) o->bcfn[f][q] = c->bc_fn[f][q];
        if (t == BC_PRES || t == BC_VELPER) o->singular = 0;
    }
    o->dx = dal(o->nx + 4); o->dy = dal(o->ny + 4); o->dz = dal(o->nz + 4);
    o->xc = dal(o->nx + 4); o->yc = dal(o->ny + 4); o->zc = dal(o->nz + 4);
    o->kxW = dal(o->nx + 4); o->kxE = dal(o->nx + 4); o->kyS = dal(o->ny + 4);
    o->kyN = dal(o->ny + 4); o->kzD = dal(o->nz + 4); o->kzU = dal(o->nz + 4);
    /* set_grid (src/ibm3d_setup.c:252-264) and assemble (:535-632). */
    for (int i = 0; i < o->nx; i++) { C1(o->dx, i) = c->xf[i + 1] - c->xf[i]; C1(o->xc, i) = (c->xf[i + 1] + c->xf[i]) / 2; }
    for (int j = 0; j < o->ny; j++) { C1(o->dy, j) = c->yf[j + 1] - c->yf[j]; C1(o->yc, j) = (c->yf[j + 1] + c->yf[j]) / 2; }
    for (int k = 0; k < o->nz; k++) { C1(o->dz, k) = c->zf[k + 1] - c->zf[k]; C1(o->zc, k) = (c->zf[k + 1] + c->zf[k]) / 2; }
    double *D[3] = {o->dx, o->dy, o->dz}, *Cc[3] = {o->xc, o->yc, o->zc};
    int Ns[3] = {o->nx, o->ny, o->nz}, lo[3] = {FW, FS, FD}, hi[3] = {FE, FN, FU};
    for (int a = 0; a < 3; a++) {
        double *d = D[a], *cc = Cc[a];
        int N = Ns[a], pl = isper(o->bct[lo[a]]), ph = isper(o->bct[hi[a]]);
        C1(d, -1) = pl ? C1(d, N - 1) : C1(d, 0);
        C1(d, -2) = pl ? C1(d, N - 2) : C1(d, 1);
        C1(d, N) = ph ? C1(d, 0) : C1(d, N - 1);
        C1(d, N + 1) = ph ? C1(d, 1) : C1(d, N - 2);
        C1(cc, -1) = C1(cc, 0) - (C1(d, -1) + C1(d, 0)) / 2;
        C1(cc, -2) = C1(cc, -1) - (C1(d, -2) + C1(d, -1)) / 2;
        C1(cc, N) = C1(cc, N - 1) + (C1(d, N - 1) + C1(d, N)) / 2;
        C1(cc, N + 1) = C1(cc, N) + (C1(d, N) + C1(d, N + 1)) / 2;
    }
    for (int i = 0; i < o->nx; i++) {
        C1(o->kxW, i) = o->dt / (2 * o->Re * (C1(o->xc, i) - C1(o->xc, i - 1)) * C1(o->dx, i));
        C1(o->kxE, i) = o->dt / (2 * o->Re * (C1(o->xc, i + 1) - C1(o->xc, i)) * C1(o->dx, i));
    }
    for (int j = 0; j < o->ny; j++) {
        C1(o->kyS, j) = o->dt / (2 * o->Re * (C1(o->yc, j) - C1(o->yc, j - 1)) * C1(o->dy, j));
        C1(o->kyN, j) = o->dt / (2 * o->Re * (C1(o->yc, j + 1) - C1(o->yc, j)) * C1(o->dy, j));
    }
    for (int k = 0; k < o->nz; k++) {
        C1(o->kzD, k) = o->dt / (2 * o->Re * (C1(o->zc, k) - C1(o->zc, k - 1)) * C1(o->dz, k));
        C1(o->kzU, k) = o->dt / (2 * o->Re * (C1(o->zc, k + 1) - C1(o->zc, k)) * C1(o->dz, k));
    }
    long n = o->nc;
    o->flag = (int *)calloc(n, sizeof(int));
    o->lvset = dal(n);
    o->coeffsum = dal(n);
    /* Level set and flags (src/ibm3d_setup.c:1081-1254). */
    if (c->lvset_in) {
        memcpy(o->lvset, c->lvset_in, sizeof(double) * n);
    } else if (c->stl_path) {
        Poly *P = read_stl(c->stl_path);
        CptGrid G = {o->nx + 4, o->ny + 4, o->nz + 4, o->xc, o->yc, o->zc, o->lvset};
        cpt(P, &G, 15);
        free_poly(P);
    } else {
        for (long q = 0; q < n; q++) o->lvset[q] = .5;
    }
    static const int adj[6][3] = {{0, 1, 0}, {1, 0, 0}, {0, -1, 0}, {-1, 0, 0}, {0, 0, -1}, {0, 0, 1}};
    for (int i = -2; i < o->nx + 2; i++)
        for (int j = -2; j < o->ny + 2; j++)
            for (int k = -2; k < o->nz + 2; k++) {
                if (!c->stl_path && !c->lvset_in) {
                    C3(o->flag, i, j, k) = FL;
                    continue;
                }
                if (C3(o->lvset, i, j, k) > 0) {
                    C3(o->flag, i, j, k) = FL;
                    continue;
                }
                int gh = 0;
                for (int l = 0; l < 6; l++) {
                    int ni = i + adj[l][0], nj = j + adj[l][1], nk = k + adj[l][2];
                    if (ni < -2 || ni >= o->nx + 2 || nj < -2 || nj >= o->ny + 2 || nk < -2 || nk >= o->nz + 2) continue;
                    gh = gh || C3(o->lvset, ni, nj, nk) > 0;
                }
                C3(o->flag, i, j, k) = gh ? GH : SO;
            }
    /* Ghost stencils in lexicographic order. */
    o->gid = (int *)malloc(sizeof(int) * n);
    for (long q = 0; q < n; q++) o->gid[q] = -1;
    o->ng = 0;
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++)
                if (C3(o->flag, i, j, k) == GH) o->ng++;
    o->gcell = malloc(sizeof(int) * (o->ng + 1));
    o->gidx = malloc(sizeof(int[8][3]) * (o->ng + 1));
    o->gco = malloc(sizeof(double[8]) * (o->ng + 1));
    int g = 0;
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (C3(o->flag, i, j, k) != GH) continue;
                o->gcell[g] = (int)CI(o, i, j, k);
                o->gid[CI(o, i, j, k)] = g;
                ghost_interp(o, i, j, k, o->gidx[g], o->gco[g]);
                g++;
            }
    /* p_coeffsum (src/ibm3d_setup.c:1641-1649). */
    for (int i = 0; i < o->nx; i++)
        for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < o->nz; k++) {
                if (o->singular && i == 0 && j == 0 && k == 0) continue;
                if (C3(o->flag, i, j, k) != FL) continue;
                double v0 = -(-C1(o->kyN, j)) - (-C1(o->kxE, i)) - (-C1(o->kyS, j)) - (-C1(o->kxW, i)) - (-C1(o->kzD, k)) - (-C1(o->kzU, k));
                C3(o->coeffsum, i, j, k) = v0;
            }
    for (int l = 0; l < 3; l++) {
        o->u[l] = dal(n); o->un[l] = dal(n); o->us[l] = dal(n); o->ut[l] = dal(n);
        o->U[l] = dal(n); o->Un[l] = dal(n); o->Us[l] = dal(n);
        o->N[l] = dal(n); o->Np[l] = dal(n);
    }
    for (int t = 0; t < 6; t++) o->tau[t] = dal(n);
    o->p = dal(n); o->pn = dal(n); o->pp = dal(n);
    o->b = dal(n); o->x = dal(n); o->r = dal(n); o->r0 = dal(n); o->pv = dal(n);
    o->v = dal(n); o->s = dal(n); o->t = dal(n); o->ph = dal(n); o->sh = dal(n);
    o->gtmp = dal(o->ng + 1);
    mg_setup(o);
    return o;
}

void oracle_init(Oracle *o, const double *u1, const double *u2, const double *u3, const double *p) {
    size_t b = sizeof(double) * o->nc;
    memcpy(o->u[0], u1, b);
    memcpy(o->u[1], u2, b);
    memcpy(o->u[2], u3, b);
    memcpy(o->p, p, b);
    o->iter = 0;
    o->time = 0;
}

int oracle_get(Oracle *o, const char *name, double *out) {
    const size_t b = sizeof(double) * o->nc;
    const size_t bu = sizeof(double) * (o->nx + 1) * (o->ny + 4) * (o->nz + 4);
    const size_t bv = sizeof(double) * (o->nx + 4) * (o->ny + 1) * (o->nz + 4);
    const size_t bw = sizeof(double) * (o->nx + 4) * (o->ny + 4) * (o->nz + 1);
    struct { const char *n; const double *a; size_t b; } t[] = {
        {"u1", o->u[0], b}, {"u2", o->u[1], b}, {"u3", o->u[2], b}, {"p", o->p, b},
        {"U1", o->U[0], bu}, {"U2", o->U[1], bv}, {"U3", o->U[2], bw},
        {"u1star", o->us[0], b}, {"u2star", o->us[1], b}, {"u3star", o->us[2], b},
        {"U1star", o->Us[0], bu}, {"U2star", o->Us[1], bv}, {"U3star", o->Us[2], bw},
        {"pprime", o->pp, b}, {"N1", o->Np[0], b}, {"N2", o->Np[1], b}, {"N3", o->Np[2], b},
        {"lvset", o->lvset, b}, {"coeffsum", o->coeffsum, b},
    };
    for (size_t q = 0; q < sizeof t / sizeof t[0]; q++)
        if (!strcmp(t[q].n, name)) {
            memcpy(out, t[q].a, t[q].b);
            return 0;
        }
    return -1;
}

void oracle_flag(Oracle *o, int *out) { memcpy(out, o->flag, sizeof(int) * o->nc); }

int oracle_num_ghost(Oracle *o) { return o->ng; }

void oracle_ghost_stencils(Oracle *o, int *ijk, int *idx, double *coeff) {
    for (int g = 0; g < o->ng; g++) {
        long P = o->gcell[g];
        ijk[3 * g] = (int)(P / o->sx) - 2;
        ijk[3 * g + 1] = (int)((P % o->sx) / o->sy) - 2;
        ijk[3 * g + 2] = (int)(P % o->sy) - 2;
        memcpy(&idx[24 * g], o->gidx[g], sizeof(int[8][3]));
        memcpy(&coeff[8 * g], o->gco[g], sizeof(double[8]));
    }
}

void oracle_stats(Oracle *o, int *iters, double *res, double *max_div) {
    for (int q = 0; q < 4; q++) {
        iters[q] = o->iters[q];
        res[q] = o->res[q];
    }
    *max_div = o->maxdiv;
}

void oracle_destroy(Oracle *o) {
    if (!o) return;
    free(o->dx); free(o->dy); free(o->dz); free(o->xc); free(o->yc); free(o->zc);
    free(o->kxW); free(o->kxE); free(o->kyS); free(o->kyN); free(o->kzD); free(o->kzU);
    free(o->flag); free(o->lvset); free(o->coeffsum); free(o->gid); free(o->gcell); free(o->gidx); free(o->gco);
    for (int l = 0; l < 3; l++) {
        free(o->u[l]); free(o->un[l]); free(o->us[l]); free(o->ut[l]); free(o->U[l]); free(o->Un[l]);
        free(o->Us[l]); free(o->N[l]); free(o->Np[l]);
    }
    for (int t = 0; t < 6; t++) free(o->tau[t]);
    free(o->p); free(o->pn); free(o->pp); free(o->b); free(o->x); free(o->r); free(o->r0); free(o->pv);
    free(o->v); free(o->s); free(o->t); free(o->ph); free(o->sh);
    for (int l = 0; l < o->nlev; l++) {
        Level *L = &o->lev[l];
        free(L->tx); free(L->ty); free(L->tz); free(L->gx); free(L->gy); free(L->gz); free(L->diag); free(L->r); free(L->z);
    }
    free(o->gtmp);
    free(o);
}
