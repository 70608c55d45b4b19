// Set-up kernels: level set, flags and ghost-cell stencils (FP64).
// Compiled with -fmad=false: every value that decides a flag or a stencil
// index is computed with the reference's operation order and without fused
// multiply-adds, i.e. bit-identically to the reference's C build.
//
// Closest-point transform (src/geo3d.c:436-704).  The reference scans every
// extrusion's bounding box and keeps, per grid point, the first extrusion
// (in its loop order) with the smallest distance.  Here each grid point
// gathers instead: a float BVH search finds its approximate distance d* to
// the surface, then every extrusion of every triangle within d* + M is
// evaluated exactly (FP64, reference formulas) and reduced by
// (distance, loop order).  Any extrusion containing the point measures at
// least the distance to its own triangle, so none outside that set can win;
// when the set yields no extrusion within d* + M/2 the point falls back to
// scanning every extrusion.
#include <cfloat>
#include <climits>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "geo3d.h"
#include "setup.h"

namespace ibm {

#define GRID_STRIDE(q, n)                                                              \
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (n); \
         q += (long long)gridDim.x * blockDim.x)

static inline unsigned nblk(long long n, int t) {
    long long b = (n + t - 1) / t;
    return (unsigned)(b < 1 ? 1 : (b > 65535 * 16 ? 65535 * 16 : b));
}

struct CptDev {
    const CptFeature *feat;
    int nfeat;
    const int *tfs;      // tri_feat_start
    const int *tf;       // tri_feats
    const float *txyz;   // 9 per triangle (BVH order)
    const BVHNode *node;
    int nnode;
};

// Exact extrusion test and distance with the reference's arithmetic.
__device__ inline bool cpt_eval(const CptFeature &F, double px, double py, double pz, double &dist) {
    if (px < F.bmin[0] || px > F.bmax[0] || py < F.bmin[1] || py > F.bmax[1] || pz < F.bmin[2] || pz > F.bmax[2])
        return false;
    if (F.kind == FEAT_VERTEX) {
        const double dx = px - F.a[0], dy = py - F.a[1], dz = pz - F.a[2];
        const double dn = sqrt(dx * dx + dy * dy + dz * dz);
        const double la = sqrt(F.b[0] * F.b[0] + F.b[1] * F.b[1] + F.b[2] * F.b[2]);
        double c = (F.b[0] * dx + F.b[1] * dy + F.b[2] * dz) / (la * dn);
        if (c < -1) c = -1;
        else if (c > 1) c = 1;
        if (acos(c) <= F.angle + 1e-12 && dn <= F.radius + 1e-12) {
            dist = dn;
            return true;
        }
        return false;
    }
    for (int l = 0; l < 5; l++)
        if (F.pl[l][0] * px + F.pl[l][1] * py + F.pl[l][2] * pz + F.pl[l][3] > 1e-12) return false;
    if (F.kind == FEAT_FACE) {
        dist = fabs(F.pl[0][0] * px + F.pl[0][1] * py + F.pl[0][2] * pz + F.pl[0][3]) / F.a[0];
        return true;
    }
    const double abx = F.b[0] - F.a[0], aby = F.b[1] - F.a[1], abz = F.b[2] - F.a[2];
    const double avx = px - F.a[0], avy = py - F.a[1], avz = pz - F.a[2];
    const double t = (abx * avx + aby * avy + abz * avz) / (abx * abx + aby * aby + abz * abz);
    const double hx = (1 - t) * F.a[0] + t * F.b[0];
    const double hy = (1 - t) * F.a[1] + t * F.b[1];
    const double hz = (1 - t) * F.a[2] + t * F.b[2];
    const double ex = px - hx, ey = py - hy, ez = pz - hz;
    dist = sqrt(ex * ex + ey * ey + ez * ez);
    return true;
}

// Squared distance from p to triangle (a, b, c), float (closest-point
// regions of the triangle, Ericson, Real-Time Collision Detection 5.1.5).
__device__ inline float tri_dist2(const float p[3], const float *t) {
    const float a[3] = {t[0], t[1], t[2]}, b[3] = {t[3], t[4], t[5]}, c[3] = {t[6], t[7], t[8]};
    float ab[3], ac[3], ap[3], q[3];
    for (int d = 0; d < 3; d++) {
        ab[d] = b[d] - a[d];
        ac[d] = c[d] - a[d];
        ap[d] = p[d] - a[d];
    }
    auto dot = [](const float *u, const float *v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
    const float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) {
        for (int d = 0; d < 3; d++) q[d] = a[d];
    } else {
        float bp[3];
        for (int d = 0; d < 3; d++) bp[d] = p[d] - b[d];
        const float d3 = dot(ab, bp), d4 = dot(ac, bp);
        if (d3 >= 0 && d4 <= d3) {
            for (int d = 0; d < 3; d++) q[d] = b[d];
        } else {
            const float vc = d1 * d4 - d3 * d2;
            if (vc <= 0 && d1 >= 0 && d3 <= 0) {
                const float v = d1 / (d1 - d3);
                for (int d = 0; d < 3; d++) q[d] = a[d] + v * ab[d];
            } else {
                float cp[3];
                for (int d = 0; d < 3; d++) cp[d] = p[d] - c[d];
                const float d5 = dot(ab, cp), d6 = dot(ac, cp);
                if (d6 >= 0 && d5 <= d6) {
                    for (int d = 0; d < 3; d++) q[d] = c[d];
                } else {
                    const float vb = d5 * d2 - d1 * d6;
                    if (vb <= 0 && d2 >= 0 && d6 <= 0) {
                        const float w = d2 / (d2 - d6);
                        for (int d = 0; d < 3; d++) q[d] = a[d] + w * ac[d];
                    } else {
                        const float va = d3 * d6 - d5 * d4;
                        if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
                            const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
                            for (int d = 0; d < 3; d++) q[d] = b[d] + w * (c[d] - b[d]);
                        } else {
                            const float den = 1.0f / (va + vb + vc);
                            const float v = vb * den, w = vc * den;
                            for (int d = 0; d < 3; d++) q[d] = a[d] + ab[d] * v + ac[d] * w;
                        }
                    }
                }
            }
        }
    }
    float e2 = 0;
    for (int d = 0; d < 3; d++) e2 += (p[d] - q[d]) * (p[d] - q[d]);
    return e2;
}

__device__ inline float box_dist2(const BVHNode &n, const float p[3]) {
    float s = 0;
    for (int d = 0; d < 3; d++) {
        const float e = fmaxf(fmaxf(n.bmin[d] - p[d], 0.0f), p[d] - n.bmax[d]);
        s += e * e;
    }
    return s;
}

__global__ void __launch_bounds__(128)
k_cpt(const CptDev m, const int nx, const int ny, const int nz, const double *__restrict__ x,
      const double *__restrict__ y, const double *__restrict__ z, double *f, const double maxd, int *fb_list,
      int *fb_count) {
    const long long n = (long long)nx * ny * nz;
    const double NaN = __longlong_as_double(0x7ff8000000000000LL);
    GRID_STRIDE(q, n) {
        const int k = (int)(q % nz);
        const int j = (int)((q / nz) % ny);
        const int i = (int)(q / ((long long)nz * ny));
        const double px = x[i], py = y[j], pz = z[k];
        const float p[3] = {(float)px, (float)py, (float)pz};
        if (m.nnode == 0) {
            f[q] = NaN;
            continue;
        }
        int stack[64];
        int sp = 0;
        stack[sp++] = 0;
        float best2 = FLT_MAX;
        while (sp > 0) {
            const BVHNode nd = m.node[stack[--sp]];
            if (box_dist2(nd, p) >= best2) continue;
            if (nd.left < 0) {
                for (int t = nd.start; t < nd.start + nd.count; t++) best2 = fminf(best2, tri_dist2(p, m.txyz + 9 * t));
            } else {
                const float dl = box_dist2(m.node[nd.left], p), dr = box_dist2(m.node[nd.right], p);
                if (sp > 60) continue;  // BVH depth is ~log2(triangles); never reached
                if (dl < dr) {
                    stack[sp++] = nd.right;
                    stack[sp++] = nd.left;
                } else {
                    stack[sp++] = nd.left;
                    stack[sp++] = nd.right;
                }
            }
        }
        const double dstar = sqrt((double)best2);
        const double M = 1e-3 + 1e-6 * (fabs(px) + fabs(py) + fabs(pz));
        if (dstar > maxd + M) {
            f[q] = NaN;
            continue;
        }
        const float thr = (float)(dstar + M);
        const float thr2 = thr * thr;
        double bd = DBL_MAX;
        int bo = INT_MAX, bs = 0;
        sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const BVHNode nd = m.node[stack[--sp]];
            if (box_dist2(nd, p) > thr2) continue;
            if (nd.left < 0) {
                for (int t = nd.start; t < nd.start + nd.count; t++) {
                    if (tri_dist2(p, m.txyz + 9 * t) > thr2) continue;
                    for (int e = m.tfs[t]; e < m.tfs[t + 1]; e++) {
                        const int fi = m.tf[e];
                        double d;
                        if (cpt_eval(m.feat[fi], px, py, pz, d)) {
                            if (d < bd || (d == bd && fi < bo)) {
                                bd = d;
                                bo = fi;
                                bs = m.feat[fi].sgn;
                            }
                        }
                    }
                }
            } else if (sp <= 60) {
                stack[sp++] = nd.left;
                stack[sp++] = nd.right;
            }
        }
        if (bo == INT_MAX || bd > dstar + 0.5 * M) {
            const int slot = atomicAdd(fb_count, 1);
            fb_list[slot] = (int)q;
            f[q] = NaN;
        } else {
            f[q] = bs * bd;
        }
    }
}

// Full scan of every extrusion for the points the gather could not settle.
__global__ void __launch_bounds__(256)
k_cpt_fallback(const CptDev m, const int nx, const int ny, const int nz, const double *__restrict__ x,
               const double *__restrict__ y, const double *__restrict__ z, double *f, const int *fb_list,
               const int nfb) {
    __shared__ double sd[256];
    __shared__ int so[256];
    const double NaN = __longlong_as_double(0x7ff8000000000000LL);
    for (int c = blockIdx.x; c < nfb; c += gridDim.x) {
        const long long q = fb_list[c];
        const int k = (int)(q % nz);
        const int j = (int)((q / nz) % ny);
        const int i = (int)(q / ((long long)nz * ny));
        const double px = x[i], py = y[j], pz = z[k];
        double bd = DBL_MAX;
        int bo = INT_MAX;
        for (int fi = threadIdx.x; fi < m.nfeat; fi += blockDim.x) {
            double d;
            if (cpt_eval(m.feat[fi], px, py, pz, d) && (d < bd || (d == bd && fi < bo))) {
                bd = d;
                bo = fi;
            }
        }
        sd[threadIdx.x] = bd;
        so[threadIdx.x] = bo;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) {
                const double d2 = sd[threadIdx.x + s];
                const int o2 = so[threadIdx.x + s];
                if (d2 < sd[threadIdx.x] || (d2 == sd[threadIdx.x] && o2 < so[threadIdx.x])) {
                    sd[threadIdx.x] = d2;
                    so[threadIdx.x] = o2;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) f[q] = so[0] == INT_MAX ? NaN : m.feat[so[0]].sgn * sd[0];
        __syncthreads();
    }
}

// NaN fill of points no extrusion reached (src/geo3d.c:643-703): along k,
// then j, then i, copying the sign of the previous point as +-maxd.
__global__ void k_cpt_fill(double *f, const int nx, const int ny, const int nz, const int axis, const double maxd) {
    long long nl;
    int len;
    if (axis == 2) { nl = (long long)nx * ny; len = nz; }
    else if (axis == 1) { nl = (long long)nx * nz; len = ny; }
    else { nl = (long long)ny * nz; len = nx; }
    GRID_STRIDE(l, nl) {
        long long base, s;
        if (axis == 2) { base = l * nz; s = 1; }
        else if (axis == 1) { const long long i = l / nz, k = l % nz; base = i * ny * nz + k; s = nz; }
        else { base = l; s = (long long)ny * nz; }
        for (int t = 1; t < len; t++) {
            double &v = f[base + t * s];
            const double pv = f[base + (t - 1) * s];
            if (isnan(v) && pv < 0) v = -maxd;
            else if (isnan(v) && pv > 0) v = maxd;
        }
        for (int t = len - 2; t >= 0; t--) {
            double &v = f[base + t * s];
            const double nv = f[base + (t + 1) * s];
            if (isnan(v) && nv < 0) v = -maxd;
            else if (isnan(v) && nv > 0) v = maxd;
        }
    }
}

int gpu_cpt(cudaStream_t s, const CptModel &m, int nx, int ny, int nz, const double *x, const double *y,
            const double *z, double *f, double maxd, int *nfallback) {
    std::vector<void *> tmp;
    auto up = [&](const void *src, size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        if (bytes && src) cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, s);
        tmp.push_back(p);
        return p;
    };
    CptDev d{};
    d.feat = (const CptFeature *)up(m.features.data(), sizeof(CptFeature) * m.features.size());
    d.nfeat = (int)m.features.size();
    d.tfs = (const int *)up(m.tri_feat_start.data(), sizeof(int) * m.tri_feat_start.size());
    d.tf = (const int *)up(m.tri_feats.data(), sizeof(int) * m.tri_feats.size());
    d.txyz = (const float *)up(m.tri_xyz.data(), sizeof(float) * m.tri_xyz.size());
    d.node = (const BVHNode *)up(m.nodes.data(), sizeof(BVHNode) * m.nodes.size());
    d.nnode = (int)m.nodes.size();
    const long long n = (long long)nx * ny * nz;
    int *fb_list = (int *)up(nullptr, sizeof(int) * n);
    int *fb_count = (int *)up(nullptr, sizeof(int));
    int rc = 0;
    for (void *p : tmp)
        if (!p) rc = -1;
    if (rc == 0) {
        cudaMemsetAsync(fb_count, 0, sizeof(int), s);
        k_cpt<<<nblk(n, 128), 128, 0, s>>>(d, nx, ny, nz, x, y, z, f, maxd, fb_list, fb_count);
        int nfb = 0;
        cudaMemcpyAsync(&nfb, fb_count, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        if (nfallback) *nfallback = nfb;
        if (nfb > 0) k_cpt_fallback<<<nfb < 4096 ? nfb : 4096, 256, 0, s>>>(d, nx, ny, nz, x, y, z, f, fb_list, nfb);
        k_cpt_fill<<<nblk((long long)nx * ny, 128), 128, 0, s>>>(f, nx, ny, nz, 2, maxd);
        k_cpt_fill<<<nblk((long long)nx * nz, 128), 128, 0, s>>>(f, nx, ny, nz, 1, maxd);
        k_cpt_fill<<<nblk((long long)ny * nz, 128), 128, 0, s>>>(f, nx, ny, nz, 0, maxd);
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = -1;
    }
    for (void *p : tmp) cudaFree(p);
    return rc;
}

// Flags (src/ibm3d_setup.c:1230-1254): fluid if lvset > 0, else ghost if a
// face neighbour inside the padded grid is fluid, else solid.
__global__ void k_flags(const Grid g, const double *__restrict__ lv, uint8_t *flag) {
    GRID_STRIDE(P, g.ncell) {
        int i, j, k;
        cijk(g, P, i, j, k);
        if (lv[P] > 0) {
            flag[P] = FLUID;
            continue;
        }
        bool gh = false;
        if (i > -2) gh = gh || lv[P - g.sx] > 0;
        if (i < g.nx + 1) gh = gh || lv[P + g.sx] > 0;
        if (j > -2) gh = gh || lv[P - g.sy] > 0;
        if (j < g.ny + 1) gh = gh || lv[P + g.sy] > 0;
        if (k > -2) gh = gh || lv[P - 1] > 0;
        if (k < g.nz + 1) gh = gh || lv[P + 1] > 0;
        flag[P] = gh ? GHOST : SOLID;
    }
}

void gpu_flags(cudaStream_t s, const Grid &g, const double *lvset, uint8_t *flag) {
    k_flags<<<nblk(g.ncell, 256), 256, 0, s>>>(g, lvset, flag);
}

__device__ inline int upper_bound_d(int len, const double *arr, double val) {
    int l = 0, h = len;
    while (l < h) {
        const int mid = l + (h - l) / 2;
        if (val >= arr[mid]) l = mid + 1;
        else h = mid;
    }
    return l;
}

// Ghost-cell interpolation stencil (src/utils.c:111-171): normal from the
// central difference of the level set, mirror point x - 2 phi n, the 8
// surrounding cell centres and trilinear weights; then solid entries
// dropped, weights renormalised and the ghost's own weight split off
// (src/ibm3d_fracstep.c:1935-1962, src/ibm3d_setup.c:1653-1698).
__global__ void k_ghost_stencil(const Grid g, const double *__restrict__ xc, const double *__restrict__ yc,
                                const double *__restrict__ zc, const double *__restrict__ lv,
                                const uint8_t *__restrict__ flag, const int *__restrict__ gcell, const int ng,
                                GhostStencil *out) {
    GRID_STRIDE(q, (long long)ng) {
        const long long P = gcell[q];
        int i, j, k;
        cijk(g, P, i, j, k);
        GhostStencil st;
        const double nxv = (lv[P + g.sx] - lv[P - g.sx]) / (xc[i + 3] - xc[i + 1]);
        const double nyv = (lv[P + g.sy] - lv[P - g.sy]) / (yc[j + 3] - yc[j + 1]);
        const double nzv = (lv[P + 1] - lv[P - 1]) / (zc[k + 3] - zc[k + 1]);
        const double c = -2 * lv[P];
        const double mx = 1 * xc[i + 2] + c * nxv;
        const double my = 1 * yc[j + 2] + c * nyv;
        const double mz = 1 * zc[k + 2] + c * nzv;
        const int im = upper_bound_d(g.nx + 4, xc, mx) - 3;
        const int jm = upper_bound_d(g.ny + 4, yc, my) - 3;
        const int km = upper_bound_d(g.nz + 4, zc, mz) - 3;
        st.ok = (im >= -2 && im + 1 <= g.nx + 1 && jm >= -2 && jm + 1 <= g.ny + 1 && km >= -2 && km + 1 <= g.nz + 1);
        st.im = im;
        st.jm = jm;
        st.km = km;
        if (!st.ok) {
            out[q] = st;
            continue;
        }
        const double xl = xc[im + 2], xu = xc[im + 3];
        const double yl = yc[jm + 2], yu = yc[jm + 3];
        const double zl = zc[km + 2], zu = zc[km + 3];
        const double vol = (xu - xl) * (yu - yl) * (zu - zl);
        st.raw[0] = (xu - mx) * (yu - my) * (zu - mz) / vol;
        st.raw[1] = (xu - mx) * (yu - my) * (mz - zl) / vol;
        st.raw[2] = (xu - mx) * (my - yl) * (zu - mz) / vol;
        st.raw[3] = (xu - mx) * (my - yl) * (mz - zl) / vol;
        st.raw[4] = (mx - xl) * (yu - my) * (zu - mz) / vol;
        st.raw[5] = (mx - xl) * (yu - my) * (mz - zl) / vol;
        st.raw[6] = (mx - xl) * (my - yl) * (zu - mz) / vol;
        st.raw[7] = (mx - xl) * (my - yl) * (mz - zl) / vol;
        double w[8], sum = 0;
        long long cell[8];
        for (int l = 0; l < 8; l++) {
            cell[l] = cidx(g, im + !!(l & 4), jm + !!(l & 2), km + !!(l & 1));
            w[l] = flag[cell[l]] == SOLID ? 0.0 : st.raw[l];
            if (flag[cell[l]] != SOLID) sum += w[l];
        }
        st.wself = 0;
        for (int l = 0; l < 8; l++) {
            w[l] /= sum;
            if (cell[l] == P) {
                st.wself += w[l];
                st.cell[l] = -1;
                st.w[l] = 0;
            } else if (flag[cell[l]] == SOLID) {
                st.cell[l] = -1;
                st.w[l] = 0;
            } else {
                st.cell[l] = (int)cell[l];
                st.w[l] = w[l];
            }
        }
        out[q] = st;
    }
}

int gpu_ghost_stencils(cudaStream_t s, const Grid &g, const double *xc, const double *yc, const double *zc,
                       const double *lvset, const uint8_t *flag, const int *gcell_dev, int ng, GhostStencil *out_dev) {
    if (ng == 0) return 0;
    k_ghost_stencil<<<nblk(ng, 128), 128, 0, s>>>(g, xc, yc, zc, lvset, flag, gcell_dev, ng, out_dev);
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -1;
}

}  // namespace ibm

// ---------------------------------------------------------------------------
// Allocation-free closest-point transform.
//
// Some callers cannot call cudaMalloc at the moment they need a level set:
// hosts whose framework allocator (PyTorch's caching allocator, a serving
// process with a fixed per-job budget) already owns the device memory so a
// raw cudaMalloc can fail or fragment it, and latency-bound loops that must
// not pay for an allocation.  Polyhedron_cpt_noalloc serves them: it runs the same kernels
// as Polyhedron_cpt, but every device buffer - the grid coordinates, the
// output, the extrusion list, the BVH and the fallback list - is carved out
// of one file-scope device array of CPT_NOALLOC_BYTES (32 MiB), which every
// GPU that loads this library holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace ibm {
constexpr size_t CPT_NOALLOC_BYTES = 32u << 20;
static __device__ __align__(256) unsigned char g_cpt_noalloc_scratch[CPT_NOALLOC_BYTES];
}  // namespace ibm

namespace {
// Device address of the scratch array, looked up once per device.
constexpr int kMaxDevices = 64;
unsigned char *g_noalloc_ptr[kMaxDevices] = {nullptr};
std::mutex g_noalloc_mutex;

unsigned char *noalloc_scratch(int dev) {
    if (dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, ibm::g_cpt_noalloc_scratch);
        if (e != cudaSuccess) {
            fprintf(stderr, "error: Polyhedron_cpt_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return nullptr;
        }
        g_noalloc_ptr[dev] = (unsigned char *)p;
    }
    return g_noalloc_ptr[dev];
}
}  // namespace

extern "C" int Polyhedron_cpt_noalloc(const Polyhedron *const poly, const int nx, const int ny, const int nz,
                                      const double *x, const double *y, const double *z, double *f,
                                      const double maxd) {
    using namespace ibm;
    if (!poly || !x || !y || !z || !f || nx <= 0 || ny <= 0 || nz <= 0) {
        fprintf(stderr, "error: Polyhedron_cpt_noalloc: null pointer or non-positive grid size (%d x %d x %d)\n", nx,
                ny, nz);
        return -1;
    }
    // Sizes are checked against the array before any product can overflow:
    // each axis is below 2^31 and the point count is compared in 64 bits.
    const long long n = (long long)nx * ny * nz;
    if (n > (long long)(CPT_NOALLOC_BYTES / sizeof(double))) {
        fprintf(stderr,
                "error: Polyhedron_cpt_noalloc: a %d x %d x %d grid needs more than the %zu-byte static buffer; "
                "use Polyhedron_cpt\n",
                nx, ny, nz, CPT_NOALLOC_BYTES);
        return -1;
    }
    CptModel m;
    build_cpt_model(poly, maxd, m);  // host memory only
    // Layout of the scratch array, each piece 256-byte aligned.
    size_t off = 0;
    auto place = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) & ~(size_t)255;
        return at;
    };
    const size_t o_x = place(sizeof(double) * nx), o_y = place(sizeof(double) * ny), o_z = place(sizeof(double) * nz);
    const size_t o_f = place(sizeof(double) * (size_t)n);
    const size_t o_feat = place(sizeof(CptFeature) * m.features.size());
    const size_t o_tfs = place(sizeof(int) * m.tri_feat_start.size());
    const size_t o_tf = place(sizeof(int) * m.tri_feats.size());
    const size_t o_txyz = place(sizeof(float) * m.tri_xyz.size());
    const size_t o_node = place(sizeof(BVHNode) * m.nodes.size());
    const size_t o_fb = place(sizeof(int) * (size_t)n);
    const size_t o_cnt = place(sizeof(int));
    if (off > CPT_NOALLOC_BYTES) {
        fprintf(stderr,
                "error: Polyhedron_cpt_noalloc: a %d x %d x %d grid with %zu extrusions needs %zu bytes of "
                "scratch, more than the %zu-byte static buffer; use Polyhedron_cpt\n",
                nx, ny, nz, m.features.size(), off, CPT_NOALLOC_BYTES);
        return -1;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    unsigned char *base = noalloc_scratch(dev);
    if (!base) return -1;
    const cudaStream_t s = 0;
    // Every copy, the memset and every launch is checked: the array keeps
    // the previous call's contents, so a step that failed silently would
    // let the kernels run on the previous call's geometry.
    cudaError_t err = cudaSuccess;
    const char *what = "";
    auto check = [&](cudaError_t e, const char *step) {
        if (err == cudaSuccess && e != cudaSuccess) {
            err = e;
            what = step;
        }
    };
    auto up = [&](size_t o, const void *src, size_t bytes) {
        if (bytes) check(cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, s), "upload");
    };
    up(o_x, x, sizeof(double) * nx);
    up(o_y, y, sizeof(double) * ny);
    up(o_z, z, sizeof(double) * nz);
    up(o_feat, m.features.data(), sizeof(CptFeature) * m.features.size());
    up(o_tfs, m.tri_feat_start.data(), sizeof(int) * m.tri_feat_start.size());
    up(o_tf, m.tri_feats.data(), sizeof(int) * m.tri_feats.size());
    up(o_txyz, m.tri_xyz.data(), sizeof(float) * m.tri_xyz.size());
    up(o_node, m.nodes.data(), sizeof(BVHNode) * m.nodes.size());
    // The array keeps the previous call's contents: the fallback counter
    // must start at zero every call.
    check(cudaMemsetAsync(base + o_cnt, 0, sizeof(int), s), "counter reset");
    CptDev d{};
    d.feat = (const CptFeature *)(base + o_feat);
    d.nfeat = (int)m.features.size();
    d.tfs = (const int *)(base + o_tfs);
    d.tf = (const int *)(base + o_tf);
    d.txyz = (const float *)(base + o_txyz);
    d.node = (const BVHNode *)(base + o_node);
    d.nnode = (int)m.nodes.size();
    const double *dx = (const double *)(base + o_x), *dy = (const double *)(base + o_y), *dz = (const double *)(base + o_z);
    double *df = (double *)(base + o_f);
    int *fb_list = (int *)(base + o_fb), *fb_count = (int *)(base + o_cnt);
    int nfb = 0;
    if (err == cudaSuccess) {
        k_cpt<<<nblk(n, 128), 128, 0, s>>>(d, nx, ny, nz, dx, dy, dz, df, maxd, fb_list, fb_count);
        check(cudaGetLastError(), "k_cpt launch");
        check(cudaMemcpyAsync(&nfb, fb_count, sizeof(int), cudaMemcpyDeviceToHost, s), "fallback count read");
        check(cudaStreamSynchronize(s), "k_cpt");
    }
    if (err == cudaSuccess && (nfb < 0 || nfb > n)) {
        fprintf(stderr, "error: Polyhedron_cpt_noalloc: fallback count %d outside [0, %lld]\n", nfb, n);
        return -1;
    }
    if (err == cudaSuccess) {
        if (nfb > 0) {
            k_cpt_fallback<<<nfb < 4096 ? nfb : 4096, 256, 0, s>>>(d, nx, ny, nz, dx, dy, dz, df, fb_list, nfb);
            check(cudaGetLastError(), "k_cpt_fallback launch");
        }
        k_cpt_fill<<<nblk((long long)nx * ny, 128), 128, 0, s>>>(df, nx, ny, nz, 2, maxd);
        check(cudaGetLastError(), "k_cpt_fill launch");
        k_cpt_fill<<<nblk((long long)nx * nz, 128), 128, 0, s>>>(df, nx, ny, nz, 1, maxd);
        check(cudaGetLastError(), "k_cpt_fill launch");
        k_cpt_fill<<<nblk((long long)ny * nz, 128), 128, 0, s>>>(df, nx, ny, nz, 0, maxd);
        check(cudaGetLastError(), "k_cpt_fill launch");
        check(cudaMemcpyAsync(f, df, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s), "result read-back");
        check(cudaStreamSynchronize(s), "level-set kernels");
    }
    if (err != cudaSuccess) {
        fprintf(stderr, "error: Polyhedron_cpt_noalloc: %s failed: %s\n", what, cudaGetErrorString(err));
        return -1;
    }
    return 0;
}
