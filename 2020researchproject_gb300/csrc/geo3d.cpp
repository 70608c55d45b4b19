// Polyhedron topology and closest-point-transform feature list (host).
//
// Polyhedron_read_stl follows src/geo3d.c:229-401: vertices are merged by
// exact coordinate equality and numbered in first-seen order, edges are
// unordered vertex pairs numbered in first-seen order (face_idx[0] = first
// face, face_idx[1] = last later face), and each vertex's faces are ordered
// by walking around it.  The file's facet normals are used as given.
//
// build_cpt_model lists the extrusions of Polyhedron_cpt
// (src/geo3d.c:436-641) in the reference's order - per face an outward and
// an inward prism, per edge one to three wedges, per vertex an outward
// and/or inward cone - with the same bounding planes and bounding boxes,
// so that the GPU can evaluate exactly the reference's candidate set for a
// cell.  The vector helpers keep the reference's operation order so that
// every derived coordinate is bit-identical (build with -ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>

#include "geo3d.h"

extern "C" {

Vector Vector_add(const Vector a, const Vector b) { return Vector{a.x + b.x, a.y + b.y, a.z + b.z}; }
Vector Vector_sub(const Vector a, const Vector b) { return Vector{a.x - b.x, a.y - b.y, a.z - b.z}; }
double Vector_dot(const Vector a, const Vector b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
Vector Vector_crs(const Vector a, const Vector b) {
    return Vector{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
double Vector_norm(const Vector v) { return std::sqrt(Vector_dot(v, v)); }
double Vector_dist(const Vector a, const Vector b) { return Vector_norm(Vector_sub(a, b)); }
double Vector_angle(const Vector a, const Vector b) {
    const double la = Vector_norm(a), lb = Vector_norm(b);
    double c = Vector_dot(a, b) / (la * lb);
    if (c < -1) c = -1;
    else if (c > 1) c = 1;
    return std::acos(c);
}
Vector Vector_normalize(const Vector v) {
    const double len = Vector_norm(v);
    return Vector{v.x / len, v.y / len, v.z / len};
}
Vector Vector_lincom(const double a, const Vector u, const double b, const Vector v) {
    return Vector{a * u.x + b * v.x, a * u.y + b * v.y, a * u.z + b * v.z};
}
// Rodrigues rotation of v about axis by angle (the matrix form the reference
// uses, src/geo3d.c:180-194, evaluated term by term in the same order).
Vector Vector_rot(const Vector v, const Vector axis, const double angle) {
    const Vector n = Vector_normalize(axis);
    const double c = std::cos(angle), s = std::sin(angle);
    Vector r;
    r.x = (c + n.x * n.x * (1 - c)) * v.x + (n.x * n.y * (1 - c) - n.z * s) * v.y + (n.x * n.z * (1 - c) + n.y * s) * v.z;
    r.y = (n.x * n.y * (1 - c) + n.z * s) * v.x + (c + n.y * n.y * (1 - c)) * v.y + (n.y * n.z * (1 - c) - n.x * s) * v.z;
    r.z = (n.x * n.z * (1 - c) - n.y * s) * v.x + (n.y * n.z * (1 - c) + n.x * s) * v.y + (c + n.z * n.z * (1 - c)) * v.z;
    return r;
}

Polyhedron *Polyhedron_new(void) { return new _polyhedron(); }

void Polyhedron_destroy(Polyhedron *poly) { delete poly; }

void Polyhedron_read_stl(Polyhedron *poly, FILE *f) {
    char header[80];
    uint32_t nf = 0;
    if (fread(header, 1, 80, f) != 80 || fread(&nf, 4, 1, f) != 1) {
        fprintf(stderr, "error: cannot read STL header\n");
        std::abort();
    }
    poly->faces.assign(nf, FaceRec{});
    struct VKey {
        double x, y, z;
        bool operator<(const VKey &o) const {
            if (x != o.x) return x < o.x;
            if (y != o.y) return y < o.y;
            if (z != o.z) return z < o.z;
            return false;
        }
    };
    struct VVal {
        int idx, nfaces, first_face;
    };
    std::map<VKey, VVal> vmap;
    std::vector<Vector> vcoord;
    for (uint32_t i = 0; i < nf; i++) {
        float rec[12];
        uint16_t attr;
        if (fread(rec, 4, 12, f) != 12 || fread(&attr, 2, 1, f) != 1) {
            fprintf(stderr, "error: truncated STL file\n");
            std::abort();
        }
        poly->faces[i].n = Vector{rec[0], rec[1], rec[2]};
        for (int j = 0; j < 3; j++) {
            VKey key{rec[3 + 3 * j], rec[4 + 3 * j], rec[5 + 3 * j]};
            auto it = vmap.find(key);
            if (it == vmap.end()) {
                it = vmap.emplace(key, VVal{(int)vmap.size(), 0, (int)i}).first;
                vcoord.push_back(Vector{key.x, key.y, key.z});
            }
            poly->faces[i].vertex_idx[j] = it->second.idx;
            it->second.nfaces++;
        }
    }
    poly->vertices.assign(vmap.size(), VertexRec{});
    for (auto &kv : vmap) {
        VertexRec &v = poly->vertices[kv.second.idx];
        v.coord = Vector{kv.first.x, kv.first.y, kv.first.z};
        v.num_faces = kv.second.nfaces;
        v.face_idx.assign(v.num_faces, -1);
        v.face_idx[0] = kv.second.first_face;
    }
    // Edges keyed by the unordered vertex pair, numbered in first-seen order.
    std::map<std::pair<int, int>, int> emap;
    for (uint32_t i = 0; i < nf; i++) {
        for (int j = 0; j < 3; j++) {
            const int a = poly->faces[i].vertex_idx[j], b = poly->faces[i].vertex_idx[(j + 1) % 3];
            const std::pair<int, int> key(std::min(a, b), std::max(a, b));
            auto it = emap.find(key);
            if (it == emap.end()) {
                it = emap.emplace(key, (int)poly->edges.size()).first;
                EdgeRec e;
                e.vertex_idx[0] = a;
                e.vertex_idx[1] = b;
                e.face_idx[0] = (int)i;
                e.face_idx[1] = -1;
                poly->edges.push_back(e);
            } else {
                poly->edges[it->second].face_idx[1] = (int)i;
            }
            poly->faces[i].edge_idx[j] = it->second;
        }
    }
    // Faces around each vertex, walking across the edge that precedes the
    // vertex in the current face.
    for (int v = 0; v < (int)poly->vertices.size(); v++) {
        VertexRec &vr = poly->vertices[v];
        int cur = vr.face_idx[0];
        for (int j = 1; j < vr.num_faces; j++) {
            const FaceRec &fc = poly->faces[cur];
            int e;
            if (fc.vertex_idx[0] == v) e = fc.edge_idx[2];
            else if (fc.vertex_idx[1] == v) e = fc.edge_idx[0];
            else e = fc.edge_idx[1];
            cur = poly->edges[e].face_idx[0] == cur ? poly->edges[e].face_idx[1] : poly->edges[e].face_idx[0];
            if (cur < 0) {
                fprintf(stderr, "error: polyhedron is not a closed 2-manifold (open edge %d)\n", e);
                std::abort();
            }
            vr.face_idx[j] = cur;
        }
    }
}

void Polyhedron_print_stats(Polyhedron *poly) {
    double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY, zmin = INFINITY, zmax = -INFINITY;
    printf("Input polyhedron size: %zu faces, %zu edges, %zu vertices\n", poly->faces.size(), poly->edges.size(),
           poly->vertices.size());
    for (auto &v : poly->vertices) {
        xmin = std::min(xmin, v.coord.x); xmax = std::max(xmax, v.coord.x);
        ymin = std::min(ymin, v.coord.y); ymax = std::max(ymax, v.coord.y);
        zmin = std::min(zmin, v.coord.z); zmax = std::max(zmax, v.coord.z);
    }
    printf("  xmin: %10.4lf, xmax: %10.4lf\n", xmin, xmax);
    printf("  ymin: %10.4lf, ymax: %10.4lf\n", ymin, ymax);
    printf("  zmin: %10.4lf, zmax: %10.4lf\n", zmin, zmax);
}

void Polyhedron_scale(Polyhedron *poly, double scale) {
    for (auto &v : poly->vertices) {
        v.coord.x *= scale;
        v.coord.y *= scale;
        v.coord.z *= scale;
    }
}

}  // extern "C"

namespace ibm {

static const double kPi = 3.141592653589793;

// Plane through three points: n = (b-a) x (c-a), d = -n.a.
static void plane3(const Vector &a, const Vector &b, const Vector &c, double out[4]) {
    const Vector n = Vector_crs(Vector_sub(b, a), Vector_sub(c, a));
    out[0] = n.x;
    out[1] = n.y;
    out[2] = n.z;
    out[3] = -Vector_dot(n, a);
}

static void bbox6(const Vector p[6], CptFeature &f) {
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < 6; i++) {
        const double c[3] = {p[i].x, p[i].y, p[i].z};
        for (int d = 0; d < 3; d++) {
            mx[d] = mx[d] > c[d] ? mx[d] : c[d];
            mn[d] = mn[d] < c[d] ? mn[d] : c[d];
        }
    }
    for (int d = 0; d < 3; d++) {
        f.bmin[d] = mn[d];
        f.bmax[d] = mx[d];
    }
}

static CptFeature face_feature(const Vector p[6], int sgn) {
    CptFeature f{};
    f.kind = FEAT_FACE;
    f.sgn = sgn;
    bbox6(p, f);
    plane3(p[0], p[2], p[1], f.pl[0]);
    plane3(p[3], p[4], p[5], f.pl[1]);
    plane3(p[0], p[1], p[4], f.pl[2]);
    plane3(p[1], p[2], p[5], f.pl[3]);
    plane3(p[0], p[3], p[5], f.pl[4]);
    f.a[0] = Vector_norm(Vector{f.pl[0][0], f.pl[0][1], f.pl[0][2]});
    return f;
}

static CptFeature edge_feature(const Vector p[6], int sgn) {
    CptFeature f{};
    f.kind = FEAT_EDGE;
    f.sgn = sgn;
    bbox6(p, f);
    plane3(p[0], p[4], p[2], f.pl[0]);
    plane3(p[1], p[3], p[5], f.pl[1]);
    plane3(p[0], p[2], p[3], f.pl[2]);
    plane3(p[2], p[4], p[5], f.pl[3]);
    plane3(p[0], p[1], p[5], f.pl[4]);
    f.a[0] = p[0].x; f.a[1] = p[0].y; f.a[2] = p[0].z;
    f.b[0] = p[1].x; f.b[1] = p[1].y; f.b[2] = p[1].z;
    return f;
}

static CptFeature vertex_feature(const Vector &v, const Vector &axis, double angle, double radius, int sgn) {
    CptFeature f{};
    f.kind = FEAT_VERTEX;
    f.sgn = sgn;
    f.a[0] = v.x; f.a[1] = v.y; f.a[2] = v.z;
    f.b[0] = axis.x; f.b[1] = axis.y; f.b[2] = axis.z;
    f.angle = angle;
    f.radius = radius;
    f.bmin[0] = v.x - radius; f.bmax[0] = v.x + radius;
    f.bmin[1] = v.y - radius; f.bmax[1] = v.y + radius;
    f.bmin[2] = v.z - radius; f.bmax[2] = v.z + radius;
    return f;
}

static int build_bvh(CptModel &m, std::vector<int> &ids, int lo, int hi, const std::vector<float> &cent,
                     const std::vector<float> &tmin, const std::vector<float> &tmax) {
    BVHNode node{};
    for (int d = 0; d < 3; d++) {
        node.bmin[d] = INFINITY;
        node.bmax[d] = -INFINITY;
    }
    for (int q = lo; q < hi; q++)
        for (int d = 0; d < 3; d++) {
            node.bmin[d] = std::min(node.bmin[d], tmin[3 * ids[q] + d]);
            node.bmax[d] = std::max(node.bmax[d], tmax[3 * ids[q] + d]);
        }
    const int me = (int)m.nodes.size();
    m.nodes.push_back(node);
    if (hi - lo <= 4) {
        m.nodes[me].left = m.nodes[me].right = -1;
        m.nodes[me].start = lo;
        m.nodes[me].count = hi - lo;
        return me;
    }
    int axis = 0;
    float ext = -1;
    for (int d = 0; d < 3; d++)
        if (node.bmax[d] - node.bmin[d] > ext) {
            ext = node.bmax[d] - node.bmin[d];
            axis = d;
        }
    const int mid = (lo + hi) / 2;
    std::nth_element(ids.begin() + lo, ids.begin() + mid, ids.begin() + hi, [&](int a, int b) {
        if (cent[3 * a + axis] != cent[3 * b + axis]) return cent[3 * a + axis] < cent[3 * b + axis];
        return a < b;
    });
    const int l = build_bvh(m, ids, lo, mid, cent, tmin, tmax);
    const int r = build_bvh(m, ids, mid, hi, cent, tmin, tmax);
    m.nodes[me].left = l;
    m.nodes[me].right = r;
    m.nodes[me].start = m.nodes[me].count = 0;
    return me;
}

void build_cpt_model(const Polyhedron *poly, double maxd, CptModel &m) {
    m = CptModel();
    const int nf = (int)poly->faces.size(), ne = (int)poly->edges.size(), nv = (int)poly->vertices.size();
    std::vector<std::vector<int>> edge_feats(ne), vert_feats(nv);
    std::vector<int> face_feats(2 * nf);
    auto coord = [&](int v) { return poly->vertices[v].coord; };

    for (int i = 0; i < nf; i++) {
        const FaceRec &fc = poly->faces[i];
        Vector p[6];
        for (int j = 0; j < 3; j++) {
            p[j] = coord(fc.vertex_idx[j]);
            p[j + 3] = Vector_lincom(1, p[j], maxd, fc.n);
        }
        face_feats[2 * i] = (int)m.features.size();
        m.features.push_back(face_feature(p, 1));
        for (int j = 0; j < 3; j++) {
            p[j] = coord(fc.vertex_idx[(3 - j) % 3]);
            p[j + 3] = Vector_lincom(1, p[j], -maxd, fc.n);
        }
        face_feats[2 * i + 1] = (int)m.features.size();
        m.features.push_back(face_feature(p, -1));
    }

    for (int i = 0; i < ne; i++) {
        const EdgeRec &e = poly->edges[i];
        Vector p[6];
        p[0] = coord(e.vertex_idx[0]);
        p[1] = coord(e.vertex_idx[1]);
        const Vector v = Vector_sub(p[1], p[0]);
        const Vector nl = poly->faces[e.face_idx[0]].n;
        const Vector nr = poly->faces[e.face_idx[1]].n;
        const int sgn = Vector_dot(Vector_crs(v, nl), nr) >= 0 ? 1 : -1;
        const double angle = Vector_angle(nl, nr);
        // Normals bounding each wedge, in the reference's order.
        std::vector<std::pair<Vector, Vector>> wedges;
        if (angle <= kPi / 3) {
            if (sgn == 1) wedges.push_back({nl, nr});
            else wedges.push_back({nr, nl});
        } else if (angle <= 2 * kPi / 3) {
            const Vector nm = Vector_rot(nl, v, angle / 2);
            if (sgn == 1) {
                wedges.push_back({nl, nm});
                wedges.push_back({nm, nr});
            } else {
                wedges.push_back({nr, nm});
                wedges.push_back({nm, nl});
            }
        } else {
            if (sgn == 1) {
                const Vector n1 = Vector_rot(nl, v, angle / 3);
                const Vector n2 = Vector_rot(nl, v, 2 * angle / 3);
                wedges.push_back({nl, n1});
                wedges.push_back({n1, n2});
                wedges.push_back({n2, nr});
            } else {
                const Vector n1 = Vector_rot(nl, v, -angle / 3);
                const Vector n2 = Vector_rot(nl, v, -2 * angle / 3);
                wedges.push_back({nr, n2});
                wedges.push_back({n2, n1});
                wedges.push_back({n1, nl});
            }
        }
        const double s = sgn == 1 ? maxd : -maxd;
        for (auto &w : wedges) {
            p[2] = Vector_lincom(1, p[0], s, w.first);
            p[3] = Vector_lincom(1, p[1], s, w.first);
            p[4] = Vector_lincom(1, p[0], s, w.second);
            p[5] = Vector_lincom(1, p[1], s, w.second);
            edge_feats[i].push_back((int)m.features.size());
            m.features.push_back(edge_feature(p, sgn));
        }
    }

    for (int i = 0; i < nv; i++) {
        const VertexRec &vr = poly->vertices[i];
        const Vector vx = vr.coord;
        std::vector<int> adj(vr.num_faces, i);
        double adj_angle = 0;
        Vector axis{0, 0, 0};
        for (int j = 0; j < vr.num_faces; j++) {
            const FaceRec &af = poly->faces[vr.face_idx[j]];
            for (int k = 0; k < 3; k++) {
                if (af.vertex_idx[k] == i) {
                    adj_angle = Vector_angle(Vector_sub(coord(af.vertex_idx[(k + 1) % 3]), vx),
                                             Vector_sub(coord(af.vertex_idx[(k + 2) % 3]), vx));
                    adj[j] = af.vertex_idx[(k + 2) % 3];
                }
            }
            axis = Vector_lincom(1, axis, adj_angle, af.n);
        }
        axis = Vector_normalize(axis);
        double cone = 0;
        for (int j = 0; j < vr.num_faces; j++) {
            const Vector an = poly->faces[vr.face_idx[j]].n;
            if (Vector_dot(axis, an) > 0) {
                const double a = Vector_angle(axis, an);
                cone = cone > a ? cone : a;
            }
        }
        bool convex = true, concave = true;
        for (int j = 0; j < vr.num_faces; j++) {
            const double d = Vector_dot(Vector_sub(coord(adj[j]), vx), axis);
            if (d > 0) convex = false;
            if (d < 0) concave = false;
        }
        if (!concave) {
            vert_feats[i].push_back((int)m.features.size());
            m.features.push_back(vertex_feature(vx, axis, cone, maxd, 1));
        }
        if (!convex) {
            vert_feats[i].push_back((int)m.features.size());
            m.features.push_back(vertex_feature(vx, Vector{-axis.x, -axis.y, -axis.z}, cone, maxd, -1));
        }
    }

    // Triangle -> features (its two prisms, its edges' wedges, its vertices' cones).
    std::vector<int> ids(nf);
    std::iota(ids.begin(), ids.end(), 0);
    std::vector<float> cent(3 * nf), tmin(3 * nf), tmax(3 * nf);
    for (int t = 0; t < nf; t++) {
        for (int d = 0; d < 3; d++) {
            float mn = INFINITY, mx = -INFINITY, s = 0;
            for (int j = 0; j < 3; j++) {
                const Vector c = coord(poly->faces[t].vertex_idx[j]);
                const float x = (float)(d == 0 ? c.x : d == 1 ? c.y : c.z);
                mn = std::min(mn, x);
                mx = std::max(mx, x);
                s += x;
            }
            // Widen by a few float ulps so float distances never exceed the truth.
            const float pad = 1e-6f * (1.0f + std::max(std::fabs(mn), std::fabs(mx)));
            tmin[3 * t + d] = mn - pad;
            tmax[3 * t + d] = mx + pad;
            cent[3 * t + d] = s / 3;
        }
    }
    if (nf > 0) build_bvh(m, ids, 0, nf, cent, tmin, tmax);
    m.tri_id = ids;
    m.tri_feat_start.assign(nf + 1, 0);
    for (int q = 0; q < nf; q++) {
        const int t = ids[q];
        std::vector<int> fl;
        fl.push_back(face_feats[2 * t]);
        fl.push_back(face_feats[2 * t + 1]);
        for (int j = 0; j < 3; j++)
            for (int x : edge_feats[poly->faces[t].edge_idx[j]]) fl.push_back(x);
        for (int j = 0; j < 3; j++)
            for (int x : vert_feats[poly->faces[t].vertex_idx[j]]) fl.push_back(x);
        m.tri_feats.insert(m.tri_feats.end(), fl.begin(), fl.end());
        m.tri_feat_start[q + 1] = (int)m.tri_feats.size();
        for (int j = 0; j < 3; j++) {
            const Vector c = coord(poly->faces[t].vertex_idx[j]);
            m.tri_xyz.push_back((float)c.x);
            m.tri_xyz.push_back((float)c.y);
            m.tri_xyz.push_back((float)c.z);
        }
    }
}

}  // namespace ibm
