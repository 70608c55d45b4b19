// Internal geometry interface: polyhedron topology (host) and the feature
// list / triangle BVH that the GPU closest-point transform consumes.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/geo3d.h"

struct VertexRec {
    Vector coord;
    int num_faces;
    std::vector<int> face_idx;
};
struct EdgeRec {
    int vertex_idx[2];
    int face_idx[2];
};
struct FaceRec {
    int vertex_idx[3];
    int edge_idx[3];
    Vector n;
};

struct _polyhedron {
    std::vector<VertexRec> vertices;
    std::vector<EdgeRec> edges;
    std::vector<FaceRec> faces;
};

namespace ibm {

enum { FEAT_FACE = 0, FEAT_EDGE = 1, FEAT_VERTEX = 2 };

// One extrusion of the closest-point transform (src/geo3d.c:436-641), in
// the reference's evaluation order (its index is the tie-break order).
struct CptFeature {
    int kind;
    int sgn;
    double pl[5][4];   // face / edge: the 5 bounding planes (n.x, n.y, n.z, d)
    double a[3];       // face: norm of plane 0 in a[0]; edge: segment start; vertex: apex
    double b[3];       // edge: segment end; vertex: axis
    double angle;      // vertex: cone half-angle
    double radius;     // vertex: cone length
    double bmin[3], bmax[3];  // bounding box of the extrusion (index ranges come from it)
};

struct BVHNode {
    float bmin[3], bmax[3];
    int left, right;   // children, or -1
    int start, count;  // triangle range when leaf
};

struct CptModel {
    std::vector<CptFeature> features;
    std::vector<int> tri_feat_start;   // CSR: features touched by each triangle
    std::vector<int> tri_feats;
    std::vector<float> tri_xyz;        // 9 floats per triangle (BVH order)
    std::vector<int> tri_id;           // BVH order -> face index
    std::vector<BVHNode> nodes;
};

// Builds the extrusion list of Polyhedron_cpt and a BVH over the faces.
void build_cpt_model(const Polyhedron *poly, double maxd, CptModel &m);

}  // namespace ibm
