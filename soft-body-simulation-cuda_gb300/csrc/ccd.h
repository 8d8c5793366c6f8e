// Continuous collision between bodies (internal to the engine).
//
// The reference runs, after every PD step with collision handling on
// (PdSolver::Update, pdSolver.cu:218-224), CollisionDetection::DetectCollision
// (src/collision/bvh.cu:153-165: LBVH over the surface triangles' swept
// boxes, candidate pairs of triangles of different bodies, point-face and
// edge-edge continuous tests, earliest contact per vertex / edge) and then
// CCDKernel (collisionUtil.cu:50-70).  CcdContext is the GPU form of both.
#pragma once
#include <memory>
#include <vector>

#include "engine.h"

namespace pdgb {

// Surface of a collision system, in the engine's vertex order.  Triangle t
// keeps its caller index t (face queries break contact-time ties by it);
// its vertices are stored in ascending caller id (the reference sorts a
// face query's face vertices), edges likewise, edge ids follow the
// lexicographic order of (smaller, larger) caller id.
struct CcdSurface {
    int nv = 0, ntris = 0, nedges = 0;
    std::vector<uint4> tri;        // x, y, z: internal vertex ids; w: body
    std::vector<uint4> tri_edges;  // x, y, z: edge ids of the triangle
    std::vector<uint2> edges;      // internal vertex ids (ascending caller id)
};

// tris: [3 ntris] caller vertex ids; tri_body: [ntris]; viperm: caller ->
// internal vertex (null: identity).  Throws Error on bad input.
CcdSurface build_ccd_surface(int nv, int ntris, const uint32_t* tris, const int* tri_body, const int* viperm);

struct CcdStats {
    long long pairs = 0;        // candidate triangle pairs of the last detection
    long long sources = 0;      // vertices / edges whose earliest contact is before t = 1
    int marked = 0;             // vertices with tI < 1
    int regrows = 0;            // candidate buffer enlargements so far
    double ms = 0.0;            // device time of the last detection + response
};

class CcdContext {
public:
    // vcaller: device array internal -> caller vertex id (null: identity),
    // kept by the caller for the context's lifetime.
    CcdContext(const CcdSurface& s, const int* vcaller, cudaStream_t stream);
    ~CcdContext();
    CcdContext(const CcdContext&) = delete;
    CcdContext& operator=(const CcdContext&) = delete;

    // Detection between x (start, internal order) and xt (end): fills tI and
    // normals (device, internal order).  Waits for the stream (the candidate
    // count decides the narrow phase's size, as in the reference).
    void detect(const float4* x, const float4* xt);
    // CCDKernel + the fixed-body correction of XTilde and v (the reference
    // applies it after the collision response, pdSolver.cu:228-231).
    void respond(float4* x, const float4* xt, float4* v, const SceneArgs& sc);

    const float* tI() const;
    const float4* normals() const;
    const CcdStats& stats() const { return stats_; }
    int nv() const { return nv_; }

private:
    struct Buffers;
    std::unique_ptr<Buffers> b_;
    int nv_ = 0, ntris_ = 0, nedges_ = 0;
    const int* vcaller_ = nullptr;
    cudaStream_t stream_ = nullptr;
    CcdStats stats_;
};

}  // namespace pdgb
