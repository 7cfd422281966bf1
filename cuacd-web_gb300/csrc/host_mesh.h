// host_mesh.h — triangle meshes on the host for the decomposition loop:
// volumes, closedness, normalisation, the capped plane cut, concave-edge
// planes, hull compaction and the CPU Hausdorff distance.
//
// Geometry follows the reference's JavaScript arithmetic: every quantity is
// computed in double from float32 inputs and rounded to float32 only where
// the reference stores a Float32Array. The unit is compiled without
// floating-point contraction so a * b + c rounds twice, as in JavaScript.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace cuacd {
namespace host {

struct Mesh {
  std::vector<float> v;     // 3 floats per vertex
  std::vector<uint32_t> t;  // 3 indices per triangle
  size_t nv() const { return v.size() / 3; }
  size_t nt() const { return t.size() / 3; }
};

// plane a x + b y + c z + d = 0 (src/cpu/cut.ts:14)
struct Plane {
  double a, b, c, d;
};

// signed volume by the divergence theorem anchored at vertex 0 (src/mesh.ts:58-72)
double signed_volume(const Mesh& m);
inline double volume(const Mesh& m) {
  const double s = signed_volume(m);
  return s < 0 ? -s : s;
}

// directed edges grouped by source vertex (src/mesh.ts:79-98)
struct EdgeCSR {
  std::vector<uint32_t> off, dst, face;
};
EdgeCSR edge_csr(const Mesh& m);

// every directed edge occurs once and its reverse once (src/mesh.ts:101-115)
bool is_closed(const Mesh& m);

void bbox(const Mesh& m, float lo[3], float hi[3]);

// centre and scale so the largest extent is 2 (src/mesh.ts:129-141)
struct Normalization {
  double scale;
  double center[3];
};
Mesh normalize(const Mesh& m, Normalization& norm);
Mesh denormalize(const Mesh& m, const Normalization& norm);
// plane in normalised space expressed in input units (src/decompose.ts:398-400)
Plane denormalize_plane(const Plane& p, const Normalization& n);

// concatenation, second mesh's indices offset (src/mesh.ts:38-47)
Mesh merge_meshes(const Mesh& a, const Mesh& b);

// Capped plane cut (src/cpu/cut.ts:33-315): vertices within eps of the plane
// are on it, intersection vertices are shared per edge, boundary loops are
// capped (outer loops with their holes by ear clipping, zero-area loops and
// failed clippings by centroid fans). ok = false when the plane does not split
// the mesh or a boundary loop cannot be closed.
struct CutResult {
  bool ok = false;
  Mesh pos, neg;
  const char* reason = nullptr;
};
CutResult plane_cut(const Mesh& m, const Plane& plane, double eps = 1e-6);

// The cut's unit normal n and offset d (the plane divided by the length of
// its normal, std::hypot) and the orthonormal basis (u, v) of the plane in
// which its caps are triangulated. The host cut and the GPU cut both take
// these from here, so both see the same constants.
struct PlaneFrame {
  double n[3], d, u[3], v[3];
};
PlaneFrame plane_frame(const Plane& plane);

// Triangulates a polygon with holes given as one coordinate ring (outer
// first, then each hole from holeStart[k]); returns vertex-index triples into
// the ring. A complete triangulation has n + 2h - 2 triangles; fewer means
// the polygon could not be clipped.
std::vector<uint32_t> ear_clip(const std::vector<double>& xy, const std::vector<uint32_t>& holeStart);

// Candidate planes from sampled concave edges (src/cpu/concave.ts:25-92):
// 4 floats per plane.
std::vector<float> concave_edge_planes(const Mesh& m, int nConcaveEdges, double concaveEps, double concaveThreshold,
                                       uint32_t seed);

// hull faces (indices into pts) compacted to their own vertex list and
// wound outward by the sign of the volume (src/cpu/hull.ts:157-185)
Mesh compact_hull(const float* pts, const uint32_t* tris, size_t ntris, double* volumeOut);

// Hausdorff distance between two meshes by the reference's sampling rule
// (src/cpu/hausdorff.ts): the larger directed distance, exhaustive search
double hausdorff_cpu(const Mesh& a, const Mesh& b);

// The reference's CPU hull (wasm/quickhull/QuickHull.cpp via wasm/qh.cpp):
// double-precision quickhull of n points with epsilon relative to the
// largest extreme coordinate; vOut = hull vertices by first appearance,
// tOut = triangles (counter-clockwise seen from outside).
void quickhull(const double* pts, size_t n, double eps, std::vector<double>& vOut, std::vector<uint32_t>& tOut);

// cleanHullFaces (src/cpu/hull.ts:87-155): the hull faces T (indices into
// V, nv vertices) rebuilt by quickhull from their own vertices, dropping
// vertices of thin faces, accepted only when closed, of the same volume
// and containing every vertex; otherwise T itself.
std::vector<uint32_t> clean_hull_faces(const float* V, size_t nv, const uint32_t* T, size_t nIdx, double eps);

// convexHull (src/cpu/hull.ts:64-73): quickhull at epsilon 1e-7, compacted
// and wound outward
Mesh convex_hull_cpu(const float* pts, size_t n, double* volumeOut);

}  // namespace host
}  // namespace cuacd
