// cpu_hull.cpp — the reference's CPU hull and its output cleanup on the host.
//
// quickhull(): the double-precision quickhull the reference runs on the CPU
// (Antti Kuukka's public-domain quickhull, wasm/quickhull/QuickHull.cpp,
// behind wasm/qh.cpp and src/cpu/hull.ts:44-60), restated on flat arrays:
// the same initial tetrahedron, the same face-stack order, visibility walk,
// horizon loop, slot reuse and point assignment, so its triangles (and their
// order) are that implementation's for the same points and epsilon.
//
// clean_hull_faces(): cleanHullFaces (src/cpu/hull.ts:87-155), which rebuilds
// an exact grid hull's output faces from the hull's own vertices with that
// quickhull and keeps the rebuilt faces only when they are closed, keep the
// volume and contain every vertex.
//
// Compiled without floating-point contraction, like the rest of the host
// geometry, so every product and sum rounds as the reference's does.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <deque>
#include <cstring>
#include <map>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host_mesh.h"

namespace cuacd {
namespace host {

namespace {

constexpr uint32_t QH_NONE = 0xffffffffu;

struct V3 {
  double x, y, z;
};
inline double dot3(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// (a - c) x (b - c), the orientation normal of triangle (a, b, c)
inline V3 tri_normal(const V3& a, const V3& b, const V3& c) {
  const double x = a.x - c.x, y = a.y - c.y, z = a.z - c.z;
  const double rx = b.x - c.x, ry = b.y - c.y, rz = b.z - c.z;
  return V3{y * rz - z * ry, z * rx - x * rz, x * ry - y * rx};
}

struct HalfEdge {
  uint32_t end, opp, face, next;  // end == QH_NONE: free slot
};

struct QFace {
  uint32_t he = QH_NONE;  // QH_NONE: free slot
  V3 n{0, 0, 0};
  double d = 0, nn = 0;   // plane n . p + d = 0, nn = |n|^2
  double far = 0;         // most distant assigned point and its distance
  uint32_t farPt = 0;
  uint64_t checked = 0;   // pass in which visibility was last tested
  bool visible = false, queued = false;
  uint8_t horizon = 0;    // bit j: half edge j of the face is a horizon edge
  std::vector<uint32_t> pts;  // points on the positive side; empty = none
};

class QuickHull {
 public:
  QuickHull(const double* p, size_t n, double eps) : n_(n) {
    P_.resize(n);
    for (size_t i = 0; i < n; i++) P_[i] = V3{p[3 * i], p[3 * i + 1], p[3 * i + 2]};
    extremes();
    eps_ = eps * scale_;
    eps2_ = eps_ * eps_;
  }

  void run() {
    tetrahedron();
    iterate();
    if (planar_) {
      // the helper point becomes vertex 0 of the output
      const uint32_t extra = (uint32_t)P_.size() - 1;
      for (HalfEdge& e : E_)
        if (e.end == extra) e.end = 0;
      P_.resize(n_);
    }
  }

  // Output faces by a depth-first walk from the first live slot; vertices
  // numbered by first appearance, triangles wound (v0, v2, v1).
  void output(std::vector<double>& vOut, std::vector<uint32_t>& tOut) const {
    vOut.clear();
    tOut.clear();
    std::vector<char> done(F_.size(), 0);
    std::vector<uint32_t> stack;
    for (size_t i = 0; i < F_.size(); i++)
      if (F_[i].he != QH_NONE) {
        stack.push_back((uint32_t)i);
        break;
      }
    std::map<uint32_t, uint32_t> remap;
    while (!stack.empty()) {
      const uint32_t f = stack.back();
      stack.pop_back();
      if (done[f]) continue;
      done[f] = 1;
      uint32_t he[3];
      face_edges(f, he);
      for (int k = 0; k < 3; k++) {
        const uint32_t g = E_[E_[he[k]].opp].face;
        if (!done[g] && F_[g].he != QH_NONE) stack.push_back(g);
      }
      uint32_t v[3];
      for (int k = 0; k < 3; k++) {
        const uint32_t pi = E_[he[k]].end;
        auto it = remap.find(pi);
        if (it == remap.end()) {
          const uint32_t id = (uint32_t)(vOut.size() / 3);
          remap.emplace(pi, id);
          vOut.push_back(P_[pi].x);
          vOut.push_back(P_[pi].y);
          vOut.push_back(P_[pi].z);
          v[k] = id;
        } else {
          v[k] = it->second;
        }
      }
      tOut.push_back(v[0]);
      tOut.push_back(v[2]);
      tOut.push_back(v[1]);
    }
  }

 private:
  size_t n_;
  std::vector<V3> P_;
  std::vector<HalfEdge> E_;
  std::vector<QFace> F_;
  std::vector<uint32_t> freeF_, freeE_;
  uint32_t ext_[6] = {0, 0, 0, 0, 0, 0};
  double scale_ = 0, eps_ = 0, eps2_ = 0;
  bool planar_ = false;

  void face_edges(uint32_t f, uint32_t he[3]) const {
    he[0] = F_[f].he;
    he[1] = E_[he[0]].next;
    he[2] = E_[he[1]].next;
  }
  void face_verts(uint32_t f, uint32_t v[3]) const {
    uint32_t he[3];
    face_edges(f, he);
    for (int k = 0; k < 3; k++) v[k] = E_[he[k]].end;
  }
  void set_plane(QFace& f, const V3& n, const V3& on) {
    f.n = n;
    f.d = -dot3(n, on);
    f.nn = n.x * n.x + n.y * n.y + n.z * n.z;
  }
  double signed_dist(const QFace& f, const V3& p) const { return dot3(f.n, p) + f.d; }

  // Max/min point along each axis, first index on ties; a new maximum is
  // not also tested as a minimum. The scale is the largest magnitude of
  // those extreme coordinates.
  void extremes() {
    if (n_ == 0) return;
    double ev[6] = {P_[0].x, P_[0].x, P_[0].y, P_[0].y, P_[0].z, P_[0].z};
    for (size_t i = 1; i < n_; i++) {
      const double c[3] = {P_[i].x, P_[i].y, P_[i].z};
      for (int a = 0; a < 3; a++) {
        if (c[a] > ev[2 * a]) {
          ev[2 * a] = c[a];
          ext_[2 * a] = (uint32_t)i;
        } else if (c[a] < ev[2 * a + 1]) {
          ev[2 * a + 1] = c[a];
          ext_[2 * a + 1] = (uint32_t)i;
        }
      }
    }
    double s = 0;
    for (int i = 0; i < 6; i++) {
      const V3& p = P_[ext_[i]];
      const double c = i / 2 == 0 ? p.x : (i / 2 == 1 ? p.y : p.z);
      const double a = std::fabs(c);
      if (a > s) s = a;
    }
    scale_ = s;
  }

  // Tetrahedron (a, b, c, d): faces abc, acd, bad, cbd with their half
  // edges in slots 0-11; the opposite-edge table is the tetrahedron's.
  void setup(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    E_.clear();
    F_.clear();
    freeF_.clear();
    freeE_.clear();
    // per half edge: end vertex, opposite, face, next
    const uint32_t v[4] = {a, b, c, d};
    static const uint8_t tab[12][4] = {{1, 6, 0, 1}, {2, 9, 0, 2},  {0, 3, 0, 0},  {2, 2, 1, 4},
                                       {3, 11, 1, 5}, {0, 7, 1, 3},  {0, 0, 2, 7},  {3, 5, 2, 8},
                                       {1, 10, 2, 6}, {1, 1, 3, 10}, {3, 8, 3, 11}, {2, 4, 3, 9}};
    for (int k = 0; k < 12; k++) E_.push_back(HalfEdge{v[tab[k][0]], tab[k][1], tab[k][2], tab[k][3]});
    F_.resize(4);
    for (int f = 0; f < 4; f++) F_[f].he = (uint32_t)(3 * f);
  }

  bool add_point(QFace& f, uint32_t i) {
    const double D = signed_dist(f, P_[i]);
    if (D > 0 && D * D > eps2_ * f.nn) {
      f.pts.push_back(i);
      if (D > f.far) {
        f.far = D;
        f.farPt = i;
      }
      return true;
    }
    return false;
  }

  void tetrahedron() {
    const size_t vc = n_;
    if (vc <= 4) {
      uint32_t v[4] = {0, (uint32_t)std::min<size_t>(1, vc - 1), (uint32_t)std::min<size_t>(2, vc - 1),
                       (uint32_t)std::min<size_t>(3, vc - 1)};
      QFace tmp;
      set_plane(tmp, tri_normal(P_[v[0]], P_[v[1]], P_[v[2]]), P_[v[0]]);
      if (signed_dist(tmp, P_[v[3]]) >= 0) std::swap(v[0], v[1]);
      setup(v[0], v[1], v[2], v[3]);
      return;
    }
    // the two most distant extreme points
    double maxD = eps2_;
    uint32_t s0 = 0, s1 = 0;
    for (int i = 0; i < 6; i++)
      for (int j = i + 1; j < 6; j++) {
        const V3 &p = P_[ext_[i]], &q = P_[ext_[j]];
        const double dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        const double d = dx * dx + dy * dy + dz * dz;
        if (d > maxD) {
          maxD = d;
          s0 = ext_[i];
          s1 = ext_[j];
        }
      }
    if (maxD == eps2_) {
      // one point, repeated
      setup(0, (uint32_t)std::min<size_t>(1, vc - 1), (uint32_t)std::min<size_t>(2, vc - 1),
            (uint32_t)std::min<size_t>(3, vc - 1));
      return;
    }
    // the point farthest from the line through them
    const V3 S = P_[s0];
    const V3 Vd{P_[s1].x - S.x, P_[s1].y - S.y, P_[s1].z - S.z};
    const double inv = 1 / (Vd.x * Vd.x + Vd.y * Vd.y + Vd.z * Vd.z);
    maxD = eps2_;
    uint32_t mi = QH_NONE;
    for (size_t i = 0; i < vc; i++) {
      const V3 s{P_[i].x - S.x, P_[i].y - S.y, P_[i].z - S.z};
      const double t = dot3(s, Vd);
      const double d = (s.x * s.x + s.y * s.y + s.z * s.z) - t * t * inv;
      if (d > maxD) {
        maxD = d;
        mi = (uint32_t)i;
      }
    }
    if (maxD == eps2_) {
      // collinear: a flat tetrahedron from the first points off the two ends
      auto same = [&](size_t i, uint32_t j) { return P_[i].x == P_[j].x && P_[i].y == P_[j].y && P_[i].z == P_[j].z; };
      uint32_t third = s0, fourth = s0;
      for (size_t i = 0; i < vc; i++)
        if (!same(i, s0) && !same(i, s1)) {
          third = (uint32_t)i;
          break;
        }
      for (size_t i = 0; i < vc; i++)
        if (!same(i, s0) && !same(i, s1) && !same(i, third)) {
          fourth = (uint32_t)i;
          break;
        }
      setup(s0, s1, third, fourth);
      return;
    }
    uint32_t base[3] = {s0, s1, mi};
    const V3 b0 = P_[base[0]], b1 = P_[base[1]], b2 = P_[base[2]];
    // the point farthest from the base plane
    maxD = eps_;
    mi = 0;
    const V3 N = tri_normal(b0, b1, b2);
    QFace bp;
    set_plane(bp, N, b0);
    for (size_t i = 0; i < vc; i++) {
      const double d = std::fabs(signed_dist(bp, P_[i]));
      if (d > maxD) {
        maxD = d;
        mi = (uint32_t)i;
      }
    }
    if (maxD == eps_) {
      // coplanar points: a helper point off the plane gives the hull volume
      planar_ = true;
      const V3 N1 = tri_normal(b1, b2, b0);
      P_.push_back(V3{N1.x + P_[0].x, N1.y + P_[0].y, N1.z + P_[0].z});
      mi = (uint32_t)P_.size() - 1;
    }
    if (signed_dist(bp, P_[mi]) >= 0) std::swap(base[0], base[1]);
    setup(base[0], base[1], base[2], mi);
    for (uint32_t f = 0; f < 4; f++) {
      uint32_t v[3];
      face_verts(f, v);
      set_plane(F_[f], tri_normal(P_[v[0]], P_[v[1]], P_[v[2]]), P_[v[0]]);
    }
    for (size_t i = 0; i < vc; i++)
      for (uint32_t f = 0; f < 4; f++)
        if (add_point(F_[f], (uint32_t)i)) break;
  }

  uint32_t add_face() {
    if (!freeF_.empty()) {
      const uint32_t i = freeF_.back();
      freeF_.pop_back();
      F_[i].far = 0;
      return i;
    }
    F_.emplace_back();
    return (uint32_t)F_.size() - 1;
  }
  uint32_t add_edge() {
    if (!freeE_.empty()) {
      const uint32_t i = freeE_.back();
      freeE_.pop_back();
      return i;
    }
    E_.push_back(HalfEdge{0, 0, 0, 0});
    return (uint32_t)E_.size() - 1;
  }

  // chain the horizon edges into a loop, each starting where the previous ends
  bool order_horizon(std::vector<uint32_t>& h) const {
    for (size_t i = 0; i + 1 < h.size(); i++) {
      const uint32_t endV = E_[h[i]].end;
      bool found = false;
      for (size_t j = i + 1; j < h.size(); j++)
        if (E_[E_[h[j]].opp].end == endV) {
          std::swap(h[i + 1], h[j]);
          found = true;
          break;
        }
      if (!found) return false;
    }
    return true;
  }

  void iterate() {
    std::deque<uint32_t> queue;
    for (uint32_t i = 0; i < 4; i++)
      if (!F_[i].pts.empty()) {
        queue.push_back(i);
        F_[i].queued = true;
      }
    std::vector<uint32_t> horizon, visible, newFaces, newEdges;
    std::vector<std::pair<uint32_t, uint32_t>> walk;  // (face, half edge entered through)
    // the visible faces' points in visible-face order (their lists keep
    // their storage for the faces that reuse the slots)
    std::vector<uint32_t> orphans;
    uint64_t pass = 0;
    while (!queue.empty()) {
      pass++;
      const uint32_t top = queue.front();
      queue.pop_front();
      F_[top].queued = false;
      if (F_[top].pts.empty() || F_[top].he == QH_NONE) continue;
      const uint32_t eye = F_[top].farPt;
      const V3 ep = P_[eye];
      // faces that see the eye point, depth first from the top face; a face
      // that does not see it closes a horizon edge
      horizon.clear();
      visible.clear();
      walk.clear();
      walk.emplace_back(top, QH_NONE);
      while (!walk.empty()) {
        const auto [fi, from] = walk.back();
        walk.pop_back();
        QFace& f = F_[fi];
        if (f.checked == pass) {
          if (f.visible) continue;
        } else {
          f.checked = pass;
          if (signed_dist(f, ep) > 0) {
            f.visible = true;
            f.horizon = 0;
            visible.push_back(fi);
            uint32_t he[3];
            face_edges(fi, he);
            for (int k = 0; k < 3; k++)
              if (E_[he[k]].opp != from) walk.emplace_back(E_[E_[he[k]].opp].face, he[k]);
            continue;
          }
        }
        f.visible = false;
        horizon.push_back(from);
        const uint32_t owner = E_[from].face;
        uint32_t he[3];
        face_edges(owner, he);
        const int ind = he[0] == from ? 0 : (he[1] == from ? 1 : 2);
        F_[owner].horizon |= (uint8_t)(1u << ind);
      }
      const size_t hc = horizon.size();
      if (!order_horizon(horizon)) {
        // the horizon does not close (rounding): this point is given up
        std::vector<uint32_t>& tp = F_[top].pts;
        auto it = std::find(tp.begin(), tp.end(), eye);
        if (it != tp.end()) tp.erase(it);
        if (tp.empty()) std::vector<uint32_t>().swap(tp);
        continue;
      }
      // the visible faces' half edges (horizon edges excepted) are reused
      // for the new faces first, then freed; their points wait for the new
      // faces
      newFaces.clear();
      newEdges.clear();
      orphans.clear();
      size_t reused = 0;
      for (uint32_t fi : visible) {
        uint32_t he[3];
        face_edges(fi, he);
        for (int j = 0; j < 3; j++) {
          if (F_[fi].horizon & (1u << j)) continue;
          if (reused < 2 * hc) {
            newEdges.push_back(he[j]);
            reused++;
          } else {
            E_[he[j]].end = QH_NONE;
            freeE_.push_back(he[j]);
          }
        }
        F_[fi].he = QH_NONE;
        freeF_.push_back(fi);
        orphans.insert(orphans.end(), F_[fi].pts.begin(), F_[fi].pts.end());
        F_[fi].pts.clear();
      }
      while (reused < 2 * hc) {
        newEdges.push_back(add_edge());
        reused++;
      }
      // one new face per horizon edge AB: triangle (A, B, eye)
      for (size_t i = 0; i < hc; i++) {
        const uint32_t AB = horizon[i];
        const uint32_t A = E_[E_[AB].opp].end, B = E_[AB].end;
        const uint32_t nf = add_face();
        newFaces.push_back(nf);
        const uint32_t CA = newEdges[2 * i], BC = newEdges[2 * i + 1];
        E_[AB].next = BC;
        E_[BC].next = CA;
        E_[CA].next = AB;
        E_[BC].face = nf;
        E_[CA].face = nf;
        E_[AB].face = nf;
        E_[CA].end = A;
        E_[BC].end = eye;
        set_plane(F_[nf], tri_normal(P_[A], P_[B], ep), ep);
        F_[nf].he = AB;
        E_[CA].opp = newEdges[i > 0 ? 2 * i - 1 : 2 * hc - 1];
        E_[BC].opp = newEdges[(2 * (i + 1)) % (2 * hc)];
      }
      // each orphaned point goes to the first new face that sees it
      for (uint32_t q : orphans) {
        if (q == eye) continue;
        for (size_t j = 0; j < hc; j++)
          if (add_point(F_[newFaces[j]], q)) break;
      }
      for (uint32_t nf : newFaces)
        if (!F_[nf].pts.empty() && !F_[nf].queued) {
          queue.push_back(nf);
          F_[nf].queued = true;
        }
    }
  }
};

inline V3 vat(const float* V, uint32_t i) { return V3{(double)V[3 * (size_t)i], (double)V[3 * (size_t)i + 1], (double)V[3 * (size_t)i + 2]}; }

// signed volume of triangles T over vertices V, anchored at vertex 0 of V
// (src/mesh.ts:59-72)
double signed_volume_ptr(const float* V, const uint32_t* T, size_t nIdx) {
  if (nIdx == 0) return 0;
  const double ox = V[0], oy = V[1], oz = V[2];
  double s = 0;
  for (size_t i = 0; i + 2 < nIdx; i += 3) {
    const float* a = V + 3 * (size_t)T[i];
    const float* b = V + 3 * (size_t)T[i + 1];
    const float* c = V + 3 * (size_t)T[i + 2];
    const double ax = a[0] - ox, ay = a[1] - oy, az = a[2] - oz;
    const double bx = b[0] - ox, by = b[1] - oy, bz = b[2] - oz;
    const double cx = c[0] - ox, cy = c[1] - oy, cz = c[2] - oz;
    s += ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
  }
  return s / 6;
}

// every directed edge of T once and its reverse once (src/mesh.ts:104-119)
bool closed_ptr(const uint32_t* T, size_t nIdx, size_t nv) {
  std::vector<uint64_t> e;
  e.reserve(nIdx);
  for (size_t t = 0; t + 2 < nIdx; t += 3)
    for (int k = 0; k < 3; k++) {
      const uint32_t a = T[t + k], b = T[t + (k + 1) % 3];
      if (a >= nv || b >= nv) return false;
      e.push_back(((uint64_t)a << 32) | b);
    }
  std::sort(e.begin(), e.end());
  for (size_t i = 0; i < e.size(); i++) {
    if (i + 1 < e.size() && e[i + 1] == e[i]) return false;  // a directed edge twice
    const uint64_t r = (e[i] << 32) | (e[i] >> 32);
    if (!std::binary_search(e.begin(), e.end(), r)) return false;
  }
  return true;
}

// a point's coordinates as a key; -0 and 0 are one key, as the reference's
// printed-number key makes them
struct PtKey {
  uint64_t x, y, z;
  bool operator==(const PtKey& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct PtKeyHash {
  size_t operator()(const PtKey& k) const {
    uint64_t h = k.x * 0x9E3779B97F4A7C15ull;
    h ^= (k.y + 0x632BE59BD9B4E019ull + (h << 6) + (h >> 2));
    h ^= (k.z + 0x85157AF5ull + (h << 6) + (h >> 2));
    return (size_t)h;
  }
};
inline PtKey pt_key(double x, double y, double z) {
  PtKey k;
  const double a = x + 0.0, b = y + 0.0, c = z + 0.0;
  std::memcpy(&k.x, &a, 8);
  std::memcpy(&k.y, &b, 8);
  std::memcpy(&k.z, &c, 8);
  return k;
}

double hyp3(double x, double y, double z) { return std::hypot(x, y, z); }

// every point within tol of every plane (n . p - d <= tol). The points are
// grouped, 32 consecutive points in Morton order of their coordinates, each
// group with a bounding sphere; a plane skips a group whose sphere lies
// below tol by more than a slack that covers the rounding of the bound and
// of every per-point value (both at most a few units in the last place of
// |n| |p| + |d|; the slack is 1e-9 of that), so the answer is the per-point
// loop's. A large set is split over threads.
bool all_inside(const std::vector<double>& planes, const float* V, const std::vector<uint32_t>& idx, double tol) {
  constexpr size_t GS = 32;
  const size_t n = idx.size(), nf = planes.size() / 4;
  if (n == 0) return true;
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, maxAbs = 0;
  for (size_t k = 0; k < n; k++)
    for (int a = 0; a < 3; a++) {
      const double c = V[3 * (size_t)idx[k] + a];
      lo[a] = std::min(lo[a], c);
      hi[a] = std::max(hi[a], c);
      maxAbs = std::max(maxAbs, std::fabs(c));
    }
  // Morton order on a 1024^3 grid over the bounding box
  auto spread = [](uint64_t v) {
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x30000ffull;
    v = (v | (v << 8)) & 0x300f00full;
    v = (v | (v << 4)) & 0x30c30c3ull;
    v = (v | (v << 2)) & 0x9249249ull;
    return v;
  };
  std::vector<std::pair<uint64_t, uint32_t>> order(n);
  for (size_t k = 0; k < n; k++) {
    uint64_t code = 0;
    for (int a = 0; a < 3; a++) {
      const double span = hi[a] - lo[a];
      const double t = span > 0 ? ((double)V[3 * (size_t)idx[k] + a] - lo[a]) / span : 0.0;
      const uint64_t q = (uint64_t)std::min(1023.0, std::max(0.0, t * 1024.0));
      code |= spread(q) << a;
    }
    order[k] = {code, (uint32_t)k};
  }
  std::sort(order.begin(), order.end());
  std::vector<double> px(n), py(n), pz(n);
  for (size_t k = 0; k < n; k++) {
    const size_t i = 3 * (size_t)idx[order[k].second];
    px[k] = V[i];
    py[k] = V[i + 1];
    pz[k] = V[i + 2];
  }
  const size_t ng = (n + GS - 1) / GS;
  std::vector<double> gx(ng), gy(ng), gz(ng), gr(ng);
  for (size_t g = 0; g < ng; g++) {
    const size_t k0 = g * GS, k1 = std::min(n, k0 + GS);
    double bl[3] = {INFINITY, INFINITY, INFINITY}, bh[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t k = k0; k < k1; k++) {
      bl[0] = std::min(bl[0], px[k]); bh[0] = std::max(bh[0], px[k]);
      bl[1] = std::min(bl[1], py[k]); bh[1] = std::max(bh[1], py[k]);
      bl[2] = std::min(bl[2], pz[k]); bh[2] = std::max(bh[2], pz[k]);
    }
    gx[g] = 0.5 * (bl[0] + bh[0]);
    gy[g] = 0.5 * (bl[1] + bh[1]);
    gz[g] = 0.5 * (bl[2] + bh[2]);
    double r = 0;
    for (size_t k = k0; k < k1; k++) {
      const double dx = px[k] - gx[g], dy = py[k] - gy[g], dz = pz[k] - gz[g];
      r = std::max(r, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    gr[g] = r * (1 + 1e-9) + 1e-300;
  }
  std::atomic<bool> outside{false};
  auto range = [&](size_t f0, size_t f1) {
    for (size_t f = f0; f < f1 && !outside.load(std::memory_order_relaxed); f++) {
      const double nx = planes[4 * f], ny = planes[4 * f + 1], nz = planes[4 * f + 2], d = planes[4 * f + 3];
      const double nlen = std::sqrt(nx * nx + ny * ny + nz * nz) * (1 + 1e-9);
      const double cut = tol - 1e-9 * (6 * nlen * maxAbs + std::fabs(d)) - 1e-300;
      bool out = false;
      for (size_t g = 0; g < ng && !out; g++) {
        if (nx * gx[g] + ny * gy[g] + nz * gz[g] - d + gr[g] * nlen <= cut) continue;
        const size_t k1 = std::min(n, g * GS + GS);
        for (size_t k = g * GS; k < k1; k++)
          if (nx * px[k] + ny * py[k] + nz * pz[k] - d > tol) out = true;
      }
      if (out) outside.store(true, std::memory_order_relaxed);
    }
  };
  const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = (double)nf * (double)ng > 4e6 ? std::min<size_t>(hc, 16) : 1;
  if (nt <= 1) {
    range(0, nf);
  } else {
    std::vector<std::thread> th;
    const size_t per = (nf + nt - 1) / nt;
    for (size_t t = 0; t < nt; t++) {
      const size_t f0 = t * per, f1 = std::min(nf, f0 + per);
      if (f0 < f1) th.emplace_back(range, f0, f1);
    }
    for (std::thread& x : th) x.join();
  }
  return !outside.load();
}

}  // namespace

void quickhull(const double* pts, size_t n, double eps, std::vector<double>& vOut, std::vector<uint32_t>& tOut) {
  vOut.clear();
  tOut.clear();
  if (n == 0) return;
  QuickHull qh(pts, n, eps);
  qh.run();
  qh.output(vOut, tOut);
}

std::vector<uint32_t> clean_hull_faces(const float* V, size_t nv, const uint32_t* T, size_t nIdx, double eps) {
  std::vector<uint32_t> raw(T, T + nIdx);
  if (nIdx < 12) return raw;
  std::vector<uint32_t> cand;
  {
    std::vector<char> seen(nv, 0);
    for (size_t i = 0; i < nIdx; i++)
      if (T[i] < nv && !seen[T[i]]) {
        seen[T[i]] = 1;
        cand.push_back(T[i]);
      }
  }
  const double vRaw = std::fabs(signed_volume_ptr(V, T, nIdx));
  double lo = INFINITY, hi = -INFINITY;
  for (uint32_t c : cand)
    for (int a = 0; a < 3; a++) {
      lo = std::min(lo, (double)V[3 * (size_t)c + a]);
      hi = std::max(hi, (double)V[3 * (size_t)c + a]);
    }
  const double extent = std::max(hi - lo, 1e-30);
  const double tol = 5 * eps * extent;
  std::vector<double> pts, hv;
  std::vector<uint32_t> ht;
  for (int round = 0; round < 6; round++) {
    const size_t n = cand.size();
    if (n < 4) return raw;
    pts.resize(3 * n);
    // hull vertices map back to the candidate with those coordinates (the
    // last one when several share them)
    std::unordered_map<PtKey, uint32_t, PtKeyHash> byKey;
    byKey.reserve(2 * n);
    for (size_t k = 0; k < n; k++) {
      const V3 p = vat(V, cand[k]);
      pts[3 * k] = p.x;
      pts[3 * k + 1] = p.y;
      pts[3 * k + 2] = p.z;
      byKey[pt_key(p.x, p.y, p.z)] = cand[k];
    }
    quickhull(pts.data(), n, eps, hv, ht);
    std::vector<uint32_t> out(ht.size());
    for (size_t i = 0; i < ht.size(); i++) {
      const size_t h = 3 * (size_t)ht[i];
      auto it = byKey.find(pt_key(hv[h], hv[h + 1], hv[h + 2]));
      if (it == byKey.end()) return raw;
      out[i] = it->second;
    }
    if (!closed_ptr(out.data(), out.size(), nv)) return raw;
    const double svNew = signed_volume_ptr(V, out.data(), out.size());
    if (svNew < 0)
      for (size_t i = 0; i + 2 < out.size(); i += 3) std::swap(out[i + 1], out[i + 2]);
    if (!(std::fabs(std::fabs(svNew) - vRaw) <= 10 * eps * vRaw + 1e-30)) return raw;
    // a thin face drops the vertex between the other two; every vertex must
    // lie within the tolerance of every other face's plane. The reference
    // stops at the first vertex outside a face; whichever it is, the raw
    // faces are returned, so the faces are tested in any order here.
    std::vector<uint32_t> drop;
    std::vector<double> planes;  // unit normal and offset of each non-thin face
    for (size_t t = 0; t + 2 < out.size(); t += 3) {
      const uint32_t ia = out[t], ib = out[t + 1], ic = out[t + 2];
      const V3 a = vat(V, ia), b = vat(V, ib), c = vat(V, ic);
      const double ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z;
      const double wx = c.x - a.x, wy = c.y - a.y, wz = c.z - a.z;
      double nx = uy * wz - uz * wy, ny = uz * wx - ux * wz, nz = ux * wy - uy * wx;
      const double l = hyp3(nx, ny, nz);
      const double lab = hyp3(ux, uy, uz), lac = hyp3(wx, wy, wz), lbc = hyp3(c.x - b.x, c.y - b.y, c.z - b.z);
      const double longest = std::max(std::max(lab, lac), lbc);
      if (!(l > eps * extent * longest)) {
        const uint32_t d = lbc >= lab && lbc >= lac ? ia : (lac >= lab ? ib : ic);
        if (std::find(drop.begin(), drop.end(), d) == drop.end()) drop.push_back(d);
        continue;
      }
      nx /= l;
      ny /= l;
      nz /= l;
      planes.insert(planes.end(), {nx, ny, nz, nx * a.x + ny * a.y + nz * a.z});
    }
    if (!all_inside(planes, V, cand, tol)) return raw;
    if (drop.empty()) return out;
    std::vector<uint32_t> kept;
    for (uint32_t c : cand)
      if (std::find(drop.begin(), drop.end(), c) == drop.end()) kept.push_back(c);
    cand.swap(kept);
  }
  return raw;
}

Mesh convex_hull_cpu(const float* pts, size_t n, double* volumeOut) {
  if (n < 4) {
    Mesh m;
    m.v.assign(pts, pts + 3 * n);
    if (volumeOut) *volumeOut = 0;
    return m;
  }
  std::vector<double> p(pts, pts + 3 * n), hv;
  std::vector<uint32_t> ht;
  quickhull(p.data(), n, 1e-7, hv, ht);
  std::vector<float> hf(hv.size());
  for (size_t i = 0; i < hv.size(); i++) hf[i] = (float)hv[i];
  return compact_hull(hf.data(), ht.data(), ht.size() / 3, volumeOut);
}

}  // namespace host
}  // namespace cuacd
