// plane_cut.cpp — the capped plane cut of the decomposition loop
// (src/cpu/cut.ts:33-315) and the ear clipper for its caps.
//
// The reference triangulates caps with earcut@3.0.1, a third-party package
// absent here; the clipper below is this project's own (outer loop
// counter-clockwise, holes bridged to it from their leftmost vertex by a
// leftward ray, then ears clipped). Both produce n + 2h - 2 triangles for a
// polygon they can clip, so the reference's count check and centroid-fan
// fallback apply unchanged; the cap triangles themselves may differ, the cap
// vertices (and so the part's vertex set, volume and hull) do not.
#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <unordered_set>

#include "host_mesh.h"

namespace cuacd {
namespace host {

// ---------------------------------------------------------------------------
// ear clipping

namespace {

struct Node {
  uint32_t i;  // ring vertex index
  double x, y;
  int32_t prev, next;
};

inline double orient2(const Node& a, const Node& b, const Node& c) {
  return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
}
inline bool same_pos(const Node& a, const Node& b) { return a.x == b.x && a.y == b.y; }

struct Poly {
  std::vector<Node> n;
  int32_t add(uint32_t i, double x, double y, int32_t last) {
    Node v{i, x, y, -1, -1};
    const int32_t k = (int32_t)n.size();
    n.push_back(v);
    if (last < 0) {
      n[k].prev = n[k].next = k;
    } else {
      n[k].next = n[last].next;
      n[k].prev = last;
      n[n[last].next].prev = k;
      n[last].next = k;
    }
    return k;
  }
  // links ring vertices [s, e) so that the loop winds counter-clockwise
  // (ccw = true) or clockwise; returns one node of the loop
  int32_t ring(const std::vector<double>& xy, uint32_t s, uint32_t e, bool ccw) {
    double a = 0;
    for (uint32_t k = s; k < e; k++) {
      const uint32_t j = k + 1 < e ? k + 1 : s;
      a += xy[2 * k] * xy[2 * j + 1] - xy[2 * j] * xy[2 * k + 1];
    }
    int32_t last = -1;
    if ((a > 0) == ccw) {
      for (uint32_t k = s; k < e; k++) last = add(k, xy[2 * k], xy[2 * k + 1], last);
    } else {
      for (uint32_t k = e; k-- > s;) last = add(k, xy[2 * k], xy[2 * k + 1], last);
    }
    return last;
  }
  // splices the loop holding b into the loop holding a with two bridge edges
  // a -> b and b' -> a' (copies of the two vertices)
  void bridge(int32_t a, int32_t b) {
    const int32_t a2 = (int32_t)n.size();
    n.push_back(n[a]);
    const int32_t b2 = (int32_t)n.size();
    n.push_back(n[b]);
    const int32_t an = n[a].next, bp = n[b].prev;
    n[a].next = b;
    n[b].prev = a;
    n[a2].next = an;
    n[an].prev = a2;
    n[b2].next = a2;
    n[a2].prev = b2;
    n[bp].next = b2;
    n[b2].prev = bp;
  }
  bool reflex(int32_t k) const { return orient2(n[n[k].prev], n[k], n[n[k].next]) < 0; }
};

// an outer vertex visible from hole vertex h (leftmost of its loop): the
// nearest crossing of the leftward ray from h with a downward edge of the
// counter-clockwise outer loop, then its endpoint of larger x, replaced by
// the reflex vertex of smallest angle to the ray inside the triangle
// (h, crossing, endpoint) when there is one
int32_t find_bridge(const Poly& P, int32_t h, int32_t outer) {
  const double hx = P.n[h].x, hy = P.n[h].y;
  double qx = -INFINITY;
  int32_t m = -1;
  int32_t p = outer;
  do {
    const Node& a = P.n[p];
    const Node& b = P.n[a.next];
    if (hy <= a.y && hy >= b.y && b.y != a.y) {
      const double x = a.x + (hy - a.y) * (b.x - a.x) / (b.y - a.y);
      if (x <= hx && x > qx) {
        qx = x;
        if (x == hx) {
          if (hy == a.y) return p;
          if (hy == b.y) return a.next;
        }
        m = a.x < b.x ? a.next : p;
      }
    }
    p = a.next;
  } while (p != outer);
  if (m < 0) return -1;
  if (hx == qx) return m;
  const int32_t stop = m;
  const double mx = P.n[m].x, my = P.n[m].y;
  double tanMin = INFINITY;
  p = m;
  do {
    const Node& c = P.n[p];
    if (hx >= c.x && c.x >= mx && hx != c.x) {
      // inside or on the triangle (h, (qx, hy), m), either winding
      const Node A{0, hx, hy, 0, 0}, B{0, qx, hy, 0, 0}, M{0, mx, my, 0, 0};
      const double d1 = orient2(A, B, c), d2 = orient2(B, M, c), d3 = orient2(M, A, c);
      const bool inTri = (d1 >= 0 && d2 >= 0 && d3 >= 0) || (d1 <= 0 && d2 <= 0 && d3 <= 0);
      if (inTri && P.reflex(p)) {
        const double tn = std::fabs(hy - c.y) / (hx - c.x);
        if (tn < tanMin || (tn == tanMin && c.x > P.n[m].x)) {
          m = p;
          tanMin = tn;
        }
      }
    }
    p = c.next;
  } while (p != stop);
  return m;
}

// no other vertex of the loop inside (or on) the triangle of ear k. A vertex
// must also lie in the triangle's bounding box: for a sliver ear the rounded
// orientation tests can admit nearly collinear vertices far along its edge
// lines, which the box excludes (earcut's hashed ear test looks only inside
// the box too), and it lets the GPU cut look at a grid's cells instead of
// every vertex with the same result
bool is_ear(const Poly& P, int32_t k, bool allowFlat) {
  const Node& a = P.n[P.n[k].prev];
  const Node& b = P.n[k];
  const Node& c = P.n[b.next];
  const double ar = orient2(a, b, c);
  if (ar < 0 || (ar == 0 && !allowFlat)) return false;
  const double bx0 = std::min(std::min(a.x, b.x), c.x), bx1 = std::max(std::max(a.x, b.x), c.x);
  const double by0 = std::min(std::min(a.y, b.y), c.y), by1 = std::max(std::max(a.y, b.y), c.y);
  int32_t p = c.next;
  while (p != b.prev) {
    const Node& q = P.n[p];
    if (q.x >= bx0 && q.x <= bx1 && q.y >= by0 && q.y <= by1 && !same_pos(q, a) && !same_pos(q, b) &&
        !same_pos(q, c) && orient2(a, b, q) >= 0 && orient2(b, c, q) >= 0 && orient2(c, a, q) >= 0 &&
        (ar > 0 || (q.x >= std::min(a.x, c.x) && q.x <= std::max(a.x, c.x) && q.y >= std::min(a.y, c.y) &&
                    q.y <= std::max(a.y, c.y))))
      return false;
    p = q.next;
  }
  return true;
}

}  // namespace

std::vector<uint32_t> ear_clip(const std::vector<double>& xy, const std::vector<uint32_t>& holeStart) {
  std::vector<uint32_t> out;
  const uint32_t nAll = (uint32_t)(xy.size() / 2);
  const uint32_t outerEnd = holeStart.empty() ? nAll : holeStart[0];
  if (outerEnd < 3) return out;
  Poly P;
  P.n.reserve(nAll + 2 * holeStart.size());
  int32_t outer = P.ring(xy, 0, outerEnd, true);
  // holes by their leftmost vertex, left to right
  std::vector<std::pair<double, int32_t>> holes;
  for (size_t k = 0; k < holeStart.size(); k++) {
    const uint32_t s = holeStart[k], e = k + 1 < holeStart.size() ? holeStart[k + 1] : nAll;
    if (e <= s) continue;
    const int32_t h = P.ring(xy, s, e, false);
    int32_t left = h, p = h;
    do {
      if (P.n[p].x < P.n[left].x || (P.n[p].x == P.n[left].x && P.n[p].y < P.n[left].y)) left = p;
      p = P.n[p].next;
    } while (p != h);
    holes.push_back({P.n[left].x, left});
  }
  // stable, as JavaScript's Array.prototype.sort that earcut relies on
  std::stable_sort(holes.begin(), holes.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  for (const auto& hv : holes) {
    const int32_t m = find_bridge(P, hv.second, outer);
    if (m < 0) return out;  // not clippable: the caller falls back
    P.bridge(m, hv.second);
  }
  // ear clipping over the single loop
  int32_t count = 0;
  {
    int32_t p = outer;
    do {
      count++;
      p = P.n[p].next;
    } while (p != outer);
  }
  out.reserve(3 * (size_t)std::max(count - 2, 0));
  int32_t ear = outer, stop = outer;
  bool flat = false;
  while (count > 3) {
    if (is_ear(P, ear, flat)) {
      const int32_t a = P.n[ear].prev, c = P.n[ear].next;
      out.push_back(P.n[a].i);
      out.push_back(P.n[ear].i);
      out.push_back(P.n[c].i);
      P.n[a].next = c;
      P.n[c].prev = a;
      count--;
      ear = c;
      stop = c;
      flat = false;
      continue;
    }
    ear = P.n[ear].next;
    if (ear == stop) {
      if (flat) return out;  // no ear left: incomplete, the caller falls back
      flat = true;
    }
  }
  const int32_t a = P.n[ear].prev, c = P.n[ear].next;
  out.push_back(P.n[a].i);
  out.push_back(P.n[ear].i);
  out.push_back(P.n[c].i);
  return out;
}

// ---------------------------------------------------------------------------
// capped cut

namespace {

inline uint64_t ekey(uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | b; }

struct Cap {
  std::vector<double>& xyz;
  std::vector<uint32_t>& tris;
  double n[3];
  double dir;
  const double* basis_u;
  const double* basis_v;

  // centroid fan: cap triangle (c, q, p) twins each loop edge p -> q
  void fan(const std::vector<uint32_t>& loop) {
    double cx = 0, cy = 0, cz = 0;
    for (uint32_t v : loop) {
      cx += xyz[3 * (size_t)v];
      cy += xyz[3 * (size_t)v + 1];
      cz += xyz[3 * (size_t)v + 2];
    }
    const uint32_t c = (uint32_t)(xyz.size() / 3);
    const double len = (double)loop.size();
    xyz.push_back(cx / len);
    xyz.push_back(cy / len);
    xyz.push_back(cz / len);
    for (size_t k = 0; k < loop.size(); k++) {
      tris.push_back(c);
      tris.push_back(loop[(k + 1) % loop.size()]);
      tris.push_back(loop[k]);
    }
  }
  double tri_normal_dot(uint32_t i0, uint32_t i1, uint32_t i2) const {
    const double* p0 = &xyz[3 * (size_t)i0];
    const double* p1 = &xyz[3 * (size_t)i1];
    const double* p2 = &xyz[3 * (size_t)i2];
    const double ax = p1[0] - p0[0], ay = p1[1] - p0[1], az = p1[2] - p0[2];
    const double bx = p2[0] - p0[0], by = p2[1] - p0[1], bz = p2[2] - p0[2];
    const double cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
    return cx * n[0] + cy * n[1] + cz * n[2];
  }

  const char* run() {
    // boundary edges: directed edges without a reverse twin, in first-seen
    // order, each distinct edge once. The directed edges are grouped by
    // source vertex (counting sort, each group in edge order), so a repeat
    // and a twin are found in the short lists of the edge's two vertices.
    const size_t ne = tris.size();
    const uint32_t nvx = (uint32_t)(xyz.size() / 3);
    std::vector<uint32_t> off(nvx + 1, 0), dst(ne), fill;
    for (size_t i = 0; i < ne; i++) off[tris[i] + 1]++;
    for (uint32_t v = 0; v < nvx; v++) off[v + 1] += off[v];
    fill.assign(off.begin(), off.end() - 1);
    for (size_t i = 0; i < ne; i += 3)
      for (int e = 0; e < 3; e++) dst[fill[tris[i + e]]++] = tris[i + (e + 1) % 3];
    std::fill(fill.begin(), fill.end(), 0u);
    std::vector<uint64_t> order;
    for (size_t i = 0; i < ne; i += 3)
      for (int e = 0; e < 3; e++) {
        const uint32_t a = tris[i + e], b = tris[i + (e + 1) % 3];
        // this edge's place in a's list; an earlier a -> b there is a repeat
        const uint32_t at = off[a] + fill[a]++;
        bool seen = false;
        for (uint32_t k = off[a]; k < at && !seen; k++) seen = dst[k] == b;
        if (seen) continue;
        bool twin = false;
        for (uint32_t k = off[b]; k < off[b + 1] && !twin; k++) twin = dst[k] == a;
        if (!twin) order.push_back(ekey(a, b));
      }
    std::vector<uint32_t> starts;
    std::unordered_map<uint32_t, std::vector<uint32_t>> next;
    size_t nBoundary = 0;
    for (uint64_t k : order) {
      const uint32_t a = (uint32_t)(k >> 32), b = (uint32_t)k;
      nBoundary++;
      auto it = next.find(a);
      if (it == next.end()) {
        starts.push_back(a);
        it = next.emplace(a, std::vector<uint32_t>()).first;
      }
      it->second.push_back(b);
    }
    if (nBoundary == 0) return nullptr;
    // boundary loops
    std::vector<std::vector<uint32_t>> loops;
    std::unordered_set<uint64_t> used;
    for (uint32_t start : starts) {
      const std::vector<uint32_t> outs = next[start];
      for (uint32_t first : outs) {
        if (used.count(ekey(start, first))) continue;
        std::vector<uint32_t> loop{start};
        uint32_t cur = first;
        used.insert(ekey(start, first));
        size_t guard = 0;
        while (cur != start) {
          loop.push_back(cur);
          auto it = next.find(cur);
          if (it == next.end()) return "open boundary chain";
          int64_t nx = -1;
          for (uint32_t cnd : it->second)
            if (!used.count(ekey(cur, cnd))) {
              nx = cnd;
              break;
            }
          if (nx < 0) return "boundary chain dead end";
          used.insert(ekey(cur, (uint32_t)nx));
          cur = (uint32_t)nx;
          if (++guard > nBoundary + 1) return "boundary chain cycle";
        }
        if (loop.size() >= 3) loops.push_back(std::move(loop));
      }
    }
    if (loops.empty()) return nullptr;
    // a 2-D basis of the plane
    const double* u = basis_u;
    const double* v = basis_v;
    const size_t L = loops.size();
    std::vector<std::vector<double>> l2(L);
    std::vector<double> area(L);
    for (size_t i = 0; i < L; i++) {
      for (uint32_t q : loops[i]) {
        const double x = xyz[3 * (size_t)q], y = xyz[3 * (size_t)q + 1], z = xyz[3 * (size_t)q + 2];
        l2[i].push_back(x * u[0] + y * u[1] + z * u[2]);
        l2[i].push_back(x * v[0] + y * v[1] + z * v[2]);
      }
      double s = 0;
      const size_t m = loops[i].size();
      for (size_t k = 0; k < m; k++) {
        const size_t j = (k + 1) % m;
        s += l2[i][2 * k] * l2[i][2 * j + 1] - l2[i][2 * j] * l2[i][2 * k + 1];
      }
      area[i] = s / 2;
    }
    // outer loops wind like the largest loop; a hole's parent is the smallest
    // larger outer loop containing the hole's area centroid
    std::vector<int> depth(L, 0);
    std::vector<int64_t> parent(L, -1);
    int64_t largest = -1;
    for (size_t i = 0; i < L; i++)
      if (largest < 0 || std::fabs(area[i]) > std::fabs(area[(size_t)largest])) largest = (int64_t)i;
    auto sgn = [](double x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); };
    const int outerSign = largest >= 0 ? sgn(area[(size_t)largest]) : 1;
    for (size_t i = 0; i < L; i++) {
      if (std::fabs(area[i]) < 1e-18) continue;
      if (sgn(area[i]) == outerSign) continue;
      depth[i] = 1;
      double cx, cy;
      {
        const std::vector<double>& p = l2[i];
        const size_t m = loops[i].size();
        double sx = 0, sy = 0;
        for (size_t k = 0; k < m; k++) {
          const size_t j = (k + 1) % m;
          const double w = p[2 * k] * p[2 * j + 1] - p[2 * j] * p[2 * k + 1];
          sx += (p[2 * k] + p[2 * j]) * w;
          sy += (p[2 * k + 1] + p[2 * j + 1]) * w;
        }
        cx = sx / (6 * area[i]);
        cy = sy / (6 * area[i]);
      }
      double bestArea = INFINITY, fallbackArea = -INFINITY;
      int64_t fallback = -1;
      for (size_t j = 0; j < L; j++) {
        if (i == j || std::fabs(area[j]) < 1e-18 || sgn(area[j]) != outerSign) continue;
        if (std::fabs(area[j]) > fallbackArea) {
          fallbackArea = std::fabs(area[j]);
          fallback = (int64_t)j;
        }
        if (std::fabs(area[j]) <= std::fabs(area[i])) continue;
        // crossing-number test of the centroid against loop j
        bool inside = false;
        const std::vector<double>& p = l2[j];
        const size_t m = loops[j].size();
        for (size_t a = 0, b = m - 1; a < m; b = a++) {
          const double xi = p[2 * a], yi = p[2 * a + 1], xj = p[2 * b], yj = p[2 * b + 1];
          if ((yi > cy) != (yj > cy) && cx < (xj - xi) * (cy - yi) / (yj - yi) + xi) inside = !inside;
        }
        if (inside && std::fabs(area[j]) < bestArea) {
          bestArea = std::fabs(area[j]);
          parent[i] = (int64_t)j;
        }
      }
      if (parent[i] < 0) parent[i] = fallback;
    }
    for (size_t i = 0; i < L; i++)
      if (std::fabs(area[i]) < 1e-18) fan(loops[i]);
    for (size_t i = 0; i < L; i++) {
      if (std::fabs(area[i]) < 1e-18 || depth[i] % 2 != 0) continue;
      std::vector<double> ring(l2[i]);
      std::vector<uint32_t> ids(loops[i]);
      std::vector<uint32_t> holeStart;
      std::vector<size_t> group{i};
      for (size_t j = 0; j < L; j++) {
        if (parent[j] == (int64_t)i && depth[j] % 2 == 1 && std::fabs(area[j]) >= 1e-18) {
          holeStart.push_back((uint32_t)ids.size());
          ring.insert(ring.end(), l2[j].begin(), l2[j].end());
          ids.insert(ids.end(), loops[j].begin(), loops[j].end());
          group.push_back(j);
        }
      }
      const std::vector<uint32_t> tri = ear_clip(ring, holeStart);
      const size_t expected = ids.size() + 2 * holeStart.size() - 2;
      if (tri.size() / 3 != expected) {
        for (size_t j : group) fan(loops[j]);
        continue;
      }
      // one flip for the whole cap, decided by its largest triangle
      double bestAbs = 0, bestDot = 0;
      for (size_t k = 0; k < tri.size(); k += 3) {
        const double d = tri_normal_dot(ids[tri[k]], ids[tri[k + 1]], ids[tri[k + 2]]);
        if (std::fabs(d) > bestAbs) {
          bestAbs = std::fabs(d);
          bestDot = d;
        }
      }
      const bool flip = bestDot * dir < 0;
      for (size_t k = 0; k < tri.size(); k += 3) {
        tris.push_back(ids[tri[k]]);
        tris.push_back(ids[tri[k + (flip ? 2 : 1)]]);
        tris.push_back(ids[tri[k + (flip ? 1 : 2)]]);
      }
    }
    return nullptr;
  }
};

// unreferenced vertices dropped, vertices numbered by first use
Mesh compact(const std::vector<double>& xyz, const std::vector<uint32_t>& tris) {
  Mesh m;
  std::vector<int64_t> remap(xyz.size() / 3, -1);
  m.t.resize(tris.size());
  uint32_t nOut = 0;
  for (size_t i = 0; i < tris.size(); i++) {
    const uint32_t v = tris[i];
    if (remap[v] < 0) remap[v] = nOut++;
    m.t[i] = (uint32_t)remap[v];
  }
  m.v.resize(3 * (size_t)nOut);
  for (size_t v = 0; v < remap.size(); v++) {
    if (remap[v] < 0) continue;
    const size_t r = (size_t)remap[v];
    m.v[3 * r] = (float)xyz[3 * v];
    m.v[3 * r + 1] = (float)xyz[3 * v + 1];
    m.v[3 * r + 2] = (float)xyz[3 * v + 2];
  }
  return m;
}

}  // namespace

PlaneFrame plane_frame(const Plane& pl) {
  PlaneFrame f;
  double nlen = std::hypot(pl.a, pl.b, pl.c);
  if (!(nlen != 0)) nlen = 1;
  f.n[0] = pl.a / nlen;
  f.n[1] = pl.b / nlen;
  f.n[2] = pl.c / nlen;
  f.d = pl.d / nlen;
  const double* n = f.n;
  const double ax[3] = {std::fabs(n[0]) < 0.9 ? 1.0 : 0.0, std::fabs(n[0]) < 0.9 ? 0.0 : 1.0, 0.0};
  double u[3] = {ax[1] * n[2] - ax[2] * n[1], ax[2] * n[0] - ax[0] * n[2], ax[0] * n[1] - ax[1] * n[0]};
  double ul = std::hypot(u[0], u[1], u[2]);
  if (ul == 0) ul = 1;
  for (double& x : u) x /= ul;
  for (int a = 0; a < 3; a++) f.u[a] = u[a];
  f.v[0] = n[1] * u[2] - n[2] * u[1];
  f.v[1] = n[2] * u[0] - n[0] * u[2];
  f.v[2] = n[0] * u[1] - n[1] * u[0];
  return f;
}

CutResult plane_cut(const Mesh& m, const Plane& pl, double eps) {
  CutResult r;
  const size_t nv = m.nv(), nt = m.nt();
  const PlaneFrame fr = plane_frame(pl);
  const double* n = fr.n;
  const double dd = fr.d;
  const float* V = m.v.data();
  std::vector<double> dist(nv);
  std::vector<int8_t> sign(nv);
  bool anyPos = false, anyNeg = false;
  for (size_t i = 0; i < nv; i++) {
    const double v = n[0] * V[3 * i] + n[1] * V[3 * i + 1] + n[2] * V[3 * i + 2] + dd;
    dist[i] = v;
    sign[i] = v > eps ? 1 : (v < -eps ? -1 : 0);
    anyPos |= sign[i] > 0;
    anyNeg |= sign[i] < 0;
  }
  if (!anyPos || !anyNeg) {
    r.reason = "plane does not split";
    return r;
  }
  std::vector<double> xyz(m.v.begin(), m.v.end());
  std::unordered_map<uint64_t, uint32_t> isect;
  auto isect_idx = [&](uint32_t i, uint32_t j) {
    const uint32_t lo = std::min(i, j), hi = std::max(i, j);
    const uint64_t key = ekey(lo, hi);
    auto it = isect.find(key);
    if (it != isect.end()) return it->second;
    const double t = dist[lo] / (dist[lo] - dist[hi]);
    const uint32_t idx = (uint32_t)(xyz.size() / 3);
    for (int a = 0; a < 3; a++) {
      const double p = V[3 * (size_t)lo + a], q = V[3 * (size_t)hi + a];
      xyz.push_back(p + t * (q - p));
    }
    isect.emplace(key, idx);
    return idx;
  };
  std::vector<uint32_t> pos, neg;
  uint32_t poly[4];
  auto clip = [&](std::vector<uint32_t>& side, int keep, const uint32_t ids[3]) {
    // Sutherland-Hodgman on one triangle; on-plane vertices stay on both sides
    int np = 0;
    for (int k = 0; k < 3; k++) {
      const uint32_t p = ids[k], q = ids[(k + 1) % 3];
      const int sp = sign[p] * keep, sq = sign[q] * keep;
      if (sp >= 0) poly[np++] = p;
      if (sign[p] != 0 && sign[q] != 0 && sp * sq < 0) poly[np++] = isect_idx(p, q);
    }
    for (int k = 1; k + 1 < np; k++) {
      side.push_back(poly[0]);
      side.push_back(poly[k]);
      side.push_back(poly[k + 1]);
    }
  };
  for (size_t t = 0; t < nt; t++) {
    const uint32_t ids[3] = {m.t[3 * t], m.t[3 * t + 1], m.t[3 * t + 2]};
    const int s0 = sign[ids[0]], s1 = sign[ids[1]], s2 = sign[ids[2]];
    const bool hasPos = s0 > 0 || s1 > 0 || s2 > 0;
    const bool hasNeg = s0 < 0 || s1 < 0 || s2 < 0;
    // triangles in the plane are dropped: the caps replace them
    if (!hasPos && !hasNeg) continue;
    if (!hasNeg) {
      pos.insert(pos.end(), ids, ids + 3);
    } else if (!hasPos) {
      neg.insert(neg.end(), ids, ids + 3);
    } else {
      clip(pos, 1, ids);
      clip(neg, -1, ids);
    }
  }
  Cap cp{xyz, pos, {n[0], n[1], n[2]}, -1.0, fr.u, fr.v};
  if (const char* why = cp.run()) {
    r.reason = why;
    return r;
  }
  Cap cn{xyz, neg, {n[0], n[1], n[2]}, 1.0, fr.u, fr.v};
  if (const char* why = cn.run()) {
    r.reason = why;
    return r;
  }
  r.ok = true;
  r.pos = compact(xyz, pos);
  r.neg = compact(xyz, neg);
  return r;
}

}  // namespace host
}  // namespace cuacd
