// cpu_helpers.cpp — CPU restatements of the reference's CPU helpers, used as
// the parity checker for mesh-level properties and as the timed CPU
// baseline of candidate-cut evaluation:
//   * planeCut with cap triangulation (src/cpu/cut.ts:33-315)
//   * signedVolume / volume / isClosed / edgeCSR (src/mesh.ts:59-119)
//   * concaveEdgePlanes (src/cpu/concave.ts:25-92)
//   * per-candidate evaluation: capped cut, hull, volumes, rv, Hausdorff
//     (what the reference does for the persistent parts, decompose.ts:336-352)
//
// TEST INFRASTRUCTURE ONLY.
//
// The reference triangulates caps with earcut@3.0.1 (npm, absent here). This
// file uses its own ear clipper with hole bridging; the reference's own
// guard (n + 2h - 2 triangles, else centroid fans, cut.ts:219-224) keeps the
// result closed with an exact cap area, so volumes and closedness are pinned
// while the exact cap triangles are not.
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <vector>

#include "oracle.h"
#include "oracle_api.h"

namespace orc {

struct MeshD {
  std::vector<float> V;
  std::vector<uint32_t> T;
};

// ---------------- mesh.ts ----------------
double signed_volume(const float* v, const uint32_t* t, uint32_t nt) {
  if (nt == 0) return 0;
  double ox = v[0], oy = v[1], oz = v[2], s = 0;
  for (uint32_t i = 0; i < 3 * nt; i += 3) {
    uint32_t a = t[i] * 3, b = t[i + 1] * 3, c = t[i + 2] * 3;
    double ax = v[a] - ox, ay = v[a + 1] - oy, az = v[a + 2] - oz;
    double bx = v[b] - ox, by = v[b + 1] - oy, bz = v[b + 2] - oz;
    double cx = v[c] - ox, cy = v[c + 1] - oy, cz = v[c + 2] - oz;
    s += ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
  }
  return s / 6;
}

bool is_closed(uint32_t nv, const uint32_t* T, uint32_t nt) {
  std::vector<uint32_t> off(nv + 1, 0);
  for (uint32_t i = 0; i < 3 * nt; i++) {
    if (T[i] >= nv) return false;
    off[T[i] + 1]++;
  }
  for (uint32_t v = 0; v < nv; v++) off[v + 1] += off[v];
  std::vector<uint32_t> fill(off.begin(), off.end() - 1), dst(3 * (size_t)nt);
  for (uint32_t i = 0; i < 3 * nt; i += 3)
    for (int e = 0; e < 3; e++) dst[fill[T[i + e]]++] = T[i + (e + 1) % 3];
  auto count = [&](uint32_t a, uint32_t b) {
    int c = 0;
    for (uint32_t k = off[a]; k < off[a + 1]; k++) if (dst[k] == b) c++;
    return c;
  };
  for (uint32_t a = 0; a < nv; a++)
    for (uint32_t k = off[a]; k < off[a + 1]; k++) {
      uint32_t b = dst[k];
      if (count(a, b) != 1 || count(b, a) != 1) return false;
    }
  return true;
}

// ---------------- ear clipping with holes ----------------
struct P2 { double x, y; };
static double area2(P2 a, P2 b, P2 c) { return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x); }
static bool in_tri(P2 p, P2 a, P2 b, P2 c) {  // inclusive, for a CCW triangle
  return area2(a, b, p) >= 0 && area2(b, c, p) >= 0 && area2(c, a, p) >= 0;
}
static double ring_area(const std::vector<P2>& r) {
  double s = 0;
  for (size_t i = 0; i < r.size(); i++) { size_t j = (i + 1) % r.size(); s += r[i].x * r[j].y - r[j].x * r[i].y; }
  return s / 2;
}

// Triangulates an outer ring with holes. pts[k] and ids[k] describe every
// ring vertex (outer first, then each hole from holeStart[h]). Returns
// triangles as indices into ids; fewer than n + 2h - 2 means failure.
static std::vector<uint32_t> ear_clip(const std::vector<P2>& pts, const std::vector<uint32_t>& holeStart) {
  size_t nAll = pts.size();
  size_t outerEnd = holeStart.empty() ? nAll : holeStart[0];
  std::vector<uint32_t> ring;
  for (size_t i = 0; i < outerEnd; i++) ring.push_back((uint32_t)i);
  std::vector<P2> tmp;
  for (uint32_t i : ring) tmp.push_back(pts[i]);
  if (ring_area(tmp) < 0) std::reverse(ring.begin(), ring.end());
  // holes: clockwise, bridged from their rightmost vertex, rightmost hole first
  struct H { std::vector<uint32_t> v; double maxx; };
  std::vector<H> holes;
  for (size_t h = 0; h < holeStart.size(); h++) {
    size_t s = holeStart[h], e = h + 1 < holeStart.size() ? holeStart[h + 1] : nAll;
    H hh;
    for (size_t i = s; i < e; i++) hh.v.push_back((uint32_t)i);
    std::vector<P2> hp;
    for (uint32_t i : hh.v) hp.push_back(pts[i]);
    if (ring_area(hp) > 0) std::reverse(hh.v.begin(), hh.v.end());
    hh.maxx = -INFINITY;
    for (uint32_t i : hh.v) hh.maxx = std::max(hh.maxx, pts[i].x);
    holes.push_back(hh);
  }
  std::sort(holes.begin(), holes.end(), [](const H& a, const H& b) { return a.maxx > b.maxx; });
  for (const H& hh : holes) {
    size_t mi = 0;
    for (size_t i = 1; i < hh.v.size(); i++) if (pts[hh.v[i]].x > pts[hh.v[mi]].x) mi = i;
    P2 M = pts[hh.v[mi]];
    // closest ring vertex visible from M along +x (nearest intersection edge endpoint)
    double bestX = INFINITY;
    long bestK = -1;
    for (size_t k = 0; k < ring.size(); k++) {
      P2 a = pts[ring[k]], b = pts[ring[(k + 1) % ring.size()]];
      if ((a.y > M.y) == (b.y > M.y)) continue;
      double x = a.x + (M.y - a.y) * (b.x - a.x) / (b.y - a.y);
      if (x >= M.x && x < bestX) { bestX = x; bestK = (long)(a.x > b.x ? k : (k + 1) % ring.size()); }
    }
    if (bestK < 0) {  // fall back to the nearest ring vertex
      double bd = INFINITY;
      for (size_t k = 0; k < ring.size(); k++) {
        double dx = pts[ring[k]].x - M.x, dy = pts[ring[k]].y - M.y, d = dx * dx + dy * dy;
        if (d < bd) { bd = d; bestK = (long)k; }
      }
    }
    std::vector<uint32_t> ins;
    for (size_t i = 0; i <= hh.v.size(); i++) ins.push_back(hh.v[(mi + i) % hh.v.size()]);
    ins.push_back(ring[bestK]);
    ring.insert(ring.begin() + bestK + 1, ins.begin(), ins.end());
  }
  std::vector<uint32_t> out;
  size_t guard = 0;
  while (ring.size() > 3 && guard++ < 4 * nAll * nAll + 64) {
    bool clipped = false;
    size_t n = ring.size();
    for (size_t i = 0; i < n; i++) {
      uint32_t ia = ring[(i + n - 1) % n], ib = ring[i], ic = ring[(i + 1) % n];
      P2 a = pts[ia], b = pts[ib], c = pts[ic];
      if (area2(a, b, c) <= 0) continue;
      bool ok = true;
      for (size_t k = 0; k < n && ok; k++) {
        uint32_t ip = ring[k];
        if (ip == ia || ip == ib || ip == ic) continue;
        P2 p = pts[ip];
        if ((p.x == a.x && p.y == a.y) || (p.x == b.x && p.y == b.y) || (p.x == c.x && p.y == c.y)) continue;
        if (in_tri(p, a, b, c)) ok = false;
      }
      if (!ok) continue;
      out.push_back(ia); out.push_back(ib); out.push_back(ic);
      ring.erase(ring.begin() + i);
      clipped = true;
      break;
    }
    if (!clipped) break;
  }
  if (ring.size() == 3) { out.push_back(ring[0]); out.push_back(ring[1]); out.push_back(ring[2]); }
  return out;
}

// ---------------- cut.ts ----------------
typedef double Vec3[3];

static void fan_loop(std::vector<double>& xyz, std::vector<uint32_t>& tris, const std::vector<uint32_t>& loop) {
  double cx = 0, cy = 0, cz = 0;
  for (uint32_t v : loop) { cx += xyz[3 * v]; cy += xyz[3 * v + 1]; cz += xyz[3 * v + 2]; }
  uint32_t c = (uint32_t)(xyz.size() / 3);
  xyz.push_back(cx / loop.size()); xyz.push_back(cy / loop.size()); xyz.push_back(cz / loop.size());
  for (size_t k = 0; k < loop.size(); k++) {
    uint32_t p = loop[k], q = loop[(k + 1) % loop.size()];
    tris.push_back(c); tris.push_back(q); tris.push_back(p);
  }
}

static bool point_in_poly(P2 pt, const std::vector<P2>& poly) {
  bool inside = false;
  for (size_t i = 0, j = poly.size() - 1; i < poly.size(); j = i++) {
    double xi = poly[i].x, yi = poly[i].y, xj = poly[j].x, yj = poly[j].y;
    if ((yi > pt.y) != (yj > pt.y) && pt.x < (xj - xi) * (pt.y - yi) / (yj - yi) + xi) inside = !inside;
  }
  return inside;
}

// cut.ts:110-240
static bool cap(std::vector<double>& xyz, std::vector<uint32_t>& tris, const Vec3 n, double capDir) {
  auto key = [](uint64_t a, uint64_t b) { return a * 4294967296ull + b; };
  std::unordered_map<uint64_t, int> edges;
  std::vector<uint64_t> edgeOrder;
  for (size_t i = 0; i < tris.size(); i += 3)
    for (int e = 0; e < 3; e++) {
      uint64_t k = key(tris[i + e], tris[i + (e + 1) % 3]);
      if (edges.emplace(k, 1).second) edgeOrder.push_back(k);
    }
  std::unordered_map<uint32_t, std::vector<uint32_t>> next;
  std::vector<uint32_t> starts;
  size_t nBoundary = 0;
  for (uint64_t k : edgeOrder) {
    uint32_t a = (uint32_t)(k / 4294967296ull), b = (uint32_t)(k % 4294967296ull);
    if (!edges.count(key(b, a))) {
      nBoundary++;
      auto it = next.find(a);
      if (it == next.end()) { next[a] = {b}; starts.push_back(a); } else it->second.push_back(b);
    }
  }
  if (nBoundary == 0) return true;
  std::vector<std::vector<uint32_t>> loops;
  std::unordered_map<uint64_t, char> used;
  for (uint32_t start : starts) {
    std::vector<uint32_t> outs = next[start];
    for (uint32_t first : outs) {
      if (used.count(key(start, first))) continue;
      std::vector<uint32_t> loop{start};
      uint32_t cur = first;
      used[key(start, first)] = 1;
      size_t guard = 0;
      while (cur != start) {
        loop.push_back(cur);
        auto it = next.find(cur);
        if (it == next.end()) return false;
        long nxt = -1;
        for (uint32_t c : it->second) if (!used.count(key(cur, c))) { nxt = c; break; }
        if (nxt < 0) return false;
        used[key(cur, (uint32_t)nxt)] = 1;
        cur = (uint32_t)nxt;
        if (++guard > nBoundary + 1) return false;
      }
      if (loop.size() >= 3) loops.push_back(loop);
    }
  }
  if (loops.empty()) return true;
  Vec3 ax = {std::fabs(n[0]) < 0.9 ? 1.0 : 0.0, std::fabs(n[0]) < 0.9 ? 0.0 : 1.0, 0.0};
  Vec3 u = {ax[1] * n[2] - ax[2] * n[1], ax[2] * n[0] - ax[0] * n[2], ax[0] * n[1] - ax[1] * n[0]};
  double ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  if (ul == 0) ul = 1;
  for (double& c : u) c /= ul;
  Vec3 v = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2], n[0] * u[1] - n[1] * u[0]};
  auto project = [&](uint32_t i) {
    double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    return P2{x * u[0] + y * u[1] + z * u[2], x * v[0] + y * v[1] + z * v[2]};
  };
  size_t L = loops.size();
  std::vector<std::vector<P2>> l2(L);
  std::vector<double> areas(L);
  for (size_t i = 0; i < L; i++) {
    for (uint32_t p : loops[i]) l2[i].push_back(project(p));
    areas[i] = ring_area(l2[i]);
  }
  std::vector<int> depth(L, 0), parent(L, -1);
  long largest = -1;
  for (size_t i = 0; i < L; i++) if (largest < 0 || std::fabs(areas[i]) > std::fabs(areas[largest])) largest = (long)i;
  double outerSign = largest >= 0 ? (areas[largest] > 0 ? 1 : (areas[largest] < 0 ? -1 : 0)) : 1;
  auto sgn = [](double a) { return a > 0 ? 1.0 : (a < 0 ? -1.0 : 0.0); };
  for (size_t i = 0; i < L; i++) {
    if (std::fabs(areas[i]) < 1e-18) continue;
    if (sgn(areas[i]) == outerSign) continue;
    depth[i] = 1;
    // centroid of the hole
    double cx = 0, cy = 0;
    const auto& p = l2[i];
    for (size_t a = 0; a < p.size(); a++) {
      size_t b = (a + 1) % p.size();
      double w = p[a].x * p[b].y - p[b].x * p[a].y;
      cx += (p[a].x + p[b].x) * w;
      cy += (p[a].y + p[b].y) * w;
    }
    P2 c{cx / (6 * areas[i]), cy / (6 * areas[i])};
    double bestArea = INFINITY, fallbackArea = -INFINITY;
    int fallback = -1;
    for (size_t j = 0; j < L; j++) {
      if (i == j || std::fabs(areas[j]) < 1e-18 || sgn(areas[j]) != outerSign) continue;
      if (std::fabs(areas[j]) > fallbackArea) { fallbackArea = std::fabs(areas[j]); fallback = (int)j; }
      if (std::fabs(areas[j]) <= std::fabs(areas[i])) continue;
      if (point_in_poly(c, l2[j]) && std::fabs(areas[j]) < bestArea) { bestArea = std::fabs(areas[j]); parent[i] = (int)j; }
    }
    if (parent[i] < 0) parent[i] = fallback;
  }
  for (size_t i = 0; i < L; i++) if (std::fabs(areas[i]) < 1e-18) fan_loop(xyz, tris, loops[i]);
  for (size_t i = 0; i < L; i++) {
    if (std::fabs(areas[i]) < 1e-18 || depth[i] % 2 != 0) continue;
    std::vector<P2> ring;
    std::vector<uint32_t> ids, holeStart;
    for (size_t k = 0; k < loops[i].size(); k++) { ring.push_back(l2[i][k]); ids.push_back(loops[i][k]); }
    std::vector<size_t> group{i};
    for (size_t j = 0; j < L; j++) {
      if (parent[j] == (int)i && depth[j] % 2 == 1 && std::fabs(areas[j]) >= 1e-18) {
        holeStart.push_back((uint32_t)ids.size());
        for (size_t k = 0; k < loops[j].size(); k++) { ring.push_back(l2[j][k]); ids.push_back(loops[j][k]); }
        group.push_back(j);
      }
    }
    std::vector<uint32_t> tri = ear_clip(ring, holeStart);
    size_t expected = ids.size() + 2 * holeStart.size() - 2;
    if (tri.size() / 3 != expected) {
      for (size_t j : group) fan_loop(xyz, tris, loops[j]);
      continue;
    }
    double bestAbs = 0, bestDot = 0;
    for (size_t k = 0; k < tri.size(); k += 3) {
      uint32_t i0 = ids[tri[k]], i1 = ids[tri[k + 1]], i2 = ids[tri[k + 2]];
      double ax2 = xyz[3 * i1] - xyz[3 * i0], ay = xyz[3 * i1 + 1] - xyz[3 * i0 + 1], az = xyz[3 * i1 + 2] - xyz[3 * i0 + 2];
      double bx = xyz[3 * i2] - xyz[3 * i0], by = xyz[3 * i2 + 1] - xyz[3 * i0 + 1], bz = xyz[3 * i2 + 2] - xyz[3 * i0 + 2];
      double cx = ay * bz - az * by, cy = az * bx - ax2 * bz, cz = ax2 * by - ay * bx;
      double d = cx * n[0] + cy * n[1] + cz * n[2];
      if (std::fabs(d) > bestAbs) { bestAbs = std::fabs(d); bestDot = d; }
    }
    bool flip = bestDot * capDir < 0;
    for (size_t k = 0; k < tri.size(); k += 3) {
      uint32_t i0 = ids[tri[k]], i1 = ids[tri[k + 1]], i2 = ids[tri[k + 2]];
      if (flip) std::swap(i1, i2);
      tris.push_back(i0); tris.push_back(i1); tris.push_back(i2);
    }
  }
  return true;
}

static MeshD compact(const std::vector<double>& xyz, const std::vector<uint32_t>& tris) {
  std::vector<int64_t> remap(xyz.size() / 3, -1);
  MeshD m;
  m.T.resize(tris.size());
  uint32_t nvOut = 0;
  for (size_t i = 0; i < tris.size(); i++) {
    uint32_t v = tris[i];
    if (remap[v] < 0) remap[v] = nvOut++;
    m.T[i] = (uint32_t)remap[v];
  }
  m.V.assign(3 * (size_t)nvOut, 0);
  for (size_t v = 0; v < remap.size(); v++) {
    if (remap[v] < 0) continue;
    for (int a = 0; a < 3; a++) m.V[3 * remap[v] + a] = (float)xyz[3 * v + a];
  }
  return m;
}

// cut.ts:33-107; returns 0 on success
int plane_cut(const float* V, uint32_t nv, const uint32_t* T, uint32_t nt, const double plane[4], MeshD& pos, MeshD& neg,
              double eps = 1e-6) {
  double nlen = std::sqrt(plane[0] * plane[0] + plane[1] * plane[1] + plane[2] * plane[2]);
  if (nlen == 0) nlen = 1;
  Vec3 n = {plane[0] / nlen, plane[1] / nlen, plane[2] / nlen};
  double dd = plane[3] / nlen;
  std::vector<double> dist(nv);
  std::vector<int8_t> sign(nv);
  bool anyPos = false, anyNeg = false;
  for (uint32_t i = 0; i < nv; i++) {
    double d = n[0] * V[3 * i] + n[1] * V[3 * i + 1] + n[2] * V[3 * i + 2] + dd;
    dist[i] = d;
    sign[i] = d > eps ? 1 : (d < -eps ? -1 : 0);
    anyPos |= sign[i] > 0;
    anyNeg |= sign[i] < 0;
  }
  if (!anyPos || !anyNeg) return 1;
  std::vector<double> xyz(V, V + 3 * (size_t)nv);
  std::unordered_map<uint64_t, uint32_t> isect;
  auto isectIdx = [&](uint32_t i, uint32_t j) {
    uint32_t lo = std::min(i, j), hi = std::max(i, j);
    uint64_t k = (uint64_t)lo * 4294967296ull + hi;
    auto it = isect.find(k);
    if (it != isect.end()) return it->second;
    double t = dist[lo] / (dist[lo] - dist[hi]);
    uint32_t idx = (uint32_t)(xyz.size() / 3);
    for (int a = 0; a < 3; a++) xyz.push_back(V[3 * lo + a] + t * ((double)V[3 * hi + a] - V[3 * lo + a]));
    isect[k] = idx;
    return idx;
  };
  std::vector<uint32_t> pt, ngt;
  auto clip = [&](std::vector<uint32_t>& side, int keep, uint32_t i0, uint32_t i1, uint32_t i2) {
    uint32_t ids[3] = {i0, i1, i2};
    std::vector<uint32_t> poly;
    for (int k = 0; k < 3; k++) {
      uint32_t p = ids[k], q = ids[(k + 1) % 3];
      int sp = sign[p] * keep, sq = sign[q] * keep;
      if (sp >= 0) poly.push_back(p);
      if (sign[p] != 0 && sign[q] != 0 && sp * sq < 0) poly.push_back(isectIdx(p, q));
    }
    for (size_t k = 1; k + 1 < poly.size(); k++) { side.push_back(poly[0]); side.push_back(poly[k]); side.push_back(poly[k + 1]); }
  };
  for (uint32_t t = 0; t < nt; t++) {
    uint32_t i0 = T[3 * t], i1 = T[3 * t + 1], i2 = T[3 * t + 2];
    int s0 = sign[i0], s1 = sign[i1], s2 = sign[i2];
    bool hasPos = s0 > 0 || s1 > 0 || s2 > 0, hasNeg = s0 < 0 || s1 < 0 || s2 < 0;
    if (!hasPos && !hasNeg) continue;
    if (!hasNeg) { pt.push_back(i0); pt.push_back(i1); pt.push_back(i2); }
    else if (!hasPos) { ngt.push_back(i0); ngt.push_back(i1); ngt.push_back(i2); }
    else { clip(pt, 1, i0, i1, i2); clip(ngt, -1, i0, i1, i2); }
  }
  if (!cap(xyz, pt, n, -1)) return 2;
  if (!cap(xyz, ngt, n, +1)) return 3;
  pos = compact(xyz, pt);
  neg = compact(xyz, ngt);
  return 0;
}

// ---------------- concave.ts ----------------
static bool face_normal(const float* V, const uint32_t* T, uint32_t f, double out[3]) {
  uint32_t a = T[3 * f] * 3, b = T[3 * f + 1] * 3, c = T[3 * f + 2] * 3;
  double e1x = (double)V[b] - V[a], e1y = (double)V[b + 1] - V[a + 1], e1z = (double)V[b + 2] - V[a + 2];
  double e2x = (double)V[c] - V[a], e2y = (double)V[c + 1] - V[a + 1], e2z = (double)V[c + 2] - V[a + 2];
  double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  double l = std::sqrt(nx * nx + ny * ny + nz * nz);
  if (l < 1e-12) return false;
  out[0] = nx / l; out[1] = ny / l; out[2] = nz / l;
  return true;
}

std::vector<float> concave_planes(const float* V, uint32_t nv, const uint32_t* T, uint32_t nt, int nConcaveEdges,
                                  double concaveEps, double concaveThreshold, uint32_t seed) {
  std::vector<float> out;
  if (nConcaveEdges <= 0 || nt == 0) return out;
  std::vector<uint32_t> off(nv + 1, 0);
  for (uint32_t i = 0; i < 3 * nt; i++) off[T[i] + 1]++;
  for (uint32_t v = 0; v < nv; v++) off[v + 1] += off[v];
  std::vector<uint32_t> fill(off.begin(), off.end() - 1), dst(3 * (size_t)nt), face(3 * (size_t)nt);
  for (uint32_t i = 0; i < 3 * nt; i += 3)
    for (int e = 0; e < 3; e++) {
      uint32_t a = T[i + e], b = T[i + (e + 1) % 3];
      uint32_t k = fill[a]++;
      dst[k] = b;
      face[k] = i / 3;
    }
  auto findFace = [&](uint32_t a, uint32_t b) -> long {
    for (uint32_t k = off[a]; k < off[a + 1]; k++) if (dst[k] == b) return (long)face[k];
    return -1;
  };
  uint32_t rng = seed;
  auto lcg = [&]() { rng = rng * 1664525u + 1013904223u; return rng; };
  struct R { uint32_t v0, v1, f0, f1; };
  std::vector<R> reservoir;
  uint64_t seen = 0;
  std::vector<uint32_t> partners;
  for (uint32_t v0 = 0; v0 < nv; v0++) {
    partners.clear();
    for (uint32_t k = off[v0]; k < off[v0 + 1]; k++) {
      uint32_t b = dst[k];
      if (b > v0 && std::find(partners.begin(), partners.end(), b) == partners.end()) partners.push_back(b);
    }
    std::sort(partners.begin(), partners.end());
    for (uint32_t v1 : partners) {
      long fa = findFace(v0, v1), fb = findFace(v1, v0);
      if (fa < 0 || fb < 0) continue;
      uint32_t f0 = (uint32_t)std::min(fa, fb), f1 = (uint32_t)std::max(fa, fb);
      double n0[3], n1[3];
      if (!face_normal(V, T, f0, n0) || !face_normal(V, T, f1, n1)) continue;
      double cosA = n0[0] * n1[0] + n0[1] * n1[1] + n0[2] * n1[2];
      cosA = std::max(-1.0, std::min(1.0, cosA));
      double alpha = std::acos(cosA);
      long vOther = -1;
      for (int i = 0; i < 3; i++) { uint32_t vv = T[3 * f0 + i]; if (vv != v0 && vv != v1) { vOther = vv; break; } }
      if (vOther < 0) continue;
      double dx = (double)V[3 * vOther] - V[3 * v0], dy = (double)V[3 * vOther + 1] - V[3 * v0 + 1], dz = (double)V[3 * vOther + 2] - V[3 * v0 + 2];
      double d = dx * n1[0] + dy * n1[1] + dz * n1[2];
      double dihedral = d > 0 ? M_PI + alpha : M_PI - alpha;
      if (!(dihedral > concaveThreshold)) continue;
      seen++;
      if ((int)reservoir.size() < nConcaveEdges) reservoir.push_back(R{v0, v1, f0, f1});
      else {
        uint32_t r = lcg();
        double thresh = std::floor((double)nConcaveEdges / (double)seen * 4294967295.0);
        if ((double)r < thresh) {
          uint32_t slot = lcg() % (uint32_t)nConcaveEdges;
          reservoir[slot] = R{v0, v1, f0, f1};
        }
      }
    }
  }
  for (const R& e : reservoir) {
    double n0[3], n1[3];
    if (!face_normal(V, T, e.f0, n0) || !face_normal(V, T, e.f1, n1)) continue;
    double mx = ((double)V[3 * e.v0] + V[3 * e.v1]) / 2, my = ((double)V[3 * e.v0 + 1] + V[3 * e.v1 + 1]) / 2,
           mz = ((double)V[3 * e.v0 + 2] + V[3 * e.v1 + 2]) / 2;
    double eps = concaveEps;
    auto push = [&](double a, double b, double c, double d) { out.push_back((float)a); out.push_back((float)b); out.push_back((float)c); out.push_back((float)d); };
    push(n1[0], n1[1], n1[2], -(n1[0] * mx + n1[1] * my + n1[2] * mz + eps));
    push(n0[0], n0[1], n0[2], -(n0[0] * mx + n0[1] * my + n0[2] * mz + eps));
    double bx = n0[0] + n1[0], by = n0[1] + n1[1], bz = n0[2] + n1[2];
    double bl = std::sqrt(bx * bx + by * by + bz * bz);
    if (bl >= 1e-4) {
      bx /= bl; by /= bl; bz /= bl;
      push(bx, by, bz, -(bx * mx + by * my + bz * mz + eps));
      push(bx, by, bz, -(bx * mx + by * my + bz * mz - eps));
    }
  }
  return out;
}

// ---------------- reference quickhull (oracle/_ref), when built ----------------
typedef int (*qh_fn)(const double* pts, int n, double eps, double* vOut, int vCap, uint32_t* tOut, int tCap, int* nvOut);
static qh_fn g_qh = nullptr;

// Hull volume and faces of a point set: the reference's quickhull when it is
// loaded, else the oracle's grid hull. Faces index the input points.
double hull_volume_cpu(const float* V, uint32_t nv, std::vector<uint32_t>* faces, bool useRef) {
  if (nv < 4) return 0.0;
  if (useRef && g_qh) {
    std::vector<double> pts(V, V + 3 * (size_t)nv), hv(3 * (size_t)nv);
    std::vector<uint32_t> ht(6 * (size_t)nv + 12);
    int hn = 0;
    int ntri = g_qh(pts.data(), (int)nv, 1e-7, hv.data(), (int)nv, ht.data(), (int)ht.size() / 3, &hn);
    if (ntri <= 0) return 0.0;
    std::vector<float> hvf(hv.begin(), hv.begin() + 3 * hn);
    double sv = signed_volume(hvf.data(), ht.data(), (uint32_t)ntri);
    if (faces) faces->clear();  // quickhull faces index its own compacted vertices
    return std::fabs(sv);
  }
  std::vector<f3> pts(nv);
  for (uint32_t i = 0; i < nv; i++) pts[i] = mk3(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
  uint32_t fmax = 2 * std::min(nv, 4096u) + 3 * ORC_VIS_MAX + 1024;
  uint32_t slab = ((2 * nv + std::max(nv, 80u) + 7) & ~7u) + 16 * fmax;
  HullOpts o;
  HullResult r = hull_points(pts.data(), nv, slab, o);
  if (faces) *faces = r.faces;
  return r.hullVol < 0 ? 0.0 : (double)r.hullVol;
}

double hausdorff_cpu(const orc_mesh& a, const orc_mesh& b);

}  // namespace orc

using namespace orc;

extern "C" {

int orc_load_qh_ref(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  g_qh = (qh_fn)dlsym(h, "qhref_compute");
  return g_qh ? 0 : -2;
}
int orc_qh_ref_loaded(void) { return g_qh ? 1 : 0; }

double orc_signed_volume(const orc_mesh* m) { return signed_volume(m->verts, m->tris, m->nt); }
int orc_is_closed(const orc_mesh* m) { return is_closed(m->nv, m->tris, m->nt) ? 1 : 0; }

// Capped plane cut. Outputs are written into caller buffers of the given
// capacities; counts are returned through the n* pointers. Returns 0 on
// success, 1 when the plane does not split, 2/3 when a cap fails, -1 when a
// buffer is too small.
int orc_plane_cut(const orc_mesh* m, const double* plane, float* posV, uint32_t* posT, float* negV, uint32_t* negT,
                  uint32_t vCap, uint32_t tCap, uint32_t* nOut) {
  MeshD p, n;
  int rc = plane_cut(m->verts, m->nv, m->tris, m->nt, plane, p, n);
  if (rc) return rc;
  uint32_t pnv = (uint32_t)p.V.size() / 3, pnt = (uint32_t)p.T.size() / 3, nnv = (uint32_t)n.V.size() / 3, nnt = (uint32_t)n.T.size() / 3;
  nOut[0] = pnv; nOut[1] = pnt; nOut[2] = nnv; nOut[3] = nnt;
  if (pnv > vCap || nnv > vCap || pnt > tCap || nnt > tCap) return -1;
  std::memcpy(posV, p.V.data(), 12ull * pnv); std::memcpy(posT, p.T.data(), 12ull * pnt);
  std::memcpy(negV, n.V.data(), 12ull * nnv); std::memcpy(negT, n.T.data(), 12ull * nnt);
  return 0;
}

int orc_concave_planes(const orc_mesh* m, int nConcaveEdges, double eps, double thresh, uint32_t seed, float* out, int cap) {
  std::vector<float> p = concave_planes(m->verts, m->nv, m->tris, m->nt, nConcaveEdges, eps, thresh, seed);
  int n = (int)p.size() / 4;
  for (int i = 0; i < n && i < cap; i++) std::memcpy(out + 4 * i, &p[4 * i], 16);
  return n;
}

double orc_hull_volume(const orc_mesh* m, int useRef) { return hull_volume_cpu(m->verts, m->nv, nullptr, useRef != 0); }

float orc_rv_cost(float meshVol, float hullVol) { return rv_cost(meshVol, hullVol); }

// Evaluates candidate planes of one mesh the way the reference's CPU helpers
// treat a part: capped cut, hull of each half, mesh and hull volume, rv and
// (when withHd) the Hausdorff distance of each half to its hull. Candidates
// are split over nThreads host threads. out holds 8 values per candidate:
// ok, volPos, volNeg, hullPos, hullNeg, rvPos, rvNeg, max(hdPos, hdNeg).
int orc_eval_candidates(const orc_mesh* m, const double* planes, int n, int nThreads, int withHd, int useRef, double* out) {
  std::atomic<int> next(0);
  auto work = [&]() {
    for (;;) {
      int k = next.fetch_add(1);
      if (k >= n) return;
      double* o = out + 8 * (size_t)k;
      std::memset(o, 0, 64);
      MeshD p, q;
      if (plane_cut(m->verts, m->nv, m->tris, m->nt, planes + 4 * (size_t)k, p, q) != 0) continue;
      o[0] = 1;
      MeshD* half[2] = {&p, &q};
      double hd = 0;
      for (int s = 0; s < 2; s++) {
        MeshD& h = *half[s];
        uint32_t hnv = (uint32_t)h.V.size() / 3, hnt = (uint32_t)h.T.size() / 3;
        double vol = std::fabs(signed_volume(h.V.data(), h.T.data(), hnt));
        std::vector<uint32_t> faces;
        double hv = hull_volume_cpu(h.V.data(), hnv, withHd ? &faces : nullptr, useRef != 0 && !withHd);
        o[1 + s] = vol;
        o[3 + s] = hv;
        o[5 + s] = rv_cost((float)vol, (float)hv);
        if (withHd && !faces.empty()) {
          orc_mesh a{h.V.data(), h.T.data(), hnv, hnt};
          orc_mesh b{h.V.data(), faces.data(), hnv, (uint32_t)faces.size() / 3};
          hd = std::max(hd, hausdorff_cpu(a, b));
        }
      }
      o[7] = hd;
    }
  };
  std::vector<std::thread> th;
  int nt = std::max(1, nThreads);
  for (int i = 1; i < nt; i++) th.emplace_back(work);
  work();
  for (auto& t : th) t.join();
  return 0;
}

}  // extern "C"
