// merge_oracle.cpp — CPU restatement of the merge pass (src/merge.ts):
//   * seamPlane (merge.ts:114-141): the face plane of A's hull that has all
//     of B's hull on its outer side and the most coplanar mesh area of A and
//     B, planes deduplicated by their rounded key (Math.round(x * 2000));
//   * filteredConcat (merge.ts:144-157): the concatenation of two meshes
//     without the triangles lying on any of the planes;
//   * mergeHulls (merge.ts:170-303): rounds of cheap rejections (rv of the
//     two hulls' gap, bounding-box gap below threshold / 2), merged hulls of
//     the surviving pairs (the hull of both hulls' points), the Hausdorff
//     distance of the seam-filtered union to the merged hull for pairs still
//     under the threshold, greedy min-cost matching (stable order), until a
//     round merges nothing.
// The merged hulls come from the oracle's grid hull (the restatement of the
// GPU hull kernel, hull_oracle.cpp) and the Hausdorff distances from its
// float32 restatement of hausdorff_shader.ts. The reference cleans each
// merged hull mesh with its CPU quickhull before the Hausdorff pass
// (merge.ts:213); the oracle keeps the raw hull faces, so its distances match
// within the Hausdorff tolerance, not bit for bit.
//
// TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "oracle.h"
#include "oracle_api.h"

namespace orc {

float hausdorff_gpu_pair(const orc_mesh& a, const orc_mesh& b, uint32_t cap);

namespace {

struct Pl {
  double a, b, c, d;
};

struct OPart {
  std::vector<float> V;
  std::vector<uint32_t> T;
  std::vector<float> HV;
  std::vector<uint32_t> HT;
  double meshVol = 0, hullVol = 0, hd = 0;
  bool hasHd = false;
  std::vector<Pl> seams;
  int merged = 1;
  int id = 0;
  std::vector<int> members;  // input parts held, in concatenation order
};

double rv(double meshVol, double hullVol) {
  return 0.3 * std::cbrt((3 / (4 * M_PI)) * std::max(hullVol - meshVol, 0.0));
}

// Math.round: the nearest integer, halves towards +infinity
int64_t js_round(double x) { return (int64_t)std::floor(x + 0.5); }

bool tri_on_plane(const float* V, const uint32_t* T, size_t t, const Pl& p, double tol) {
  for (int e = 0; e < 3; e++) {
    const size_t i = 3 * (size_t)T[t + e];
    if (std::fabs(p.a * V[i] + p.b * V[i + 1] + p.c * V[i + 2] + p.d) > tol) return false;
  }
  return true;
}

double coplanar_area(const std::vector<float>& V, const std::vector<uint32_t>& T, const Pl& p, double tol) {
  double area = 0;
  for (size_t t = 0; t < T.size(); t += 3) {
    if (!tri_on_plane(V.data(), T.data(), t, p, tol)) continue;
    const size_t a = 3 * (size_t)T[t], b = 3 * (size_t)T[t + 1], c = 3 * (size_t)T[t + 2];
    const double abx = V[b] - V[a], aby = V[b + 1] - V[a + 1], abz = V[b + 2] - V[a + 2];
    const double acx = V[c] - V[a], acy = V[c + 1] - V[a + 1], acz = V[c + 2] - V[a + 2];
    area += 0.5 * std::hypot(aby * acz - abz * acy, abz * acx - abx * acz, abx * acy - aby * acx);
  }
  return area;
}

bool seam(const OPart& A, const OPart& B, double tol, Pl& best) {
  const std::vector<float>& hv = A.HV;
  const std::vector<uint32_t>& ht = A.HT;
  std::vector<std::array<int64_t, 4>> seen;
  double bestArea = 0;
  bool found = false;
  for (size_t t = 0; t < ht.size(); t += 3) {
    const size_t i0 = 3 * (size_t)ht[t], i1 = 3 * (size_t)ht[t + 1], i2 = 3 * (size_t)ht[t + 2];
    const double e1x = (double)hv[i1] - hv[i0], e1y = (double)hv[i1 + 1] - hv[i0 + 1], e1z = (double)hv[i1 + 2] - hv[i0 + 2];
    const double e2x = (double)hv[i2] - hv[i0], e2y = (double)hv[i2 + 1] - hv[i0 + 1], e2z = (double)hv[i2 + 2] - hv[i0 + 2];
    double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    const double len = std::hypot(nx, ny, nz);
    if (len < 1e-20) continue;
    nx /= len;
    ny /= len;
    nz /= len;
    const double d = nx * hv[i0] + ny * hv[i0 + 1] + nz * hv[i0 + 2];
    const std::array<int64_t, 4> key{js_round(nx * 2000), js_round(ny * 2000), js_round(nz * 2000), js_round(d * 2000)};
    if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
    seen.push_back(key);
    bool outer = true;
    for (size_t j = 0; j < B.HV.size() && outer; j += 3)
      if (nx * B.HV[j] + ny * B.HV[j + 1] + nz * B.HV[j + 2] - d < -tol) outer = false;
    if (!outer) continue;
    const Pl p{nx, ny, nz, -d};
    const double area = coplanar_area(A.V, A.T, p, tol) + coplanar_area(B.V, B.T, p, tol);
    if (area > bestArea) {
      bestArea = area;
      best = p;
      found = true;
    }
  }
  return found;
}

void concat(const std::vector<float>& av, const std::vector<uint32_t>& at, const std::vector<float>& bv,
            const std::vector<uint32_t>& bt, std::vector<float>& V, std::vector<uint32_t>& T) {
  V = av;
  V.insert(V.end(), bv.begin(), bv.end());
  T = at;
  const uint32_t off = (uint32_t)(av.size() / 3);
  for (uint32_t x : bt) T.push_back(x + off);
}

std::vector<uint32_t> filtered(const std::vector<float>& V, const std::vector<uint32_t>& T, const std::vector<Pl>& planes,
                               double tol) {
  if (planes.empty()) return T;
  std::vector<uint32_t> out;
  for (size_t t = 0; t < T.size(); t += 3) {
    bool drop = false;
    for (const Pl& p : planes)
      if (tri_on_plane(V.data(), T.data(), t, p, tol)) {
        drop = true;
        break;
      }
    if (!drop) out.insert(out.end(), T.begin() + t, T.begin() + t + 3);
  }
  return out;
}

struct Eval {
  double cost = 0, hullVol = 0, hd = 0;
  bool hasHull = false, hasSeam = false;
  std::vector<float> hullV;
  std::vector<uint32_t> hullT;
  Pl seamP{0, 0, 0, 0};
};

void bbox(const std::vector<float>& V, float lo[3], float hi[3]) {
  for (int a = 0; a < 3; a++) {
    lo[a] = INFINITY;
    hi[a] = -INFINITY;
  }
  for (size_t i = 0; i < V.size(); i += 3)
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], V[i + a]);
      hi[a] = std::max(hi[a], V[i + a]);
    }
}

}  // namespace
}  // namespace orc

using namespace orc;

extern "C" {

typedef struct {
  orc_mesh mesh;
  orc_mesh hull;
  double meshVol, hullVol, hausdorff;
  const double* seams;
  uint32_t nSeams;
  int32_t merged;
} orc_part_in;

static OPart to_part(const orc_part_in& in, int id) {
  OPart p;
  p.V.assign(in.mesh.verts, in.mesh.verts + 3 * (size_t)in.mesh.nv);
  p.T.assign(in.mesh.tris, in.mesh.tris + 3 * (size_t)in.mesh.nt);
  p.HV.assign(in.hull.verts, in.hull.verts + 3 * (size_t)in.hull.nv);
  p.HT.assign(in.hull.tris, in.hull.tris + 3 * (size_t)in.hull.nt);
  p.meshVol = in.meshVol;
  p.hullVol = in.hullVol;
  p.hasHd = !std::isnan(in.hausdorff);
  p.hd = p.hasHd ? in.hausdorff : 0;
  for (uint32_t k = 0; k < in.nSeams; k++)
    p.seams.push_back(Pl{in.seams[4 * k], in.seams[4 * k + 1], in.seams[4 * k + 2], in.seams[4 * k + 3]});
  p.merged = in.merged > 0 ? in.merged : 1;
  p.id = id;
  p.members = {id};
  return p;
}

int orc_seam_plane(const orc_part_in* a, const orc_part_in* b, double tol, double* out4) {
  Pl p{0, 0, 0, 0};
  if (!seam(to_part(*a, 0), to_part(*b, 1), tol, p)) return 0;
  out4[0] = p.a;
  out4[1] = p.b;
  out4[2] = p.c;
  out4[3] = p.d;
  return 1;
}

int orc_filtered_concat(const orc_mesh* a, const orc_mesh* b, const double* planes, int nPlanes, double tol,
                        uint32_t* out, int cap) {
  std::vector<float> V;
  std::vector<uint32_t> T;
  concat(std::vector<float>(a->verts, a->verts + 3 * (size_t)a->nv), std::vector<uint32_t>(a->tris, a->tris + 3 * (size_t)a->nt),
         std::vector<float>(b->verts, b->verts + 3 * (size_t)b->nv), std::vector<uint32_t>(b->tris, b->tris + 3 * (size_t)b->nt),
         V, T);
  std::vector<Pl> pl;
  for (int k = 0; k < nPlanes; k++) pl.push_back(Pl{planes[4 * k], planes[4 * k + 1], planes[4 * k + 2], planes[4 * k + 3]});
  const std::vector<uint32_t> kept = filtered(V, T, pl, tol);
  const int n = (int)(kept.size() / 3);
  if (n > cap) return -1;
  std::copy(kept.begin(), kept.end(), out);
  return n;
}

// mergeHulls. Outputs: *nOut parts; memberStart[nOut + 1] and members[] (the
// input parts each output part holds, in concatenation order); per output
// part meshVol, hullVol, hd and its seam count; stats4 = rounds, merges,
// pairsHulled, pairsHausdorff. Returns 0.
int orc_merge_hulls(const orc_part_in* in, int n, double threshold, int maxRounds, double planeTol, int* nOut,
                    int* memberStart, int* members, double* meshVol, double* hullVol, double* hd, int* nSeams,
                    int* stats4) {
  std::vector<OPart> parts;
  for (int k = 0; k < n; k++) parts.push_back(to_part(in[k], k));
  int nextId = n;
  std::map<std::pair<int, int>, Eval> cache;
  const double halfT2 = (threshold / 2) * (threshold / 2);
  int rounds = 0, mergesTot = 0, hulled = 0, hdPairs = 0;
  for (int round = 0; round < maxRounds && parts.size() > 1; round++) {
    rounds = round + 1;
    std::vector<std::pair<size_t, size_t>> todo, cands;
    std::vector<std::array<float, 6>> box(parts.size());
    for (size_t i = 0; i < parts.size(); i++) bbox(parts[i].V, &box[i][0], &box[i][3]);
    for (size_t i = 0; i < parts.size(); i++)
      for (size_t j = i + 1; j < parts.size(); j++) {
        const OPart& A = parts[i];
        const OPart& B = parts[j];
        const auto key = std::make_pair(std::min(A.id, B.id), std::max(A.id, B.id));
        if (cache.count(key)) {
          cands.push_back({i, j});
          continue;
        }
        if (rv(A.meshVol + B.meshVol, A.hullVol + B.hullVol) >= threshold) continue;
        double g2 = 0;
        for (int k = 0; k < 3; k++) {
          const double g = std::max({0.0, (double)box[i][k] - box[j][3 + k], (double)box[j][k] - box[i][3 + k]});
          g2 += g * g;
        }
        if (g2 >= halfT2) continue;
        todo.push_back({i, j});
        cands.push_back({i, j});
      }
    for (const auto& pr : todo) {
      const OPart& A = parts[pr.first];
      const OPart& B = parts[pr.second];
      Eval ev;
      std::vector<float> pts(A.HV);
      pts.insert(pts.end(), B.HV.begin(), B.HV.end());
      const uint32_t np = (uint32_t)(pts.size() / 3);
      std::vector<f3> P(np);
      for (uint32_t i = 0; i < np; i++) P[i] = mk3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
      const uint32_t fmax = 2 * std::min(np, 32768u) + 3 * ORC_VIS_MAX + 1024;
      const uint32_t slab = ((2 * np + std::max(np, 80u) + 7) & ~7u) + 16 * fmax;
      HullOpts ho;
      const HullResult hr = hull_points(P.data(), np, slab, ho);
      hulled++;
      if (hr.status != 0 || hr.hullVol < 0) {
        ev.cost = INFINITY;
      } else {
        ev.hullVol = hr.hullVol;
        ev.cost = rv(A.meshVol + B.meshVol, ev.hullVol);
        ev.hasHull = ev.cost < threshold;
        if (ev.hasHull) {
          ev.hullV = pts;
          ev.hullT = hr.faces;
        }
      }
      if (ev.hasHull) {
        ev.hasSeam = seam(A, B, planeTol, ev.seamP);
        std::vector<Pl> planes;
        if (ev.hasSeam) planes.push_back(ev.seamP);
        planes.insert(planes.end(), A.seams.begin(), A.seams.end());
        planes.insert(planes.end(), B.seams.begin(), B.seams.end());
        std::vector<float> UV;
        std::vector<uint32_t> UT;
        concat(A.V, A.T, B.V, B.T, UV, UT);
        UT = filtered(UV, UT, planes, planeTol);
        if (!UT.empty()) {
          hdPairs++;
          const orc_mesh ua{UV.data(), UT.data(), (uint32_t)(UV.size() / 3), (uint32_t)(UT.size() / 3)};
          const orc_mesh hb{ev.hullV.data(), ev.hullT.data(), (uint32_t)(ev.hullV.size() / 3), (uint32_t)(ev.hullT.size() / 3)};
          ev.hd = hausdorff_gpu_pair(ua, hb, 0);
          ev.cost = std::max(ev.cost, ev.hd);
          if (ev.cost >= threshold) ev.hasHull = false;
        }
      }
      cache[std::make_pair(std::min(A.id, B.id), std::max(A.id, B.id))] = ev;
    }
    struct Ranked {
      size_t i, j;
      const Eval* ev;
    };
    std::vector<Ranked> ranked;
    for (const auto& c : cands) {
      const Eval& ev = cache[std::make_pair(std::min(parts[c.first].id, parts[c.second].id),
                                            std::max(parts[c.first].id, parts[c.second].id))];
      if (ev.cost < threshold && ev.hasHull) ranked.push_back(Ranked{c.first, c.second, &ev});
    }
    std::stable_sort(ranked.begin(), ranked.end(), [](const Ranked& x, const Ranked& y) { return x.ev->cost < y.ev->cost; });
    std::vector<char> used(parts.size(), 0);
    std::vector<OPart> next;
    int merges = 0;
    for (const Ranked& c : ranked) {
      if (used[c.i] || used[c.j]) continue;
      used[c.i] = used[c.j] = 1;
      const OPart& A = parts[c.i];
      const OPart& B = parts[c.j];
      OPart m;
      concat(A.V, A.T, B.V, B.T, m.V, m.T);
      m.HV = c.ev->hullV;
      m.HT = c.ev->hullT;
      m.meshVol = A.meshVol + B.meshVol;
      m.hullVol = c.ev->hullVol;
      m.hd = c.ev->hd;
      m.hasHd = true;
      m.seams = A.seams;
      m.seams.insert(m.seams.end(), B.seams.begin(), B.seams.end());
      if (c.ev->hasSeam) m.seams.push_back(c.ev->seamP);
      m.merged = A.merged + B.merged;
      m.id = nextId++;
      m.members = A.members;
      m.members.insert(m.members.end(), B.members.begin(), B.members.end());
      next.push_back(std::move(m));
      merges++;
    }
    if (merges == 0) break;
    for (size_t i = 0; i < parts.size(); i++)
      if (!used[i]) next.push_back(std::move(parts[i]));
    parts = std::move(next);
    mergesTot += merges;
  }
  *nOut = (int)parts.size();
  int w = 0;
  for (size_t i = 0; i < parts.size(); i++) {
    memberStart[i] = w;
    for (int x : parts[i].members) members[w++] = x;
    meshVol[i] = parts[i].meshVol;
    hullVol[i] = parts[i].hullVol;
    hd[i] = parts[i].hasHd ? parts[i].hd : NAN;
    nSeams[i] = (int)parts[i].seams.size();
  }
  memberStart[parts.size()] = w;
  stats4[0] = rounds;
  stats4[1] = mergesTot;
  stats4[2] = hulled;
  stats4[3] = hdPairs;
  return 0;
}

}  // extern "C"
