// host_mesh.cpp — mesh utilities, concave-edge planes, hull compaction and
// the CPU Hausdorff distance of the decomposition loop (see host_mesh.h).
#include "host_mesh.h"

#include <algorithm>
#include <cmath>
#include <limits>

namespace cuacd {
namespace host {

double signed_volume(const Mesh& m) {
  if (m.t.empty()) return 0.0;
  const float* v = m.v.data();
  const double ox = v[0], oy = v[1], oz = v[2];
  double s = 0.0;
  for (size_t i = 0; i < m.t.size(); i += 3) {
    const size_t a = 3 * (size_t)m.t[i], b = 3 * (size_t)m.t[i + 1], c = 3 * (size_t)m.t[i + 2];
    const double ax = v[a] - ox, ay = v[a + 1] - oy, az = v[a + 2] - oz;
    const double bx = v[b] - ox, by = v[b + 1] - oy, bz = v[b + 2] - oz;
    const double cx = v[c] - ox, cy = v[c + 1] - oy, cz = v[c + 2] - oz;
    s += ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
  }
  return s / 6.0;
}

EdgeCSR edge_csr(const Mesh& m) {
  const size_t n = m.nv();
  EdgeCSR e;
  e.off.assign(n + 1, 0);
  for (uint32_t x : m.t) e.off[(size_t)x + 1]++;
  for (size_t v = 0; v < n; v++) e.off[v + 1] += e.off[v];
  std::vector<uint32_t> fill(e.off.begin(), e.off.end() - 1);
  e.dst.resize(m.t.size());
  e.face.resize(m.t.size());
  for (size_t i = 0; i < m.t.size(); i += 3) {
    for (int k = 0; k < 3; k++) {
      const uint32_t a = m.t[i + k], b = m.t[i + (k + 1) % 3];
      const uint32_t slot = fill[a]++;
      e.dst[slot] = b;
      e.face[slot] = (uint32_t)(i / 3);
    }
  }
  return e;
}

bool is_closed(const Mesh& m) {
  const size_t n = m.nv();
  for (uint32_t x : m.t)
    if (x >= n) return false;
  const EdgeCSR e = edge_csr(m);
  auto count = [&](uint32_t a, uint32_t b) {
    uint32_t c = 0;
    for (uint32_t k = e.off[a]; k < e.off[a + 1]; k++) c += e.dst[k] == b;
    return c;
  };
  for (uint32_t a = 0; a < n; a++)
    for (uint32_t k = e.off[a]; k < e.off[a + 1]; k++) {
      const uint32_t b = e.dst[k];
      if (count(a, b) != 1 || count(b, a) != 1) return false;
    }
  return true;
}

void bbox(const Mesh& m, float lo[3], float hi[3]) {
  for (int a = 0; a < 3; a++) {
    lo[a] = std::numeric_limits<float>::infinity();
    hi[a] = -std::numeric_limits<float>::infinity();
  }
  for (size_t i = 0; i < m.v.size(); i += 3)
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], m.v[i + a]);
      hi[a] = std::max(hi[a], m.v[i + a]);
    }
}

Mesh normalize(const Mesh& m, Normalization& norm) {
  float lo[3], hi[3];
  bbox(m, lo, hi);
  double ext = 0.0;
  for (int a = 0; a < 3; a++) {
    norm.center[a] = ((double)lo[a] + (double)hi[a]) / 2.0;
    ext = std::max(ext, (double)hi[a] - (double)lo[a]);
  }
  norm.scale = ext > 0 ? ext / 2.0 : 1.0;
  Mesh out;
  out.t = m.t;
  out.v.resize(m.v.size());
  for (size_t i = 0; i < m.v.size(); i++) out.v[i] = (float)(((double)m.v[i] - norm.center[i % 3]) / norm.scale);
  return out;
}

Mesh denormalize(const Mesh& m, const Normalization& norm) {
  Mesh out;
  out.t = m.t;
  out.v.resize(m.v.size());
  for (size_t i = 0; i < m.v.size(); i++) out.v[i] = (float)((double)m.v[i] * norm.scale + norm.center[i % 3]);
  return out;
}

Plane denormalize_plane(const Plane& p, const Normalization& n) {
  return Plane{p.a, p.b, p.c, p.d * n.scale - (p.a * n.center[0] + p.b * n.center[1] + p.c * n.center[2])};
}

Mesh merge_meshes(const Mesh& a, const Mesh& b) {
  Mesh m;
  m.v.reserve(a.v.size() + b.v.size());
  m.v.insert(m.v.end(), a.v.begin(), a.v.end());
  m.v.insert(m.v.end(), b.v.begin(), b.v.end());
  m.t.reserve(a.t.size() + b.t.size());
  m.t.insert(m.t.end(), a.t.begin(), a.t.end());
  const uint32_t off = (uint32_t)a.nv();
  for (uint32_t x : b.t) m.t.push_back(x + off);
  return m;
}

// ---------------------------------------------------------------------------
// concave-edge planes

namespace {
bool face_normal(const Mesh& m, uint32_t f, double n[3]) {
  const float* V = m.v.data();
  const size_t a = 3 * (size_t)m.t[3 * f], b = 3 * (size_t)m.t[3 * f + 1], c = 3 * (size_t)m.t[3 * f + 2];
  const double e1x = (double)V[b] - V[a], e1y = (double)V[b + 1] - V[a + 1], e1z = (double)V[b + 2] - V[a + 2];
  const double e2x = (double)V[c] - V[a], e2y = (double)V[c + 1] - V[a + 1], e2z = (double)V[c + 2] - V[a + 2];
  const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  const double l = std::sqrt(nx * nx + ny * ny + nz * nz);
  if (l < 1e-12) return false;
  n[0] = nx / l;
  n[1] = ny / l;
  n[2] = nz / l;
  return true;
}
}  // namespace

std::vector<float> concave_edge_planes(const Mesh& m, int nConcaveEdges, double concaveEps, double concaveThreshold,
                                       uint32_t seed) {
  std::vector<float> out;
  if (nConcaveEdges <= 0 || m.nt() == 0) return out;
  const EdgeCSR e = edge_csr(m);
  const uint32_t nvv = (uint32_t)(e.off.size() - 1);
  auto find_face = [&](uint32_t a, uint32_t b) -> int64_t {
    for (uint32_t k = e.off[a]; k < e.off[a + 1]; k++)
      if (e.dst[k] == b) return e.face[k];
    return -1;
  };
  uint32_t rng = seed;
  auto lcg = [&]() {
    rng = rng * 1664525u + 1013904223u;
    return rng;
  };
  struct Edge {
    uint32_t v0, v1, f0, f1;
  };
  std::vector<Edge> reservoir;
  double seen = 0;
  std::vector<uint32_t> partners;
  const float* V = m.v.data();
  for (uint32_t v0 = 0; v0 < nvv; v0++) {
    partners.clear();
    for (uint32_t k = e.off[v0]; k < e.off[v0 + 1]; k++) {
      const uint32_t b = e.dst[k];
      if (b > v0 && std::find(partners.begin(), partners.end(), b) == partners.end()) partners.push_back(b);
    }
    std::sort(partners.begin(), partners.end());
    for (uint32_t v1 : partners) {
      const int64_t fa = find_face(v0, v1), fb = find_face(v1, v0);
      if (fa < 0 || fb < 0) continue;
      const uint32_t f0 = (uint32_t)std::min(fa, fb), f1 = (uint32_t)std::max(fa, fb);
      double n0[3], n1[3];
      if (!face_normal(m, f0, n0) || !face_normal(m, f1, n1)) continue;
      double cosA = n0[0] * n1[0] + n0[1] * n1[1] + n0[2] * n1[2];
      cosA = std::max(-1.0, std::min(1.0, cosA));
      const double alpha = std::acos(cosA);
      int64_t vOther = -1;
      for (int i = 0; i < 3; i++) {
        const uint32_t vv = m.t[3 * (size_t)f0 + i];
        if (vv != v0 && vv != v1) {
          vOther = vv;
          break;
        }
      }
      if (vOther < 0) continue;
      const double dx = (double)V[3 * vOther] - V[3 * (size_t)v0];
      const double dy = (double)V[3 * vOther + 1] - V[3 * (size_t)v0 + 1];
      const double dz = (double)V[3 * vOther + 2] - V[3 * (size_t)v0 + 2];
      const double d = dx * n1[0] + dy * n1[1] + dz * n1[2];
      const double dihedral = d > 0 ? M_PI + alpha : M_PI - alpha;
      if (!(dihedral > concaveThreshold)) continue;
      seen += 1;
      if ((int)reservoir.size() < nConcaveEdges) {
        reservoir.push_back(Edge{v0, v1, f0, f1});
      } else {
        const uint32_t r = lcg();
        const double thresh = std::floor((double)nConcaveEdges / seen * 4294967295.0);
        if ((double)r < thresh) {
          const uint32_t slot = lcg() % (uint32_t)nConcaveEdges;
          reservoir[slot] = Edge{v0, v1, f0, f1};
        }
      }
    }
  }
  for (const Edge& r : reservoir) {
    double n0[3], n1[3];
    if (!face_normal(m, r.f0, n0) || !face_normal(m, r.f1, n1)) continue;
    const double mx = ((double)V[3 * (size_t)r.v0] + V[3 * (size_t)r.v1]) / 2;
    const double my = ((double)V[3 * (size_t)r.v0 + 1] + V[3 * (size_t)r.v1 + 1]) / 2;
    const double mz = ((double)V[3 * (size_t)r.v0 + 2] + V[3 * (size_t)r.v1 + 2]) / 2;
    const double eps = concaveEps;
    auto push = [&](double a, double b, double c, double d) {
      out.push_back((float)a);
      out.push_back((float)b);
      out.push_back((float)c);
      out.push_back((float)d);
    };
    push(n1[0], n1[1], n1[2], -(n1[0] * mx + n1[1] * my + n1[2] * mz + eps));
    push(n0[0], n0[1], n0[2], -(n0[0] * mx + n0[1] * my + n0[2] * mz + eps));
    double bx = n0[0] + n1[0], by = n0[1] + n1[1], bz = n0[2] + n1[2];
    const double bl = std::sqrt(bx * bx + by * by + bz * bz);
    if (bl >= 1e-4) {
      bx /= bl;
      by /= bl;
      bz /= bl;
      push(bx, by, bz, -(bx * mx + by * my + bz * mz + eps));
      push(bx, by, bz, -(bx * mx + by * my + bz * mz - eps));
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// hull compaction

Mesh compact_hull(const float* pts, const uint32_t* tris, size_t ntris, double* volumeOut) {
  Mesh m;
  std::vector<int64_t> remap;
  uint32_t maxIdx = 0;
  for (size_t i = 0; i < 3 * ntris; i++) maxIdx = std::max(maxIdx, tris[i]);
  remap.assign(ntris ? (size_t)maxIdx + 1 : 0, -1);
  m.t.resize(3 * ntris);
  for (size_t i = 0; i < 3 * ntris; i++) {
    const uint32_t v = tris[i];
    if (remap[v] < 0) {
      remap[v] = (int64_t)m.nv();
      m.v.push_back(pts[3 * (size_t)v]);
      m.v.push_back(pts[3 * (size_t)v + 1]);
      m.v.push_back(pts[3 * (size_t)v + 2]);
    }
    m.t[i] = (uint32_t)remap[v];
  }
  const double sv = signed_volume(m);
  if (sv < 0)
    for (size_t i = 0; i < m.t.size(); i += 3) std::swap(m.t[i + 1], m.t[i + 2]);
  if (volumeOut) *volumeOut = sv < 0 ? -sv : sv;
  return m;
}

// ---------------------------------------------------------------------------
// CPU Hausdorff distance

namespace {
uint32_t wang_hash(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s *= 9u;
  s = s ^ (s >> 4);
  s *= 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}

std::vector<float> sample_mesh(const Mesh& m) {
  const float* V = m.v.data();
  const size_t nt = m.nt();
  std::vector<float> areas(nt);
  double area = 0;
  for (size_t t = 0; t < nt; t++) {
    const size_t a = 3 * (size_t)m.t[3 * t], b = 3 * (size_t)m.t[3 * t + 1], c = 3 * (size_t)m.t[3 * t + 2];
    const double abx = (double)V[b] - V[a], aby = (double)V[b + 1] - V[a + 1], abz = (double)V[b + 2] - V[a + 2];
    const double acx = (double)V[c] - V[a], acy = (double)V[c + 1] - V[a + 1], acz = (double)V[c + 2] - V[a + 2];
    const double nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
    areas[t] = (float)(0.5 * std::sqrt(nx * nx + ny * ny + nz * nz));
    area += areas[t];
  }
  double res = std::floor(2000.0 * area);
  if (res < 1000.0) res = 1000.0;
  const double step = (double)nt > res ? std::floor((double)nt / res) : 0.0;
  std::vector<int64_t> counts(nt);
  size_t total = 0;
  for (size_t t = 0; t < nt; t++) {
    const double ac = area > 1e-20 ? std::floor(res / area * areas[t]) : 0.0;
    int64_t n;
    if ((double)nt > res)
      n = ac > 0 ? (int64_t)ac : (std::fmod((double)t, step) == 0.0 ? 1 : 0);
    else
      n = ac > 0 ? (int64_t)ac : (t % 2 == 0 ? 1 : 0);
    counts[t] = n;
    total += (size_t)n;
  }
  std::vector<float> out(3 * total);
  size_t idx = 0;
  for (size_t t = 0; t < nt; t++) {
    const size_t a = 3 * (size_t)m.t[3 * t], b = 3 * (size_t)m.t[3 * t + 1], c = 3 * (size_t)m.t[3 * t + 2];
    for (int64_t k = 0; k < counts[t]; k++) {
      const uint32_t ha = wang_hash((uint32_t)t * 65537u + (uint32_t)k);
      const uint32_t hb = wang_hash(ha + 0x9e3779b9u);
      const double ra = (double)(ha & 0xffffffu) / 16777215.0;
      const double rb = (double)(hb & 0xffffffu) / 16777215.0;
      const double sqa = std::sqrt(ra);
      const double w0 = 1 - sqa, w1 = sqa * (1 - rb), w2 = sqa * rb;
      for (int q = 0; q < 3; q++) out[3 * idx + q] = (float)(w0 * V[a + q] + w1 * V[b + q] + w2 * V[c + q]);
      idx++;
    }
  }
  return out;
}

double seg_sq(double px, double py, double pz, double ax, double ay, double az, double bx, double by, double bz) {
  const double abx = bx - ax, aby = by - ay, abz = bz - az;
  const double apx = px - ax, apy = py - ay, apz = pz - az;
  const double ab2 = abx * abx + aby * aby + abz * abz;
  double t = ab2 > 1e-20 ? (apx * abx + apy * aby + apz * abz) / ab2 : 0;
  t = std::max(0.0, std::min(1.0, t));
  const double dx = apx - t * abx, dy = apy - t * aby, dz = apz - t * abz;
  return dx * dx + dy * dy + dz * dz;
}

double tri_sq(double px, double py, double pz, const float* A, const float* B, const float* C) {
  const double ax = A[0], ay = A[1], az = A[2], bx = B[0], by = B[1], bz = B[2], cx = C[0], cy = C[1], cz = C[2];
  const double abx = bx - ax, aby = by - ay, abz = bz - az;
  const double acx = cx - ax, acy = cy - ay, acz = cz - az;
  const double apx = px - ax, apy = py - ay, apz = pz - az;
  const double nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
  const double n2 = nx * nx + ny * ny + nz * nz;
  if (n2 < 1e-20) {
    const double da = apx * apx + apy * apy + apz * apz;
    const double db = (px - bx) * (px - bx) + (py - by) * (py - by) + (pz - bz) * (pz - bz);
    const double dc = (px - cx) * (px - cx) + (py - cy) * (py - cy) + (pz - cz) * (pz - cz);
    return std::min(da, std::min(db, dc));
  }
  const double d00 = abx * abx + aby * aby + abz * abz;
  const double d01 = abx * acx + aby * acy + abz * acz;
  const double d02 = abx * apx + aby * apy + abz * apz;
  const double d11 = acx * acx + acy * acy + acz * acz;
  const double d12 = acx * apx + acy * apy + acz * apz;
  const double inv = 1 / (d00 * d11 - d01 * d01);
  const double u = (d11 * d02 - d01 * d12) * inv;
  const double v = (d00 * d12 - d01 * d02) * inv;
  if (u >= 0 && v >= 0 && u + v <= 1) {
    const double dist = nx * apx + ny * apy + nz * apz;
    return (dist * dist) / n2;
  }
  return std::min(seg_sq(px, py, pz, ax, ay, az, bx, by, bz),
                  std::min(seg_sq(px, py, pz, bx, by, bz, cx, cy, cz), seg_sq(px, py, pz, cx, cy, cz, ax, ay, az)));
}

double directed(const std::vector<float>& s, const Mesh& b) {
  double worst = 0;
  const float* V = b.v.data();
  for (size_t i = 0; i < s.size(); i += 3) {
    double best = std::numeric_limits<double>::infinity();
    for (size_t t = 0; t < b.nt(); t++)
      best = std::min(best, tri_sq(s[i], s[i + 1], s[i + 2], V + 3 * (size_t)b.t[3 * t], V + 3 * (size_t)b.t[3 * t + 1],
                                   V + 3 * (size_t)b.t[3 * t + 2]));
    worst = std::max(worst, best);
  }
  return std::sqrt(worst);
}
}  // namespace

double hausdorff_cpu(const Mesh& a, const Mesh& b) {
  if (a.t.empty() || b.t.empty()) return 0.0;
  return std::max(directed(sample_mesh(a), b), directed(sample_mesh(b), a));
}

}  // namespace host
}  // namespace cuacd
