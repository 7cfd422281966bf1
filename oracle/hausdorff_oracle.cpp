// hausdorff_oracle.cpp — CPU restatements of the reference's sampled
// Hausdorff distance, in its two forms:
//   * the GPU kernel (src/gpu/hausdorff_shader.ts:13-153): float32 sampling
//     and brute-force nearest triangle;
//   * the CPU helper (src/cpu/hausdorff.ts:10-231): double precision with
//     float32 sample storage and a median-split triangle BVH.
// Both use the same sampling rule: max(1000, floor(2000 * area)) samples,
// area-proportional per triangle with one sample on every step-th (or every
// even) triangle that gets none, barycentrics from a Wang hash of t*65537+k.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA Hausdorff kernels and
// the timed CPU baseline.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "oracle_api.h"
#include "oracle_geom.h"

namespace orc {

static inline uint32_t wang(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s = s * 9u;
  s = s ^ (s >> 4);
  s = s * 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}

// ---------------- GPU form, float32 ----------------
static float tri_area32(f3 a, f3 b, f3 c) {
  f3 n = cross(b - a, c - a);
  return 0.5f * std::sqrt(dot(n, n));
}
static float seg_sq32(f3 p, f3 a, f3 b) {
  f3 ab = b - a, ap = p - a;
  float ab2 = dot(ab, ab);
  float t = ab2 > 1e-20f ? dot(ap, ab) / ab2 : 0.0f;
  t = std::min(std::max(t, 0.0f), 1.0f);
  f3 d = ap - t * ab;
  return dot(d, d);
}
float tri_sq32(f3 p, f3 a, f3 b, f3 c) {
  f3 ab = b - a, ac = c - a, ap = p - a;
  f3 n = cross(ab, ac);
  float n2 = dot(n, n);
  if (n2 < 1e-20f) {
    f3 bp = p - b, cp = p - c;
    return std::min(dot(ap, ap), std::min(dot(bp, bp), dot(cp, cp)));
  }
  float d00 = dot(ab, ab), d01 = dot(ab, ac), d02 = dot(ab, ap);
  float d11 = dot(ac, ac), d12 = dot(ac, ap);
  float inv = 1.0f / (d00 * d11 - d01 * d01);
  float u = (d11 * d02 - d01 * d12) * inv;
  float v = (d00 * d12 - d01 * d02) * inv;
  if (u >= 0.0f && v >= 0.0f && u + v <= 1.0f) {
    float dist = dot(n, ap);
    return (dist * dist) / n2;
  }
  return std::min(seg_sq32(p, a, b), std::min(seg_sq32(p, b, c), seg_sq32(p, c, a)));
}

static f3 V3(const float* V, uint32_t i) { return mk3(V[3 * i], V[3 * i + 1], V[3 * i + 2]); }

// Samples of a mesh by the kernel's rule (hausdorff_shader.ts:57-110). The
// total area is summed in double and rounded once, so the per-triangle
// counts do not depend on a reduction order.
void sample_gpu(const float* V, const uint32_t* T, uint32_t nt, uint32_t cap, std::vector<f3>& out) {
  out.clear();
  std::vector<float> areas(nt);
  double tot = 0.0;
  for (uint32_t t = 0; t < nt; t++) {
    areas[t] = tri_area32(V3(V, T[3 * t]), V3(V, T[3 * t + 1]), V3(V, T[3 * t + 2]));
    tot += (double)areas[t];
  }
  float total = (float)tot;
  float res = std::floor(2000.0f * total);
  if (res < 1000.0f) res = 1000.0f;
  uint32_t step = (float)nt > res ? nt / (uint32_t)res : 0;
  uint32_t run = 0;
  for (uint32_t t = 0; t < nt; t++) {
    uint32_t areaCount = total > 1e-20f ? (uint32_t)std::floor((res / total) * areas[t]) : 0;
    uint32_t N;
    if ((float)nt > res) N = areaCount > 0 ? areaCount : ((t % std::max(step, 1u)) == 0 ? 1 : 0);
    else N = areaCount > 0 ? areaCount : ((t % 2) == 0 ? 1 : 0);
    f3 pa = V3(V, T[3 * t]), pb = V3(V, T[3 * t + 1]), pc = V3(V, T[3 * t + 2]);
    for (uint32_t k = 0; k < N; k++) {
      uint32_t idx = run + k;
      if (idx >= cap) continue;
      uint32_t ha = wang(t * 65537u + k);
      uint32_t hb = wang(ha + 0x9e3779b9u);
      float ra = (float)(ha & 0xFFFFFFu) / (float)0xFFFFFFu;
      float rb = (float)(hb & 0xFFFFFFu) / (float)0xFFFFFFu;
      float sqa = std::sqrt(ra);
      f3 s = ((1.0f - sqa) * pa + (sqa * (1.0f - rb)) * pb) + (sqa * rb) * pc;
      out.push_back(s);
    }
    run += N;
  }
}

static float directed_sq32(const std::vector<f3>& S, const float* V, const uint32_t* T, uint32_t nt) {
  float worst = 0.0f;
  for (const f3& p : S) {
    float best = 1e30f;
    for (uint32_t t = 0; t < nt; t++) best = std::min(best, tri_sq32(p, V3(V, T[3 * t]), V3(V, T[3 * t + 1]), V3(V, T[3 * t + 2])));
    worst = std::max(worst, best);
  }
  return worst;
}

// One pair as the kernel computes it; cap is the pair's sample capacity
// (half per side), 0 = unbounded.
float hausdorff_gpu_pair(const orc_mesh& a, const orc_mesh& b, uint32_t cap) {
  if (a.nt == 0 || b.nt == 0) return 0.0f;
  uint32_t capA = cap ? cap / 2 : 0xffffffffu, capB = cap ? cap - cap / 2 : 0xffffffffu;
  std::vector<f3> sa, sb;
  sample_gpu(a.verts, a.tris, a.nt, capA, sa);
  sample_gpu(b.verts, b.tris, b.nt, capB, sb);
  float w = std::max(directed_sq32(sa, b.verts, b.tris, b.nt), directed_sq32(sb, a.verts, a.tris, a.nt));
  return std::sqrt(w);
}

// ---------------- CPU helper form, double ----------------
static double tri_area64(const float* V, uint32_t a, uint32_t b, uint32_t c) {
  double abx = (double)V[b] - V[a], aby = (double)V[b + 1] - V[a + 1], abz = (double)V[b + 2] - V[a + 2];
  double acx = (double)V[c] - V[a], acy = (double)V[c + 1] - V[a + 1], acz = (double)V[c + 2] - V[a + 2];
  double nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
  return 0.5 * std::sqrt(nx * nx + ny * ny + nz * nz);
}

// hausdorff.ts:28-65
void sample_cpu(const float* V, const uint32_t* T, uint32_t nt, std::vector<float>& out) {
  std::vector<float> areas(nt);
  double area = 0.0;
  for (uint32_t t = 0; t < nt; t++) {
    areas[t] = (float)tri_area64(V, T[3 * t] * 3, T[3 * t + 1] * 3, T[3 * t + 2] * 3);
    area += (double)areas[t];
  }
  double res = std::floor(2000.0 * area);
  if (res < 1000.0) res = 1000.0;
  std::vector<int64_t> counts(nt);
  int64_t total = 0;
  double step = (double)nt > res ? std::floor((double)nt / res) : 0.0;
  for (uint32_t t = 0; t < nt; t++) {
    double areaCount = area > 1e-20 ? std::floor(res / area * (double)areas[t]) : 0.0;
    int64_t N;
    if ((double)nt > res) N = areaCount > 0 ? (int64_t)areaCount : (std::fmod((double)t, step) == 0.0 ? 1 : 0);
    else N = areaCount > 0 ? (int64_t)areaCount : (t % 2 == 0 ? 1 : 0);
    counts[t] = N;
    total += N;
  }
  out.assign(3 * (size_t)total, 0.0f);
  size_t idx = 0;
  for (uint32_t t = 0; t < nt; t++) {
    uint32_t a = T[3 * t] * 3, b = T[3 * t + 1] * 3, c = T[3 * t + 2] * 3;
    for (int64_t k = 0; k < counts[t]; k++) {
      uint32_t ha = wang(t * 65537u + (uint32_t)k);
      uint32_t hb = wang(ha + 0x9e3779b9u);
      double ra = (double)(ha & 0xffffffu) / (double)0xffffff;
      double rb = (double)(hb & 0xffffffu) / (double)0xffffff;
      double sqa = std::sqrt(ra);
      double w0 = 1 - sqa, w1 = sqa * (1 - rb), w2 = sqa * rb;
      for (int ax = 0; ax < 3; ax++) out[3 * idx + ax] = (float)(w0 * V[a + ax] + w1 * V[b + ax] + w2 * V[c + ax]);
      idx++;
    }
  }
}

static double seg_sq64(double px, double py, double pz, double ax, double ay, double az, double bx, double by, double bz) {
  double abx = bx - ax, aby = by - ay, abz = bz - az;
  double apx = px - ax, apy = py - ay, apz = pz - az;
  double ab2 = abx * abx + aby * aby + abz * abz;
  double t = ab2 > 1e-20 ? (apx * abx + apy * aby + apz * abz) / ab2 : 0;
  t = std::max(0.0, std::min(1.0, t));
  double dx = apx - t * abx, dy = apy - t * aby, dz = apz - t * abz;
  return dx * dx + dy * dy + dz * dz;
}
// hausdorff.ts:78-113
double tri_sq64(double px, double py, double pz, double ax, double ay, double az, double bx, double by, double bz,
                double cx, double cy, double cz) {
  double abx = bx - ax, aby = by - ay, abz = bz - az;
  double acx = cx - ax, acy = cy - ay, acz = cz - az;
  double apx = px - ax, apy = py - ay, apz = pz - az;
  double nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
  double n2 = nx * nx + ny * ny + nz * nz;
  if (n2 < 1e-20) {
    double da = apx * apx + apy * apy + apz * apz;
    double bpx = px - bx, bpy = py - by, bpz = pz - bz;
    double db = bpx * bpx + bpy * bpy + bpz * bpz;
    double cpx = px - cx, cpy = py - cy, cpz = pz - cz;
    double dc = cpx * cpx + cpy * cpy + cpz * cpz;
    return std::min(da, std::min(db, dc));
  }
  double d00 = abx * abx + aby * aby + abz * abz;
  double d01 = abx * acx + aby * acy + abz * acz;
  double d02 = abx * apx + aby * apy + abz * apz;
  double d11 = acx * acx + acy * acy + acz * acz;
  double d12 = acx * apx + acy * apy + acz * apz;
  double inv = 1 / (d00 * d11 - d01 * d01);
  double u = (d11 * d02 - d01 * d12) * inv;
  double v = (d00 * d12 - d01 * d02) * inv;
  if (u >= 0 && v >= 0 && u + v <= 1) {
    double dist = nx * apx + ny * apy + nz * apz;
    return (dist * dist) / n2;
  }
  return std::min(seg_sq64(px, py, pz, ax, ay, az, bx, by, bz),
                  std::min(seg_sq64(px, py, pz, bx, by, bz, cx, cy, cz), seg_sq64(px, py, pz, cx, cy, cz, ax, ay, az)));
}

// median-split BVH over triangles (hausdorff.ts:116-217)
struct BVH {
  const float* V;
  const uint32_t* T;
  std::vector<float> bmin, bmax;
  std::vector<int32_t> left, right, start, count;
  std::vector<uint32_t> order;
  std::vector<float> cent;
  int nNodes = 0;
  BVH(const float* V_, const uint32_t* T_, uint32_t nt, int leafSize = 4) : V(V_), T(T_) {
    int cap = std::max(1, 2 * (int)std::ceil((double)nt / std::max(1, leafSize / 2)) + 2);
    bmin.assign(3 * cap, 0); bmax.assign(3 * cap, 0);
    left.assign(cap, -1); right.assign(cap, -1); start.assign(cap, 0); count.assign(cap, 0);
    order.resize(nt);
    std::iota(order.begin(), order.end(), 0u);
    cent.assign(3 * (size_t)nt, 0);
    for (uint32_t t = 0; t < nt; t++)
      for (int a = 0; a < 3; a++)
        cent[3 * t + a] = (float)(((double)V[T[3 * t] * 3 + a] + V[T[3 * t + 1] * 3 + a] + V[T[3 * t + 2] * 3 + a]) / 3);
    if (nt > 0) build(0, nt, leafSize);
  }
  int build(int s, int e, int leafSize) {
    int node = nNodes++;
    float x0 = INFINITY, y0 = INFINITY, z0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY, z1 = -INFINITY;
    float cx0 = INFINITY, cy0 = INFINITY, cz0 = INFINITY, cx1 = -INFINITY, cy1 = -INFINITY, cz1 = -INFINITY;
    for (int i = s; i < e; i++) {
      uint32_t t = order[i];
      for (int k = 0; k < 3; k++) {
        uint32_t v = T[3 * t + k] * 3;
        float x = V[v], y = V[v + 1], z = V[v + 2];
        x0 = std::min(x0, x); x1 = std::max(x1, x); y0 = std::min(y0, y); y1 = std::max(y1, y); z0 = std::min(z0, z); z1 = std::max(z1, z);
      }
      float cx = cent[3 * t], cy = cent[3 * t + 1], cz = cent[3 * t + 2];
      cx0 = std::min(cx0, cx); cx1 = std::max(cx1, cx); cy0 = std::min(cy0, cy); cy1 = std::max(cy1, cy); cz0 = std::min(cz0, cz); cz1 = std::max(cz1, cz);
    }
    bmin[3 * node] = x0; bmin[3 * node + 1] = y0; bmin[3 * node + 2] = z0;
    bmax[3 * node] = x1; bmax[3 * node + 1] = y1; bmax[3 * node + 2] = z1;
    if (e - s <= leafSize) { start[node] = s; count[node] = e - s; return node; }
    float ex = cx1 - cx0, ey = cy1 - cy0, ez = cz1 - cz0;
    int axis = (ex >= ey && ex >= ez) ? 0 : (ey >= ez ? 1 : 2);
    std::stable_sort(order.begin() + s, order.begin() + e, [&](uint32_t p, uint32_t q) { return cent[3 * p + axis] < cent[3 * q + axis]; });
    int mid = (s + e) >> 1;
    count[node] = 0;
    left[node] = build(s, mid, leafSize);
    right[node] = build(mid, e, leafSize);
    return node;
  }
  double boxDistSq(int node, double px, double py, double pz) const {
    double dx = std::max(std::max((double)bmin[3 * node] - px, 0.0), px - (double)bmax[3 * node]);
    double dy = std::max(std::max((double)bmin[3 * node + 1] - py, 0.0), py - (double)bmax[3 * node + 1]);
    double dz = std::max(std::max((double)bmin[3 * node + 2] - pz, 0.0), pz - (double)bmax[3 * node + 2]);
    return dx * dx + dy * dy + dz * dz;
  }
  double nearestSq(double px, double py, double pz) const {
    if (nNodes == 0) return INFINITY;
    double best = INFINITY;
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
      int node = stack[--sp];
      if (boxDistSq(node, px, py, pz) >= best) continue;
      if (count[node] > 0) {
        for (int i = start[node]; i < start[node] + count[node]; i++) {
          uint32_t t = order[i];
          uint32_t a = T[3 * t] * 3, b = T[3 * t + 1] * 3, c = T[3 * t + 2] * 3;
          double d = tri_sq64(px, py, pz, V[a], V[a + 1], V[a + 2], V[b], V[b + 1], V[b + 2], V[c], V[c + 1], V[c + 2]);
          if (d < best) best = d;
        }
      } else {
        int l = left[node], r = right[node];
        double dl = boxDistSq(l, px, py, pz), dr = boxDistSq(r, px, py, pz);
        if (dl < dr) { stack[sp++] = r; stack[sp++] = l; } else { stack[sp++] = l; stack[sp++] = r; }
      }
    }
    return best;
  }
};

static double directed_cpu(const std::vector<float>& S, const BVH& b) {
  double worst = 0;
  for (size_t i = 0; i < S.size(); i += 3) {
    double d = b.nearestSq(S[i], S[i + 1], S[i + 2]);
    if (d > worst) worst = d;
  }
  return std::sqrt(worst);
}

// hausdorff.ts:225-231
double hausdorff_cpu(const orc_mesh& a, const orc_mesh& b) {
  if (a.nt == 0 || b.nt == 0) return 0.0;
  std::vector<float> sa, sb;
  sample_cpu(a.verts, a.tris, a.nt, sa);
  sample_cpu(b.verts, b.tris, b.nt, sb);
  BVH ba(a.verts, a.tris, a.nt), bb(b.verts, b.tris, b.nt);
  return std::max(directed_cpu(sa, bb), directed_cpu(sb, ba));
}

}  // namespace orc

extern "C" {

// Hausdorff of n pairs as the GPU kernel computes it; caps may be null
// (unbounded sample capacity) or hold each pair's capacity.
void orc_hausdorff_gpu(const orc_mesh* a, const orc_mesh* b, int n, const uint32_t* caps, float* out) {
  for (int k = 0; k < n; k++) out[k] = orc::hausdorff_gpu_pair(a[k], b[k], caps ? caps[k] : 0);
}
// Hausdorff of n pairs as the CPU helper computes it (double, BVH)
void orc_hausdorff_cpu(const orc_mesh* a, const orc_mesh* b, int n, double* out) {
  for (int k = 0; k < n; k++) out[k] = orc::hausdorff_cpu(a[k], b[k]);
}
// Sample points of one mesh by the GPU rule (3 floats per sample); returns the count
int orc_sample_gpu(const orc_mesh* m, uint32_t cap, float* out, uint32_t outCap) {
  std::vector<orc::f3> s;
  orc::sample_gpu(m->verts, m->tris, m->nt, cap ? cap : 0xffffffffu, s);
  uint32_t n = (uint32_t)s.size();
  for (uint32_t i = 0; i < n && i < outCap; i++) { out[3 * i] = s[i].x; out[3 * i + 1] = s[i].y; out[3 * i + 2] = s[i].z; }
  return (int)n;
}

}
