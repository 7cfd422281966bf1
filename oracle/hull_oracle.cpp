// hull_oracle.cpp — CPU restatement of the GPU hull kernel of the reference
// (src/gpu/shaders.ts:752-1401): grid quantisation, 40-axis k-DOP seeds,
// exact orientation predicates, initial simplex, farthest-first incremental
// insertion, last-level branch-and-bound pruning, volume and face export.
//
// TEST INFRASTRUCTURE ONLY: this is the checker for the CUDA hull kernel.
//
// The reference collects visible faces and new faces with atomicAdd, so its
// face-slot order depends on timing. This restatement fixes one order, which
// the CUDA kernel follows too:
//   * visible faces are listed in face-slot order;
//   * the most visible face is the largest ranking value, lowest list
//     position on ties (shaders.ts:988-1006);
//   * new faces are created in horizon-edge order e = 3*listPos + k
//     (shaders.ts:1033-1049);
//   * the next point to insert is the largest owner distance, lowest point
//     index on ties (shaders.ts:1068-1078).
// The hull volume is summed exactly: every face contributes an integer
// determinant of grid coordinates (< 2^22) and the sum is kept in 128 bits,
// where the reference sums float32 terms (shaders.ts:1132-1142).
#include <algorithm>
#include <cstdint>
#include <vector>

#include "oracle.h"
#include "oracle_geom.h"

namespace orc {

static const uint32_t NONE = 0xffffffffu;
static const uint32_t ALIVE = 0x80000000u;
static const uint32_t FW = 16;

// k-DOP seed axes (shaders.ts:769-810). The seed points must be the same
// extremes as the reference kernel picks, so the table is the same.
static const float KDOP[40][3] = {
    {-0.5786893f, 0.7696723f, 0.2696723f}, {-0.7696723f, 0.2696723f, 0.5786893f},
    {-0.2696723f, 0.5786893f, 0.7696723f}, {-0.5773503f, 0.5773503f, 0.5773503f},
    {-0.3090170f, 0.9363390f, 0.1666667f}, {0.0000000f, 0.7453560f, 0.6666667f},
    {0.3090170f, 0.9363390f, 0.1666667f},  {0.0000000f, 0.9341724f, 0.3568221f},
    {-0.3090170f, 0.9363390f, -0.1666667f}, {0.3090170f, 0.9363390f, -0.1666667f},
    {0.0000000f, 0.7453560f, -0.6666667f}, {0.0000000f, 0.9341724f, -0.3568221f},
    {-0.5786893f, 0.7696723f, -0.2696723f}, {-0.2696723f, 0.5786893f, -0.7696723f},
    {-0.7696723f, 0.2696723f, -0.5786893f}, {-0.5773503f, 0.5773503f, -0.5773503f},
    {-0.7453560f, 0.6666667f, 0.0000000f}, {-0.9363390f, 0.1666667f, -0.3090170f},
    {-0.9363390f, 0.1666667f, 0.3090170f}, {-0.9341724f, 0.3568221f, 0.0000000f},
    {0.5786893f, 0.7696723f, 0.2696723f},  {0.2696723f, 0.5786893f, 0.7696723f},
    {0.7696723f, 0.2696723f, 0.5786893f},  {0.5773503f, 0.5773503f, 0.5773503f},
    {-0.1666667f, 0.3090170f, 0.9363390f}, {-0.6666667f, 0.0000000f, 0.7453560f},
    {-0.1666667f, -0.3090170f, 0.9363390f}, {-0.3568221f, 0.0000000f, 0.9341724f},
    {-0.9363390f, -0.1666667f, 0.3090170f}, {-0.9363390f, -0.1666667f, -0.3090170f},
    {-0.7453560f, -0.6666667f, 0.0000000f}, {-0.9341724f, -0.3568221f, 0.0000000f},
    {-0.6666667f, 0.0000000f, -0.7453560f}, {-0.1666667f, 0.3090170f, -0.9363390f},
    {-0.1666667f, -0.3090170f, -0.9363390f}, {-0.3568221f, 0.0000000f, -0.9341724f},
    {0.2696723f, 0.5786893f, -0.7696723f}, {0.5786893f, 0.7696723f, -0.2696723f},
    {0.7696723f, 0.2696723f, -0.5786893f}, {0.5773503f, 0.5773503f, -0.5773503f},
};

typedef __int128 i128;

// sign of det[e1; e2; d] for integer vectors (shaders.ts:868-876), exactly
static int orient_exact(f3 e1f, f3 e2f, f3 df) {
  int64_t e1x = (int64_t)e1f.x, e1y = (int64_t)e1f.y, e1z = (int64_t)e1f.z;
  int64_t e2x = (int64_t)e2f.x, e2y = (int64_t)e2f.y, e2z = (int64_t)e2f.z;
  int64_t dx = (int64_t)df.x, dy = (int64_t)df.y, dz = (int64_t)df.z;
  int64_t cx = e1y * e2z - e1z * e2y;
  int64_t cy = e1z * e2x - e1x * e2z;
  int64_t cz = e1x * e2y - e1y * e2x;
  i128 det = (i128)cx * dx + (i128)cy * dy + (i128)cz * dz;
  return det > 0 ? 1 : (det < 0 ? -1 : 0);
}

static float l1(f3 a) { return (std::fabs(a.x) + std::fabs(a.y)) + std::fabs(a.z); }

// filtered orientation (shaders.ts:878-884)
static int orient_filtered(f3 n, f3 e1, f3 e2, f3 d) {
  float det = dot(n, d);
  float bound = ((1e-6f * l1(e1)) * l1(e2)) * l1(d);
  if (det > bound) return 1;
  if (det < -bound) return -1;
  return orient_exact(e1, e2, d);
}

struct Hull {
  const f3* pts;
  uint32_t nv;
  f3 qlo;
  float qs;
  uint32_t fmax;
  std::vector<uint32_t> faces;  // FW words per slot
  std::vector<uint32_t> owner, cand;
  std::vector<float> dist;
  uint32_t nf = 0, nalive = 0, fail = 0;
  bool compacted = false;

  f3 qvert(uint32_t i) const {
    f3 v = pts[i] - qlo;
    return mk3(std::nearbyint(v.x * qs), std::nearbyint(v.y * qs), std::nearbyint(v.z * qs));
  }
  uint32_t* F(uint32_t f) { return &faces[(size_t)FW * f]; }
  bool alive(uint32_t f) { return (F(f)[0] & ALIVE) != 0; }
  void face_abc(uint32_t f, uint32_t& a, uint32_t& b, uint32_t& c) {
    uint32_t* w = F(f);
    a = w[0] & 0x7fffffffu; b = w[1]; c = w[2];
  }
  // face record: ia|alive ib ic bf | nx ny nz ax | ay az bx by | bz cx cy cz
  void face_write(uint32_t f, uint32_t a, uint32_t b, uint32_t c) {
    f3 pa = qvert(a), pb = qvert(b), pc = qvert(c);
    f3 e1 = pb - pa, e2 = pc - pa;
    f3 n = cross(e1, e2);
    float bf = l1(e1) * l1(e2);
    uint32_t* w = F(f);
    w[0] = a | ALIVE; w[1] = b; w[2] = c; w[3] = fbits(bf);
    w[4] = fbits(n.x); w[5] = fbits(n.y); w[6] = fbits(n.z); w[7] = fbits(pa.x);
    w[8] = fbits(pa.y); w[9] = fbits(pa.z); w[10] = fbits(pb.x); w[11] = fbits(pb.y);
    w[12] = fbits(pb.z); w[13] = fbits(pc.x); w[14] = fbits(pc.y); w[15] = fbits(pc.z);
  }
  // shaders.ts:906-921 — positive = visible (ranking value), negative = not
  float face_eval(uint32_t f, f3 p) {
    uint32_t* w = F(f);
    if ((w[0] & ALIVE) == 0) return -1e30f;
    f3 n = mk3(bitsf(w[4]), bitsf(w[5]), bitsf(w[6]));
    f3 a = mk3(bitsf(w[7]), bitsf(w[8]), bitsf(w[9]));
    f3 d = p - a;
    float det = dot(n, d);
    float bound = (1e-6f * bitsf(w[3])) * l1(d);
    if (det > bound) return det / vmax(std::sqrt(dot(n, n)), 1e-30f);
    if (det < -bound) return -1.0f;
    f3 b = mk3(bitsf(w[10]), bitsf(w[11]), bitsf(w[12]));
    f3 c = mk3(bitsf(w[13]), bitsf(w[14]), bitsf(w[15]));
    int sg = orient_exact(b - a, c - a, d);
    return sg > 0 ? 1e-30f : -1.0f;
  }
  void compact() {  // shaders.ts:946-969
    uint32_t run = 0;
    for (uint32_t f = 0; f < nf; f++) {
      if (!alive(f)) continue;
      if (run != f) std::copy(F(f), F(f) + FW, F(run));
      run++;
    }
    nf = run;
    compacted = true;
  }
  static bool shares_edge(const uint32_t f[3], const uint32_t g[3]) {
    for (int k = 0; k < 3; k++) {
      uint32_t a = f[k], b = f[(k + 1) % 3];
      if ((g[0] == b && g[1] == a) || (g[1] == b && g[2] == a) || (g[2] == b && g[0] == a)) return true;
    }
    return false;
  }
  // shaders.ts:975-1055
  void insert(uint32_t pIdx) {
    f3 p = qvert(pIdx);
    if (nf + 3 * ORC_VIS_MAX > fmax || nf > 2 * nalive + 512) compact();
    std::vector<uint32_t> vis;
    std::vector<float> vd;
    for (uint32_t f = 0; f < nf; f++) {
      float dd = face_eval(f, p);
      if (dd > 0.0f) { vis.push_back(f); vd.push_back(dd); }
    }
    uint32_t nvis = (uint32_t)vis.size();
    if (nvis == 0) return;
    if (nvis > ORC_VIS_MAX) { fail = 1; return; }
    uint32_t seedK = 0;
    for (uint32_t k = 1; k < nvis; k++) if (vd[k] > vd[seedK]) seedK = k;
    std::vector<uint32_t> fa(3 * nvis);
    for (uint32_t k = 0; k < nvis; k++) face_abc(vis[k], fa[3 * k], fa[3 * k + 1], fa[3 * k + 2]);
    std::vector<char> conn(nvis, 0);
    conn[seedK] = 1;
    for (;;) {
      bool changed = false;
      for (uint32_t i = 0; i < nvis; i++) {
        if (conn[i]) continue;
        for (uint32_t j = 0; j < nvis; j++) {
          if (j != i && conn[j] && shares_edge(&fa[3 * i], &fa[3 * j])) { conn[i] = 1; changed = true; break; }
        }
      }
      if (!changed) break;
    }
    if (nf + 3 * nvis > fmax) { fail = 2; return; }
    uint32_t nnew = 0;
    for (uint32_t e = 0; e < 3 * nvis; e++) {
      uint32_t vi = e / 3, k = e % 3;
      if (!conn[vi]) continue;
      uint32_t a = fa[3 * vi + k], b = fa[3 * vi + (k + 1) % 3];
      bool found = false;
      for (uint32_t j = 0; j < nvis && !found; j++) {
        if (!conn[j]) continue;
        const uint32_t* g = &fa[3 * j];
        if ((g[0] == b && g[1] == a) || (g[1] == b && g[2] == a) || (g[2] == b && g[0] == a)) found = true;
      }
      if (!found) { face_write(nf + nnew, a, b, pIdx); nnew++; }
    }
    uint32_t killed = 0;
    for (uint32_t vi = 0; vi < nvis; vi++) if (conn[vi]) { F(vis[vi])[0] &= 0x7fffffffu; killed++; }
    nf += nnew;
    nalive = nalive + nnew - killed;
  }
  void assign(uint32_t i, uint32_t f0, uint32_t f1) {
    f3 pt = qvert(i);
    uint32_t bestF = NONE;
    float bestD = -1.0f;
    for (uint32_t f = f0; f < f1; f++) {
      float dd = face_eval(f, pt);
      if (dd > 0.0f && dd > bestD) { bestD = dd; bestF = f; }
    }
    owner[i] = bestF;
    dist[i] = bestF != NONE ? bestD : 0.0f;
  }
  // shaders.ts:1060-1129
  uint32_t grow(uint32_t& ncand, uint32_t nfPrev, uint32_t maxIter) {
    uint32_t sinceCompact = 0, nIns = 0;
    for (uint32_t iter = 0; iter < maxIter; iter++) {
      if (ncand == 0) break;
      float md = -1.0f;
      uint32_t mi = NONE;
      for (uint32_t k = 0; k < ncand; k++) {
        uint32_t i = cand[k];
        if (owner[i] == NONE) continue;
        float dd = dist[i];
        if (dd > md || (dd == md && i < mi)) { md = dd; mi = i; }
      }
      if (md < 0.0f) break;
      uint32_t pick = mi;
      compacted = false;
      insert(pick);
      nIns++;
      if (fail) break;
      uint32_t nfNow = nf;
      owner[pick] = NONE;
      dist[pick] = 0.0f;
      for (uint32_t k = 0; k < ncand; k++) {
        uint32_t i = cand[k];
        uint32_t own = owner[i];
        if (own == NONE) continue;
        if (!compacted && alive(own)) continue;
        assign(i, compacted ? 0 : nfPrev, nfNow);
      }
      nfPrev = nfNow;
      if (++sinceCompact >= 4) {
        sinceCompact = 0;
        uint32_t nc = 0;
        for (uint32_t k = 0; k < ncand; k++) if (owner[cand[k]] != NONE) cand[nc++] = cand[k];
        ncand = nc;
      }
    }
    return nIns;
  }
  // exact volume of the alive faces, in grid units
  double volume_grid() {
    uint32_t a0, b0, c0;
    face_abc(0, a0, b0, c0);
    f3 of = qvert(a0);
    int64_t ox = (int64_t)of.x, oy = (int64_t)of.y, oz = (int64_t)of.z;
    i128 v6 = 0;
    for (uint32_t f = 0; f < nf; f++) {
      if (!alive(f)) continue;
      uint32_t a, b, c;
      face_abc(f, a, b, c);
      f3 pa = qvert(a), pb = qvert(b), pc = qvert(c);
      int64_t ax = (int64_t)pa.x - ox, ay = (int64_t)pa.y - oy, az = (int64_t)pa.z - oz;
      int64_t bx = (int64_t)pb.x - ox, by = (int64_t)pb.y - oy, bz = (int64_t)pb.z - oz;
      int64_t cx = (int64_t)pc.x - ox, cy = (int64_t)pc.y - oy, cz = (int64_t)pc.z - oz;
      int64_t nx = by * cz - bz * cy, ny = bz * cx - bx * cz, nz = bx * cy - by * cx;
      v6 += (i128)ax * nx + (i128)ay * ny + (i128)az * nz;
    }
    if (v6 < 0) v6 = -v6;
    return i128_to_double(v6) / 6.0;
  }
  static double i128_to_double(i128 v) {
    int64_t hi = (int64_t)(v >> 32);
    uint32_t lo = (uint32_t)(v & 0xffffffffu);
    return (double)hi * 4294967296.0 + (double)lo;
  }
};

// rv cost (part.ts:24-26; shaders.ts:154-157), in double for the gap and the
// cube root, rounded to float32
float rv_cost(float meshVol, float hullVol) {
  double gap = (double)hullVol - (double)meshVol;
  if (gap < 0.0) gap = 0.0;
  return (float)(0.3 * std::cbrt(0.238732414637843 * gap));
}

HullResult hull_points(const f3* pts, uint32_t nv, uint32_t slabWords, const HullOpts& o) {
  HullResult r;
  uint32_t fb = (2 * nv + std::max(nv, 80u) + 7) & ~7u;
  uint32_t fmax = slabWords > fb ? (slabWords - fb) / FW : 0;
  if (fmax < 64) { r.hullVol = -1.0f; r.status = 3; return r; }
  Hull h;
  h.pts = pts; h.nv = nv; h.fmax = fmax;
  h.faces.assign((size_t)FW * fmax, 0);
  h.owner.assign(nv, NONE);
  h.dist.assign(nv, 0.0f);
  h.cand.assign(std::max(nv, 80u), 0);
  f3 lo = mk3(1e30f, 1e30f, 1e30f), hi = mk3(-1e30f, -1e30f, -1e30f);
  for (uint32_t i = 0; i < nv; i++) { lo = vmin3(lo, pts[i]); hi = vmax3(hi, pts[i]); }
  f3 ext = hi - lo;
  float scale = vmax(vmax(vmax(ext.x, ext.y), ext.z), 1e-30f);
  h.qlo = lo;
  h.qs = 2097152.0f / scale;
  float cell = scale / 2097152.0f;
  float volScale = (cell * cell) * cell;
  // k-DOP extremes: rows max a0, min a0, max a1, min a1 per pass
  uint32_t seed[80];
  for (int ps = 0; ps < 20; ps++) {
    f3 a0 = mk3(KDOP[2 * ps][0], KDOP[2 * ps][1], KDOP[2 * ps][2]);
    f3 a1 = mk3(KDOP[2 * ps + 1][0], KDOP[2 * ps + 1][1], KDOP[2 * ps + 1][2]);
    float mx0 = -1e30f, mx1 = -1e30f, mn0 = 1e30f, mn1 = 1e30f;
    uint32_t ix0 = 0, ix1 = 0, in0 = 0, in1 = 0;
    for (uint32_t i = 0; i < nv; i++) {
      f3 v = h.qvert(i);
      float d0 = dot(a0, v), d1 = dot(a1, v);
      if (d0 > mx0) { mx0 = d0; ix0 = i; }
      if (d0 < mn0) { mn0 = d0; in0 = i; }
      if (d1 > mx1) { mx1 = d1; ix1 = i; }
      if (d1 < mn1) { mn1 = d1; in1 = i; }
    }
    seed[4 * ps] = ix0; seed[4 * ps + 1] = in0; seed[4 * ps + 2] = ix1; seed[4 * ps + 3] = in1;
  }
  if (o.hullStage == 1) { r.hullVol = 0.0f; return r; }
  // initial simplex (shaders.ts:1227-1263)
  uint32_t i0 = seed[1], i1 = seed[0];
  f3 p0 = h.qvert(i0), p1 = h.qvert(i1);
  f3 d01 = p1 - p0;
  uint32_t i2 = NONE;
  float best = 0.0f;
  for (int k = 0; k < 80; k++) {
    f3 c = cross(d01, h.qvert(seed[k]) - p0);
    float v = dot(c, c);
    if (v > best) { best = v; i2 = seed[k]; }
  }
  if (i2 == NONE) { r.hullVol = 0.0f; return r; }
  f3 p2 = h.qvert(i2);
  f3 e2 = p2 - p0;
  f3 n = cross(d01, e2);
  float bd = 0.0f;
  int bs = 0;
  uint32_t i3 = NONE;
  for (int k = 0; k < 80; k++) {
    f3 dk = h.qvert(seed[k]) - p0;
    float v = std::fabs(dot(n, dk));
    if (v > bd) {
      int sgn = orient_filtered(n, d01, e2, dk);
      if (sgn != 0) { bd = v; i3 = seed[k]; bs = sgn; }
    }
  }
  if (i3 == NONE) { r.hullVol = 0.0f; return r; }
  uint32_t a = i0, b = i1, c = i2;
  if (bs > 0) { b = i2; c = i1; }
  h.face_write(0, a, b, c);
  h.face_write(1, a, i3, b);
  h.face_write(2, b, i3, c);
  h.face_write(3, c, i3, a);
  h.nf = 4; h.nalive = 4;
  // seeds first, farthest first
  for (int k = 0; k < 80; k++) {
    h.assign(seed[k], 0, 4);
    h.cand[k] = seed[k];
  }
  uint32_t ncand = 80;
  uint32_t nIns = h.grow(ncand, 4, 80);
  uint32_t fail0 = h.fail;
  uint32_t nfPrev = h.nf;
  if (o.prune && fail0 == 0) {
    float vRough = (float)(h.volume_grid() * (double)volScale);
    float bound = o.prunePartial + rv_cost(o.meshVol, vRough);
    if (bound > o.pruneUb) {
      r.hullVol = vRough; r.pruned = true; r.nIns = nIns;
      return r;
    }
  }
  ncand = 0;
  if (fail0 == 0) {
    for (uint32_t i = 0; i < nv; i++) {
      h.assign(i, 0, nfPrev);
      if (h.owner[i] != NONE) h.cand[ncand++] = i;
    }
  }
  r.ncand = ncand;
  r.assigned = true;
  uint32_t maxIter = (o.hullStage == 2 || o.hullStage == 3 || fail0 != 0) ? 0 : nv;
  nIns += h.grow(ncand, nfPrev, maxIter);
  if (h.fail) { r.hullVol = -1.0f; r.status = h.fail; r.nIns = nIns; return r; }
  r.hullVol = (float)(h.volume_grid() * (double)volScale);
  r.nIns = nIns;
  for (uint32_t f = 0; f < h.nf; f++) {
    if (!h.alive(f)) continue;
    uint32_t fa, fb2, fc;
    h.face_abc(f, fa, fb2, fc);
    r.faces.push_back(fa); r.faces.push_back(fb2); r.faces.push_back(fc);
  }
  return r;
}

}  // namespace orc
