// tree_oracle.cpp — CPU restatement of the reference's lookahead tree
// (GpuTree in src/gpu/tree.ts and the plan / scan / emit / record / evaluate
// kernels of src/gpu/shaders.ts), run sequentially in a fixed order.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine.
//
// Tables use the reference's word layouts (shaders.ts:30-60): a part is 16
// words, an item 20, a job 24; geometry lives in one u32 pool with vertex
// floats, triangle indices and 8-word open edges (shaders.ts:4-10). Offsets
// follow the reference's units (floats, u32s, edges).
//
// Two deliberate differences from the WGSL, shared with the CUDA engine:
// per-job flux sums are accumulated in double (the WGSL reduces float32 in
// a tree whose shape is an implementation detail), and hull volumes are
// exact (hull_oracle.cpp). Everything else is the same float32 arithmetic in
// the same operation order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "oracle.h"
#include "oracle_api.h"

namespace orc {

static const uint32_t NONE = 0xffffffffu;
enum { CTR_V = 0, CTR_T = 1, CTR_E = 2, CTR_S = 3, CTR_OVERFLOW = 4, CTR_HULLFAIL = 5, CTR_NPOVER = 6, CTR_PRUNED = 7 };
static const uint32_t HD_MAX_PAIRS = 1024;
static const float PC_EPS = 1e-6f;

struct Params {
  uint32_t itemsInBase = 0, nItemsIn = 0, itemsOutBase = 0, jobBase = 0;
  uint32_t width = 0, nEdgeCuts = 0, edgeStride = 0, totalWidth = 0;
  float minEdgeDist = 0;
  uint32_t level = 0, totalLevels = 0, partBase = 0;
  uint32_t edgePlaneBase = 0, hullChunkBase = 0, hullSlabWords = 0, nChildParts = 0;
  uint32_t nJobs = 0, hullChunkSize = 0, exportBase = 0, exportStride = 0;
  uint32_t lastLevel = 0, hullStage = 0, nSeeds = 0;
};

struct Poly { uint32_t n = 0; uint32_t src[4] = {0, 0, 0, 0}; };
struct PolyStats { uint32_t ntri = 0, nnew = 0, nedge = 0; };

static int vsign(float d) { return d > PC_EPS ? 1 : (d < -PC_EPS ? -1 : 0); }

// shaders.ts:171-181
static Poly clip_tri(const int sg[3], int side) {
  Poly p;
  for (uint32_t k = 0; k < 3; k++) {
    uint32_t q = (k + 1) % 3;
    int sp = sg[k] * side, sq = sg[q] * side;
    if (sp >= 0) p.src[p.n++] = k;
    if (sg[k] != 0 && sg[q] != 0 && sp * sq < 0) p.src[p.n++] = 4 + k;
  }
  return p;
}
// shaders.ts:184-198
static PolyStats poly_stats(const Poly& p, const int sg[3]) {
  PolyStats st;
  st.ntri = p.n >= 3 ? p.n - 2 : 0;
  if (p.n >= 3) {
    for (uint32_t i = 0; i < p.n; i++) {
      uint32_t u = p.src[i], v = p.src[(i + 1) % p.n];
      if (u >= 4) st.nnew++;
      bool uOn = u >= 4 || sg[u] == 0;
      bool vOn = v >= 4 || sg[v] == 0;
      if (uOn && vOn) st.nedge++;
    }
  }
  return st;
}

static f3 plane_point(f4 pl) {
  f3 n = xyz(pl);
  float n2 = vmax(dot(n, n), 1e-30f);
  return ((-pl.w) * n) / n2;
}
// shaders.ts:123-143
static f3 anchor_for(const f4* pl, uint32_t n) {
  if (n == 0) return mk3(0, 0, 0);
  if (n == 1) return plane_point(pl[0]);
  if (n >= 3) {
    f3 n1 = xyz(pl[n - 3]), n2 = xyz(pl[n - 2]), n3 = xyz(pl[n - 1]);
    float det = dot(n1, cross(n2, n3));
    if (std::fabs(det) > 1e-4f) {
      float e1 = -pl[n - 3].w, e2 = -pl[n - 2].w, e3 = -pl[n - 1].w;
      return ((e1 * cross(n2, n3) + e2 * cross(n3, n1)) + e3 * cross(n1, n2)) / det;
    }
  }
  f4 a = pl[n - 2], b = pl[n - 1];
  f3 L = cross(xyz(a), xyz(b));
  float l2 = dot(L, L);
  if (l2 > 1e-8f) {
    float e1 = -a.w, e2 = -b.w;
    return (e1 * cross(xyz(b), L) + e2 * cross(L, xyz(a))) / l2;
  }
  return plane_point(b);
}
static float tri_flux(f3 a, f3 b, f3 c, f3 o) { return dot(a - o, cross(b - o, c - o)) / 6.0f; }
static float edge_term(f3 p, f3 q, f3 c, f3 o) { return dot(c - o, cross(q - o, p - o)) / 6.0f; }

struct Tree {
  orc_config cfg;
  uint32_t edgeStride;
  std::vector<uint32_t> pool, scratch, ctr;
  std::vector<uint32_t> parts, items, jobs;  // 16 / 20 / 24 words per record
  std::vector<f4> planes;
  uint32_t capSeeds = 0, capJobs = 0, capItems = 0, capParts = 0, capPlanes = 0;
  uint32_t vBase = 0, tBase = 0, eBase = 0;
  // last run
  std::vector<uint32_t> jobsPerLevel;
  uint64_t validJobs = 0;
  uint32_t lastItems = 0;
  uint32_t lastHullSlabWords = 0;

  explicit Tree(const orc_config& c) : cfg(c) {
    if (c.width % 3 != 0 || c.width2 % 3 != 0) throw std::runtime_error("width and width2 must be multiples of 3");
    if (c.depth < 1 || c.depth > 4) throw std::runtime_error("depth must be in 1..4");
    edgeStride = (uint32_t)std::max(4 * c.nConcaveEdges, 32);
    vBase = 0;
    tBase = (uint32_t)c.vertexCap;
    eBase = (uint32_t)(c.vertexCap + c.triCap);
    pool.assign(c.vertexCap + c.triCap + 8 * c.edgeCap, 0);
    scratch.assign(c.scratchWords, 0);
    ctr.assign(8 + HD_MAX_PAIRS, 0);
    ensureTables(16);
  }
  // record accessors
  uint32_t* part(uint32_t i) { return &parts[16 * (size_t)i]; }
  uint32_t* item(uint32_t i) { return &items[20 * (size_t)i]; }
  uint32_t* job(uint32_t i) { return &jobs[24 * (size_t)i]; }
  f3 vert(uint32_t off, uint32_t i) {
    size_t b = vBase + (size_t)off + 3 * (size_t)i;
    return mk3(bitsf(pool[b]), bitsf(pool[b + 1]), bitsf(pool[b + 2]));
  }
  void put_vert(uint32_t off, uint32_t i, f3 p) {
    size_t b = vBase + (size_t)off + 3 * (size_t)i;
    pool[b] = fbits(p.x); pool[b + 1] = fbits(p.y); pool[b + 2] = fbits(p.z);
  }
  void tri(uint32_t off, uint32_t t, uint32_t r[3]) {
    size_t b = tBase + (size_t)off + 3 * (size_t)t;
    r[0] = pool[b]; r[1] = pool[b + 1]; r[2] = pool[b + 2];
  }
  void put_tri(const Params& P, uint32_t off, uint32_t t, uint32_t a, uint32_t b, uint32_t c) {
    if (P.lastLevel) return;
    size_t k = tBase + (size_t)off + 3 * (size_t)t;
    pool[k] = a; pool[k + 1] = b; pool[k + 2] = c;
  }
  f3 edge_p(uint32_t off, uint32_t e) {
    size_t b = eBase + 8 * ((size_t)off + e);
    return mk3(bitsf(pool[b]), bitsf(pool[b + 1]), bitsf(pool[b + 2]));
  }
  f3 edge_q(uint32_t off, uint32_t e) {
    size_t b = eBase + 8 * ((size_t)off + e) + 3;
    return mk3(bitsf(pool[b]), bitsf(pool[b + 1]), bitsf(pool[b + 2]));
  }
  uint32_t edge_plane(uint32_t off, uint32_t e) { return pool[eBase + 8 * ((size_t)off + e) + 6]; }
  void put_edge(const Params& P, uint32_t off, uint32_t e, f3 p, f3 q, uint32_t pl) {
    if (P.lastLevel) return;
    size_t b = eBase + 8 * ((size_t)off + e);
    pool[b] = fbits(p.x); pool[b + 1] = fbits(p.y); pool[b + 2] = fbits(p.z);
    pool[b + 3] = fbits(q.x); pool[b + 4] = fbits(q.y); pool[b + 5] = fbits(q.z);
    pool[b + 6] = pl; pool[b + 7] = 0;
  }

  // tree.ts:191-213
  void ensureTables(uint32_t nSeeds) {
    if (nSeeds <= capSeeds) return;
    uint32_t w0 = (uint32_t)cfg.width + edgeStride;
    uint64_t nItemsIn = nSeeds, totalJobs = 0;
    for (int l = 0; l < cfg.depth; l++) {
      uint64_t w = l == 0 ? w0 : (uint64_t)cfg.width2;
      totalJobs += nItemsIn * w;
      nItemsIn *= w;
    }
    uint64_t nItems = nSeeds + totalJobs;
    uint64_t nParts = std::max<uint64_t>(nSeeds + 2 * totalJobs, capParts);
    uint64_t nPlanes = totalJobs + (uint64_t)nSeeds * edgeStride + 16 + 4 * (uint64_t)nSeeds;
    parts.assign(16 * nParts, 0);
    items.assign(20 * nItems, 0);
    jobs.assign(24 * std::max<uint64_t>(totalJobs, 1), 0);
    planes.assign(std::max<uint64_t>(nPlanes, 1), f4{0, 0, 0, 0});
    capSeeds = nSeeds; capJobs = (uint32_t)totalJobs; capItems = (uint32_t)nItems;
    capParts = (uint32_t)nParts; capPlanes = (uint32_t)nPlanes;
  }
  void ensurePartSlots(uint32_t n) {
    if (n <= capParts) return;
    parts.assign(16 * (size_t)n, 0);
    capParts = n;
  }

  // tree.ts:233-278
  void uploadSeeds(const orc_mesh* seeds, uint32_t n, uint32_t& vTop, uint32_t& tTop) {
    uint64_t totV = 0, totT = 0;
    for (uint32_t k = 0; k < n; k++) { totV += 3ull * seeds[k].nv; totT += 3ull * seeds[k].nt; }
    if (totV > cfg.vertexCap || totT > cfg.triCap) throw std::runtime_error("seed meshes exceed pool capacity");
    vTop = 0; tTop = 0;
    for (uint32_t k = 0; k < n; k++) {
      const orc_mesh& m = seeds[k];
      std::memcpy(&pool[vBase + vTop], m.verts, 12ull * m.nv);
      if (m.nt) std::memcpy(&pool[tBase + tTop], m.tris, 12ull * m.nt);
      uint32_t* p = part(k);
      std::memset(p, 0, 64);
      p[0] = vTop; p[1] = m.nv; p[2] = tTop; p[3] = m.nt;
      p[8] = p[9] = p[10] = p[11] = NONE;
      p[12] = 0;
      p[13] = m.nt == 0 ? 2 : 0;
      vTop += 3 * m.nv;
      tTop += 3 * m.nt;
    }
    std::fill(ctr.begin(), ctr.begin() + 8, 0u);
    ctr[0] = vTop; ctr[1] = tTop;
    for (uint32_t k = 0; k < n && k < capItems; k++) {
      uint32_t* it = item(k);
      std::memset(it, 0, 80);
      it[0] = k; it[8] = 1; it[9] = k; it[10] = NONE; it[11] = 0; it[16] = 1; it[17] = NONE;
    }
  }

  uint32_t hullSlabWords(const orc_mesh* m, uint32_t n) {
    uint32_t maxNv = 0;
    for (uint32_t k = 0; k < n; k++) maxNv = std::max(maxNv, m[k].nv);
    uint32_t fmax = 2 * std::min<uint32_t>((uint32_t)cfg.hullMaxVerts, maxNv) + 3 * ORC_VIS_MAX + 1024;
    return ((2 * maxNv + std::max(maxNv, 80u) + 7) & ~7u) + 16 * fmax;
  }

  // ---- plan: shaders.ts:296-444 ----
  void plan(const Params& P) {
    for (uint32_t g = 0; g < P.nJobs; g++) {
      uint32_t itemIdx = g / P.totalWidth, cut = g % P.totalWidth, jobIdx = P.jobBase + g;
      uint32_t* J = job(jobIdx);
      std::memset(J, 0, 96);
      J[4] = itemIdx; J[7] = cut;
      planes[jobIdx] = f4{0, 0, 0, 0};
      uint32_t* it = item(P.itemsInBase + itemIdx);
      if (!(it[16] == 1 && it[8] > 0)) continue;
      uint32_t partId = it[it[8] - 1];
      uint32_t* pd = part(partId);
      J[5] = partId;
      uint32_t vOff = pd[0], unv = pd[1], tOff = pd[2], unt = pd[3], eOff = pd[4], une = pd[5];
      f3 lo = mk3(1e30f, 1e30f, 1e30f), hi = mk3(-1e30f, -1e30f, -1e30f);
      for (uint32_t i = 0; i < unv; i++) { f3 p = vert(vOff, i); lo = vmin3(lo, p); hi = vmax3(hi, p); }
      f3 ext = hi - lo;
      float lim = 2.0f * P.minEdgeDist + 1e-6f;
      if (ext.x <= lim && ext.y <= lim && ext.z <= lim) {
        if (cut == 0) {
          uint32_t lvl = std::min(P.totalLevels, 4u);
          for (uint32_t l = it[11]; l < lvl; l++) it[12 + l] = fbits(0.0f);
          it[11] = lvl;
          it[16] = 2;
        }
        continue;
      }
      f4 pl0{0, 0, 0, 0};
      uint32_t ok = 1;
      if (cut >= P.width) {
        pl0 = planes[P.edgePlaneBase + it[9] * P.edgeStride + (cut - P.width)];
        ok = dot(xyz(pl0), xyz(pl0)) > 0.0f ? 1 : 0;
      } else {
        uint32_t cpa = P.width / 3;
        uint32_t axis = cut / cpa, slice = cut % cpa;
        float loV = comp(lo, axis) + P.minEdgeDist;
        float hiV = comp(hi, axis) - P.minEdgeDist;
        if (loV >= hiV) ok = 0;
        float frac = ((float)slice + 1.0f) / ((float)cpa + 1.0f);
        float pos = loV + frac * (hiV - loV);
        pl0 = f4{axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f, -pos};
      }
      uint32_t sOff = 0;
      if (ok) {
        sOff = ctr[CTR_S];
        ctr[CTR_S] += 2 * unv;
        if ((uint64_t)sOff + 2 * unv > cfg.scratchWords) { ok = 0; ctr[CTR_OVERFLOW] = 1; }
      }
      if (!ok) continue;
      f4 pl = pl0;
      f3 n = xyz(pl);
      for (uint32_t i = 0; i < unv; i++) { scratch[sOff + 2 * i] = 0; scratch[sOff + 2 * i + 1] = 0; }
      uint32_t posT = 0, negT = 0, posNew = 0, negNew = 0, posE = 0, negE = 0;
      for (uint32_t t = 0; t < unt; t++) {
        uint32_t tr[3];
        tri(tOff, t, tr);
        float d[3];
        for (int k = 0; k < 3; k++) d[k] = dot(n, vert(vOff, tr[k])) + pl.w;
        int sg[3] = {vsign(d[0]), vsign(d[1]), vsign(d[2])};
        if (sg[0] == 0 && sg[1] == 0 && sg[2] == 0) continue;
        Poly pp = clip_tri(sg, 1), pn = clip_tri(sg, -1);
        PolyStats sp = poly_stats(pp, sg), sn = poly_stats(pn, sg);
        posT += sp.ntri; posNew += sp.nnew; posE += sp.nedge;
        negT += sn.ntri; negNew += sn.nnew; negE += sn.nedge;
        if (pp.n >= 3) for (uint32_t i = 0; i < pp.n; i++) if (pp.src[i] < 4) scratch[sOff + 2 * tr[pp.src[i]]] = 1;
        if (pn.n >= 3) for (uint32_t i = 0; i < pn.n; i++) if (pn.src[i] < 4) scratch[sOff + 2 * tr[pn.src[i]] + 1] = 1;
      }
      uint32_t posKept = 0, negKept = 0;
      for (uint32_t i = 0; i < unv; i++) { posKept += scratch[sOff + 2 * i]; negKept += scratch[sOff + 2 * i + 1]; }
      for (uint32_t e = 0; e < une; e++) {
        float dp = dot(n, edge_p(eOff, e)) + pl.w;
        float dq = dot(n, edge_q(eOff, e)) + pl.w;
        bool sp = dp >= 0.0f, sq = dq >= 0.0f;
        if (sp == sq) { if (sp) posE++; else negE++; } else { posE++; negE++; }
      }
      std::memcpy(J, &pl, 16);
      J[6] = 1;
      J[8] = posKept + posNew; J[9] = posT; J[10] = posE;
      J[11] = negKept + negNew; J[12] = negT; J[13] = negE;
      J[14] = posKept; J[15] = negKept;
      J[16 + 6] = sOff;
      planes[jobIdx] = pl;
      validJobs++;
    }
  }

  // ---- scan: shaders.ts:446-554 (sequential) ----
  void scan(const Params& P) {
    uint64_t run[4] = {ctr[CTR_V], ctr[CTR_T], ctr[CTR_E], ctr[CTR_S]};
    bool keepTopo = P.lastLevel == 0;
    for (uint32_t j = 0; j < P.nJobs; j++) {
      uint32_t* J = job(P.jobBase + j);
      uint32_t* cnt = J + 8;
      bool jv = J[6] == 1;
      uint64_t vNeed = jv ? 3ull * (cnt[0] + cnt[3]) : 0;
      uint64_t tNeed = (jv && keepTopo) ? 3ull * (cnt[1] + cnt[4]) : 0;
      uint64_t eNeed = (jv && keepTopo) ? (uint64_t)cnt[2] + cnt[5] : 0;
      uint64_t vOff = run[0], tOff = run[1], eOff = run[2];
      run[0] += vNeed; run[1] += tNeed; run[2] += eNeed;
      bool valid = jv;
      if (valid && (vOff + vNeed > cfg.vertexCap || tOff + tNeed > cfg.triCap || eOff + eNeed > cfg.edgeCap)) {
        valid = false;
        ctr[CTR_OVERFLOW] = 1;
      }
      uint32_t posP = P.partBase + 2 * j, negP = posP + 1, outIdx = P.itemsOutBase + j;
      uint32_t itv[20];
      std::memset(itv, 0, sizeof(itv));
      if (valid) {
        uint32_t parent[20];
        std::memcpy(parent, item(P.itemsInBase + J[4]), 80);
        uint32_t pp[16];
        std::memcpy(pp, part(J[5]), 64);
        uint32_t* off = J + 16;
        off[0] = (uint32_t)vOff; off[1] = (uint32_t)tOff; off[2] = (uint32_t)eOff;
        off[3] = (uint32_t)(vOff + 3ull * cnt[0]);
        off[4] = keepTopo ? (uint32_t)(tOff + 3ull * cnt[1]) : (uint32_t)tOff;
        off[5] = keepTopo ? (uint32_t)(eOff + cnt[2]) : (uint32_t)eOff;
        uint32_t pd[16];
        std::memset(pd, 0, sizeof(pd));
        pd[8] = pp[8]; pd[9] = pp[9]; pd[10] = pp[10]; pd[11] = pp[11];
        pd[12] = pp[12];
        if (pd[12] < 4) { pd[8 + pd[12]] = P.jobBase + j; pd[12]++; }
        else { pd[8] = pp[9]; pd[9] = pp[10]; pd[10] = pp[11]; pd[11] = P.jobBase + j; }
        uint32_t pos[16], neg[16];
        std::memcpy(pos, pd, 64);
        std::memcpy(neg, pd, 64);
        pos[0] = (uint32_t)vOff; pos[1] = cnt[0]; pos[2] = (uint32_t)tOff; pos[3] = keepTopo ? cnt[1] : 0;
        pos[4] = (uint32_t)eOff; pos[5] = keepTopo ? cnt[2] : 0;
        neg[0] = off[3]; neg[1] = cnt[3]; neg[2] = off[4]; neg[3] = keepTopo ? cnt[4] : 0;
        neg[4] = off[5]; neg[5] = keepTopo ? cnt[5] : 0;
        pos[13] = keepTopo ? 0 : 2; neg[13] = pos[13];
        std::memcpy(part(posP), pos, 64);
        std::memcpy(part(negP), neg, 64);
        bool bothNonEmpty = cnt[0] > 0 && cnt[1] > 0 && cnt[3] > 0 && cnt[4] > 0;
        std::memcpy(itv, parent, 80);
        if (parent[8] >= 8) {
          ctr[CTR_NPOVER] = 1;
          itv[16] = 0;
        } else if (bothNonEmpty) {
          itv[parent[8] - 1] = posP;
          itv[parent[8]] = negP;
          itv[8] = parent[8] + 1;
          itv[16] = 1;
          itv[17] = J[4];
          itv[18] = J[7];
          if (parent[11] == 0) itv[10] = J[7];
        } else {
          itv[16] = 0;
          J[6] = 2;
        }
      } else {
        J[6] = 0;
        std::memset(part(posP), 0, 64);
        std::memset(part(negP), 0, 64);
      }
      std::memcpy(item(outIdx), itv, 80);
    }
    ctr[CTR_V] = (uint32_t)std::min<uint64_t>(run[0], cfg.vertexCap);
    ctr[CTR_T] = (uint32_t)std::min<uint64_t>(run[1], cfg.triCap);
    ctr[CTR_E] = (uint32_t)std::min<uint64_t>(run[2], cfg.edgeCap);
    ctr[CTR_S] = 0;
  }

  // ---- emit: shaders.ts:556-750 ----
  void emit(const Params& P) {
    for (uint32_t g = 0; g < P.nJobs; g++) {
      uint32_t jobIdx = P.jobBase + g;
      uint32_t* J = job(jobIdx);
      if (J[6] != 1) continue;
      uint32_t pd[16];
      std::memcpy(pd, part(J[5]), 64);
      uint32_t pvOff = pd[0], unv = pd[1], ptOff = pd[2], unt = pd[3], peOff = pd[4], une = pd[5];
      f4 pl;
      std::memcpy(&pl, J, 16);
      f3 n = xyz(pl);
      f3 cP = plane_point(pl);
      f4 pls[4];
      uint32_t npl = 0;
      for (uint32_t k = 0; k < pd[12]; k++) pls[npl++] = planes[pd[8 + k]];
      if (npl < 4) pls[npl++] = pl;
      else { pls[0] = pls[1]; pls[1] = pls[2]; pls[2] = pls[3]; pls[3] = pl; }
      f3 o = anchor_for(pls, npl);
      uint32_t* off = J + 16;
      uint32_t* cnt = J + 8;
      uint32_t posV = off[0], posTo = off[1], posEo = off[2], negV = off[3], negTo = off[4], negEo = off[5];
      uint32_t sOff = off[6];
      uint32_t posKept = cnt[6], negKept = cnt[7];
      // 1. vertex remap and copy
      uint32_t rp = 0, rn = 0;
      for (uint32_t i = 0; i < unv; i++) {
        uint32_t fp = scratch[sOff + 2 * i], fn = scratch[sOff + 2 * i + 1];
        f3 p = vert(pvOff, i);
        uint32_t ip = NONE, in = NONE;
        if (fp == 1) { ip = rp++; put_vert(posV, ip, p); }
        if (fn == 1) { in = rn++; put_vert(negV, in, p); }
        scratch[sOff + 2 * i] = ip;
        scratch[sOff + 2 * i + 1] = in;
      }
      // 2. triangles
      double fluxPos = 0.0, fluxNeg = 0.0;
      uint32_t runT[2] = {0, 0}, runV[2] = {0, 0}, runE[2] = {0, 0};
      for (uint32_t t = 0; t < unt; t++) {
        uint32_t tr[3];
        tri(ptOff, t, tr);
        f3 pos3[3] = {vert(pvOff, tr[0]), vert(pvOff, tr[1]), vert(pvOff, tr[2])};
        float d[3];
        for (int k = 0; k < 3; k++) d[k] = dot(n, pos3[k]) + pl.w;
        int sg[3] = {vsign(d[0]), vsign(d[1]), vsign(d[2])};
        if (sg[0] == 0 && sg[1] == 0 && sg[2] == 0) continue;
        Poly polys[2] = {clip_tri(sg, 1), clip_tri(sg, -1)};
        for (int side = 0; side < 2; side++) {
          bool isPos = side == 0;
          const Poly& poly = polys[side];
          PolyStats st = poly_stats(poly, sg);
          if (poly.n < 3) continue;
          uint32_t vOff = isPos ? posV : negV, tOff = isPos ? posTo : negTo, eOff = isPos ? posEo : negEo;
          uint32_t kept = isPos ? posKept : negKept;
          uint32_t tB = runT[side];
          uint32_t vB = kept + runV[side];
          uint32_t eB = runE[side];
          uint32_t idx[4];
          f3 pts[4];
          bool onp[4];
          for (uint32_t i = 0; i < poly.n; i++) {
            uint32_t u = poly.src[i];
            if (u < 4) {
              idx[i] = scratch[sOff + 2 * tr[u] + (isPos ? 0 : 1)];
              pts[i] = pos3[u];
              onp[i] = sg[u] == 0;
            } else {
              uint32_t k = u - 4, q = (k + 1) % 3;
              float tt = d[k] / (d[k] - d[q]);
              f3 x = pos3[k] + tt * (pos3[q] - pos3[k]);
              put_vert(vOff, vB, x);
              idx[i] = vB++;
              pts[i] = x;
              onp[i] = true;
            }
          }
          float flux = 0.0f;
          for (uint32_t i = 1; i + 1 < poly.n; i++) {
            put_tri(P, tOff, tB, idx[0], idx[i], idx[i + 1]);
            tB++;
            flux += tri_flux(pts[0], pts[i], pts[i + 1], o);
          }
          for (uint32_t i = 0; i < poly.n; i++) {
            uint32_t j2 = (i + 1) % poly.n;
            if (onp[i] && onp[j2]) {
              put_edge(P, eOff, eB, pts[i], pts[j2], jobIdx);
              eB++;
              flux += edge_term(pts[i], pts[j2], cP, o);
            }
          }
          if (isPos) fluxPos += (double)flux; else fluxNeg += (double)flux;
          runT[side] += st.ntri; runV[side] += st.nnew; runE[side] += st.nedge;
        }
      }
      // 3. inherited open edges
      for (uint32_t e = 0; e < une; e++) {
        f3 p = edge_p(peOff, e), q = edge_q(peOff, e);
        uint32_t pid = edge_plane(peOff, e);
        float dp = dot(n, p) + pl.w, dq = dot(n, q) + pl.w;
        f3 cE = plane_point(planes[pid]);
        bool sp = dp >= 0.0f, sq = dq >= 0.0f;
        if (sp == sq) {
          if (sp) { put_edge(P, posEo, runE[0]++, p, q, pid); fluxPos += (double)edge_term(p, q, cE, o); }
          else { put_edge(P, negEo, runE[1]++, p, q, pid); fluxNeg += (double)edge_term(p, q, cE, o); }
        } else {
          float tt = dp / (dp - dq);
          f3 x = p + tt * (q - p);
          if (sp) {
            put_edge(P, posEo, runE[0]++, p, x, pid); fluxPos += (double)edge_term(p, x, cE, o);
            put_edge(P, negEo, runE[1]++, x, q, pid); fluxNeg += (double)edge_term(x, q, cE, o);
          } else {
            put_edge(P, negEo, runE[1]++, p, x, pid); fluxNeg += (double)edge_term(p, x, cE, o);
            put_edge(P, posEo, runE[0]++, x, q, pid); fluxPos += (double)edge_term(x, q, cE, o);
          }
        }
      }
      part(P.partBase + 2 * g)[6] = fbits((float)std::fabs(fluxPos));
      part(P.partBase + 2 * g + 1)[6] = fbits((float)std::fabs(fluxNeg));
    }
  }

  // ---- hull over the child parts: shaders.ts:1144-1400 ----
  void hull(const Params& P) {
    for (uint32_t idx = 0; idx < P.nChildParts; idx++) {
      uint32_t partIdx = P.partBase + idx;
      uint32_t* pd = part(partIdx);
      uint32_t nv = pd[1], nt = pd[3], vOff = pd[0], flags = pd[13];
      if (!(nv >= 4 && (nt > 0 || (flags & 2) != 0))) { pd[7] = fbits(0.0f); continue; }
      std::vector<f3> pts(nv);
      for (uint32_t i = 0; i < nv; i++) pts[i] = vert(vOff, i);
      HullOpts o;
      o.hullStage = (int)P.hullStage;
      o.meshVol = bitsf(pd[6]);
      if (P.lastLevel == 1 && P.level > 0 && P.nSeeds > 0 && P.exportStride == 0) {
        uint32_t* jb = job(P.jobBase + idx / 2);
        uint32_t* pit = item(P.itemsInBase + jb[4]);
        float ssum = 0.0f;
        for (uint32_t l = 0; l < pit[11]; l++) ssum += bitsf(pit[12 + l]);
        uint32_t perSeed = P.nItemsIn / P.nSeeds;
        float ub = 1e30f;
        for (uint32_t i = 0; i < perSeed; i++) {
          uint32_t* it = item(P.itemsInBase + pit[9] * perSeed + i);
          if (it[16] == 1 && it[11] > 0) {
            float ps = 0.0f;
            for (uint32_t l = 0; l < it[11]; l++) ps += bitsf(it[12 + l]);
            float u = ps + bitsf(it[12 + it[11] - 1]) * (float)(P.totalLevels - it[11]);
            ub = vmin(ub, u);
          }
        }
        o.prune = true;
        o.prunePartial = ssum;
        o.pruneUb = ub;
      }
      HullResult r = hull_points(pts.data(), nv, P.hullSlabWords, o);
      if (r.pruned) {
        pd[7] = fbits(r.hullVol);
        pd[13] |= 4;
        ctr[CTR_PRUNED]++;
        continue;
      }
      if (r.assigned && P.exportStride == 0) pd[14] = r.ncand;
      if (r.status != 0) {
        pd[7] = fbits(-1.0f);
        pd[13] = r.status;
        ctr[CTR_HULLFAIL]++;
        continue;
      }
      pd[7] = fbits(r.hullVol);
      pd[15] = r.nIns;
      if (P.exportStride != 0) {
        uint32_t nfx = (uint32_t)r.faces.size() / 3;
        uint32_t base = tBase + P.exportBase + (P.hullChunkBase + idx) * P.exportStride;
        uint32_t w = 0;
        for (uint32_t f = 0; f < nfx; f++) {
          if (3 * f + 3 > P.exportStride) break;
          pool[base + 3 * f] = r.faces[3 * f];
          pool[base + 3 * f + 1] = r.faces[3 * f + 1];
          pool[base + 3 * f + 2] = r.faces[3 * f + 2];
          w++;
        }
        pd[14] = std::min(nfx, P.exportStride / 3);
        (void)w;
        if (P.nJobs != 0) {
          uint32_t* hd = part(partIdx + P.nJobs);
          std::memset(hd, 0, 64);
          hd[0] = vOff; hd[1] = nv; hd[2] = P.exportBase + (P.hullChunkBase + idx) * P.exportStride;
          hd[3] = std::min(nfx, P.exportStride / 3);
          hd[7] = fbits(r.hullVol);
          hd[8] = hd[9] = hd[10] = hd[11] = NONE;
          hd[13] = 2;
        }
      }
    }
  }

  // ---- record: shaders.ts:1519-1544 ----
  void record(const Params& P) {
    for (uint32_t g = 0; g < P.nJobs; g++) {
      uint32_t* it = item(P.itemsOutBase + g);
      if (it[16] != 1) continue;
      float costs[8];
      bool bad = false;
      uint32_t np = it[8];
      for (uint32_t i = 0; i < np; i++) {
        uint32_t* pd = part(it[i]);
        float hv = bitsf(pd[7]);
        if (hv < 0.0f || (pd[13] & 4) != 0) bad = true;
        costs[i] = rv_cost(bitsf(pd[6]), hv);
      }
      if (bad) { it[16] = 0; continue; }
      for (uint32_t i = 1; i < np; i++) {
        float kc = costs[i];
        uint32_t kp = it[i];
        uint32_t j = i;
        while (j > 0 && costs[j - 1] > kc) { costs[j] = costs[j - 1]; it[j] = it[j - 1]; j--; }
        costs[j] = kc; it[j] = kp;
      }
      if (it[11] < 4) { it[12 + it[11]] = fbits(costs[np - 1]); it[11]++; }
    }
  }

  // ---- evaluate: shaders.ts:1404-1517 ----
  uint32_t u4(uint32_t i, int c) { uint32_t w[4]; std::memcpy(w, &planes[i], 16); return w[c]; }
  void evaluate(const Params& P, uint32_t mode, uint32_t stateBase, uint32_t headerOff) {
    uint32_t sb = stateBase, hb = sb + headerOff;
    uint32_t depth = u4(hb, 0), w0t = u4(hb, 2), nProbes = u4(hb, 3);
    for (uint32_t s = 0; s < P.nSeeds; s++) {
      float bestC = 1e30f;
      uint32_t bestCut = NONE;
      for (uint32_t l = 0; l < depth; l++) {
        uint32_t lOut = u4(hb + 1 + l, 0), lJobs = u4(hb + 1 + l, 1);
        uint32_t perSeed = lJobs / P.nSeeds;
        uint32_t wantFlag = l == depth - 1 ? 1 : 2;
        for (uint32_t i = 0; i < perSeed; i++) {
          uint32_t* it = item(lOut + s * perSeed + i);
          if (it[16] != wantFlag || it[11] == 0 || it[10] == NONE) continue;
          float sum = 0.0f;
          for (uint32_t k = 0; k < it[11]; k++) sum += bitsf(it[12 + k]);
          float c = sum / (float)it[11];
          if (c < bestC || (c == bestC && it[10] < bestCut)) { bestC = c; bestCut = it[10]; }
        }
      }
      if (bestCut == NONE) {
        uint32_t lOut = u4(hb + 1, 0), lJobs = u4(hb + 1, 1);
        uint32_t perSeed = lJobs / P.nSeeds;
        bestC = 1e30f;
        for (uint32_t i = 0; i < perSeed; i++) {
          uint32_t* it = item(lOut + s * perSeed + i);
          if (it[16] == 1 && it[11] >= 1 && it[10] != NONE) {
            float c = bitsf(it[12]);
            if (c < bestC || (c == bestC && it[10] < bestCut)) { bestC = c; bestCut = it[10]; }
          }
        }
      }
      uint32_t cut = bestCut;
      float cost = bestC;
      uint32_t st = sb + 16 + 4 * s;
      f4 plane = planes[st];
      f4 s1 = planes[st + 1];
      float half = s1.y;
      bool valid = (fbits(s1.w) & 1) != 0;
      if (mode == 0) {
        valid = cut != NONE;
        if (valid) plane = planes[P.jobBase + s * w0t + cut];
        s1 = f4{valid ? cost : 1e30f, half, bitsf(cut), bitsf(valid ? 1u : 0u)};
        half = planes[st + 2].x;
      } else {
        if (cut != NONE && cost < s1.x - 1e-7f) {
          plane = planes[P.jobBase + s * w0t + cut];
          s1 = f4{cost, s1.y, bitsf(cut), s1.w};
        }
        half = nProbes > 1 ? 2.0f * half / (float)(nProbes - 1) : 0.0f;
      }
      s1.y = half;
      planes[st] = plane;
      planes[st + 1] = s1;
      for (uint32_t i = 0; i < nProbes; i++) {
        f4 pp{0, 0, 0, 0};
        if (valid && half > 0.0f && nProbes > 1) {
          float off = half * ((2.0f * (float)i) / (float)(nProbes - 1) - 1.0f);
          pp = f4{plane.x, plane.y, plane.z, plane.w - off};
        }
        planes[P.edgePlaneBase + s * P.edgeStride + i] = pp;
      }
    }
  }

  struct Level {
    uint32_t itemsInBase, nItemsIn, itemsOutBase, jobBase, partBase, nJobs, width, nEdgeCuts, totalWidth;
  };
  std::vector<Level> layout(uint32_t nSeeds, uint32_t depth, uint32_t w0, uint32_t ne0) {
    std::vector<Level> lv;
    uint32_t itemsInBase = 0, nItemsIn = nSeeds, itemsOutBase = nSeeds, jobBase = 0;
    for (uint32_t l = 0; l < depth; l++) {
      uint32_t width = l == 0 ? w0 : (uint32_t)cfg.width2;
      uint32_t nEdge = l == 0 ? ne0 : 0;
      uint32_t tw = width + nEdge;
      uint32_t nJobs = nItemsIn * tw;
      lv.push_back(Level{itemsInBase, nItemsIn, itemsOutBase, jobBase, nSeeds + 2 * jobBase, nJobs, width, nEdge, tw});
      itemsInBase = itemsOutBase;
      nItemsIn = nJobs;
      itemsOutBase += nJobs;
      jobBase += nJobs;
    }
    return lv;
  }

  // ---- GpuTree.run: tree.ts:449-661 ----
  void run(const orc_mesh* seeds, uint32_t nSeeds, const float* edgePlanes, uint32_t planesPerSeed,
           const orc_run_opts& opt, orc_seed* out, orc_stats* stats) {
    uint32_t depth = opt.depth > 0 ? (uint32_t)opt.depth : (uint32_t)cfg.depth;
    uint32_t width0 = opt.width >= 0 ? (uint32_t)opt.width : (uint32_t)cfg.width;
    uint32_t nEdge0 = std::min<uint32_t>(opt.nEdgeCuts >= 0 ? (uint32_t)opt.nEdgeCuts : edgeStride, edgeStride);
    if (width0 % 3 != 0 || width0 > (uint32_t)cfg.width) throw std::runtime_error("width override must be a multiple of 3 and <= configured width");
    if (depth < 1 || depth > (uint32_t)cfg.depth) throw std::runtime_error("depth out of range for this tree");
    std::memset(stats, 0, sizeof(*stats));
    if (nSeeds == 0) return;
    bool refine = opt.refineRounds > 0 && opt.refineProbes >= 3;
    uint32_t nProbes = refine ? std::min<uint32_t>((uint32_t)opt.refineProbes, edgeStride) : 0;
    ensureTables(nSeeds);
    uint32_t slabWords = hullSlabWords(seeds, nSeeds);
    lastHullSlabWords = slabWords;
    uint32_t vTop, tTop;
    uploadSeeds(seeds, nSeeds, vTop, tTop);
    std::vector<Level> tree = layout(nSeeds, depth, width0, nEdge0);
    std::vector<Level> probe;
    if (refine) probe = layout(nSeeds, depth, 0, nProbes);
    uint32_t edgePlaneBase = capJobs;
    uint32_t stateBase = edgePlaneBase + capSeeds * edgeStride;
    for (uint32_t k = 0; k < nSeeds; k++) {
      for (uint32_t i = 0; i < edgeStride; i++) {
        f4 p{0, 0, 0, 0};
        if (edgePlanes && i < planesPerSeed) std::memcpy(&p, edgePlanes + 4 * ((size_t)k * planesPerSeed + i), 16);
        planes[edgePlaneBase + k * edgeStride + i] = p;
      }
    }
    // evaluate state: two level-layout headers, then 4 vec4 per seed
    for (uint32_t i = 0; i < 16 + 4 * nSeeds; i++) planes[stateBase + i] = f4{0, 0, 0, 0};
    auto writeHeader = [&](uint32_t at, const std::vector<Level>& L) {
      uint32_t w[4] = {depth, nSeeds, L[0].totalWidth, nProbes};
      std::memcpy(&planes[stateBase + at], w, 16);
      for (size_t l = 0; l < L.size(); l++) {
        uint32_t h[4] = {L[l].itemsOutBase, L[l].nJobs, 0, 0};
        std::memcpy(&planes[stateBase + at + 1 + l], h, 16);
      }
    };
    writeHeader(0, tree);
    if (refine) writeHeader(5, probe);
    for (uint32_t k = 0; k < nSeeds; k++) planes[stateBase + 16 + 4 * k + 2].x = refine && opt.refineSpacing ? opt.refineSpacing[k] : 0.0f;
    validJobs = 0;
    auto runStage = [&](const std::vector<Level>& L, uint32_t mode, uint32_t headerOff) {
      for (uint32_t l = 0; l < L.size(); l++) {
        const Level& v = L[l];
        Params P;
        P.itemsInBase = v.itemsInBase; P.nItemsIn = v.nItemsIn; P.itemsOutBase = v.itemsOutBase; P.jobBase = v.jobBase;
        P.width = v.width; P.nEdgeCuts = v.nEdgeCuts; P.edgeStride = edgeStride; P.totalWidth = v.totalWidth;
        P.minEdgeDist = cfg.minEdgeDist; P.level = l; P.totalLevels = depth; P.partBase = v.partBase;
        P.edgePlaneBase = edgePlaneBase; P.hullSlabWords = slabWords; P.nChildParts = 2 * v.nJobs; P.nJobs = v.nJobs;
        P.lastLevel = l == depth - 1; P.nSeeds = cfg.pruneLastLevel ? nSeeds : 0;
        plan(P); scan(P); emit(P); hull(P); record(P);
      }
      Params E;
      E.jobBase = L[0].jobBase; E.width = L[0].width; E.nEdgeCuts = L[0].nEdgeCuts; E.totalWidth = L[0].totalWidth;
      E.edgeStride = edgeStride; E.edgePlaneBase = edgePlaneBase; E.nSeeds = nSeeds;
      evaluate(E, mode, stateBase, headerOff);
    };
    runStage(tree, 0, 0);
    if (refine) {
      for (int r = 0; r < opt.refineRounds; r++) {
        ctr[0] = vTop; ctr[1] = tTop; ctr[2] = 0; ctr[3] = 0;
        runStage(probe, 1, 5);
      }
    }
    const std::vector<Level>& last = refine ? probe : tree;
    lastItems = last.back().itemsOutBase + last.back().nJobs;
    for (uint32_t k = 0; k < nSeeds; k++) {
      uint32_t o = stateBase + 16 + 4 * k;
      bool valid = (fbits(planes[o + 1].w) & 1) != 0;
      out[k].valid = valid ? 1 : 0;
      out[k].bestCut = valid ? (int32_t)fbits(planes[o + 1].z) : -1;
      out[k].bestCost = valid ? planes[o + 1].x : INFINITY;
      f4 p = planes[o];
      out[k].plane[0] = valid ? p.x : 0; out[k].plane[1] = valid ? p.y : 0;
      out[k].plane[2] = valid ? p.z : 0; out[k].plane[3] = valid ? p.w : 0;
    }
    stats->overflow = ctr[4] != 0; stats->hullFail = ctr[5] != 0; stats->hullFailCount = ctr[5];
    stats->npOverflow = ctr[6] != 0; stats->pruned = ctr[7];
    stats->nLevels = (uint32_t)tree.size();
    for (size_t l = 0; l < tree.size(); l++) stats->jobsPerLevel[l] = tree[l].nJobs;
    stats->validJobs = validJobs;
    stats->hullSlabWords = slabWords;
  }

  // ---- GpuTree.hullMeshes: tree.ts:382-443 ----
  void hullMeshes(const orc_mesh* m, uint32_t n, int hullStage, int noExport, uint32_t* trisOut,
                  uint32_t exportStrideOut, float* volOut, uint32_t* ntOut, int32_t* status) {
    ensureTables(1);
    ensurePartSlots(n);
    uint32_t vTop, tTop;
    uploadSeeds(m, n, vTop, tTop);
    uint32_t slabWords = hullSlabWords(m, n);
    uint32_t maxNv = 0;
    for (uint32_t k = 0; k < n; k++) maxNv = std::max(maxNv, m[k].nv);
    uint32_t exportStride = noExport ? 0 : 3 * 2 * std::min<uint32_t>((uint32_t)cfg.hullMaxVerts, maxNv);
    if ((uint64_t)tTop + (uint64_t)n * exportStride > cfg.triCap) throw std::runtime_error("hull export exceeds triangle pool");
    Params P;
    P.itemsInBase = 0; P.nItemsIn = n; P.itemsOutBase = n; P.totalLevels = 1; P.edgePlaneBase = capJobs;
    P.hullSlabWords = slabWords; P.nChildParts = n; P.nJobs = 0; P.exportBase = tTop; P.exportStride = exportStride;
    P.hullStage = (uint32_t)hullStage;
    hull(P);
    for (uint32_t k = 0; k < n; k++) {
      uint32_t* pd = part(k);
      float vol = bitsf(pd[7]);
      uint32_t nf = pd[14];
      bool ok = !(vol < 0.0f || nf < 4);
      status[k] = ok ? 0 : (vol < 0.0f ? (int32_t)((pd[13] & 3) ? (pd[13] & 3) : 9) : 8);
      volOut[k] = vol;
      ntOut[k] = ok ? nf : 0;
      if (ok && trisOut && exportStride) {
        uint32_t cpy = std::min(3 * nf, exportStrideOut);
        std::memcpy(trisOut + (size_t)k * exportStrideOut, &pool[tBase + tTop + (size_t)k * exportStride], 4ull * cpy);
      }
    }
  }
};

}  // namespace orc

// ------------------------------------------------------------------------
// C API for the test harness (ctypes)
// ------------------------------------------------------------------------
using orc::Tree;

static thread_local std::string g_err;

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

void* orc_tree_create(const orc_config* c) {
  try { return new Tree(*c); } catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_tree_destroy(void* h) { delete (Tree*)h; }
int orc_plane_slots(void* h) { return (int)((Tree*)h)->edgeStride; }

int orc_tree_run(void* h, const orc_mesh* seeds, int nSeeds, const float* edgePlanes, int planesPerSeed,
                 const orc_run_opts* opts, orc_seed* out, orc_stats* stats) {
  try {
    ((Tree*)h)->run(seeds, (uint32_t)nSeeds, edgePlanes, (uint32_t)planesPerSeed, *opts, out, stats);
    return 0;
  } catch (std::exception& e) { g_err = e.what(); return -1; }
}

int orc_tree_hull_meshes(void* h, const orc_mesh* m, int n, int hullStage, int noExport, uint32_t* trisOut,
                         uint32_t exportStride, float* volOut, uint32_t* ntOut, int32_t* status) {
  try {
    ((Tree*)h)->hullMeshes(m, (uint32_t)n, hullStage, noExport, trisOut, exportStride, volOut, ntOut, status);
    return 0;
  } catch (std::exception& e) { g_err = e.what(); return -1; }
}

// Table readers: items (20 words), parts (16 words), jobs (24 words)
int orc_read_items(void* h, uint32_t first, uint32_t n, uint32_t* out) {
  Tree* t = (Tree*)h;
  if ((uint64_t)first + n > t->capItems) return -1;
  std::memcpy(out, t->item(first), 80ull * n);
  return 0;
}
int orc_read_parts(void* h, uint32_t first, uint32_t n, uint32_t* out) {
  Tree* t = (Tree*)h;
  if ((uint64_t)first + n > t->capParts) return -1;
  std::memcpy(out, t->part(first), 64ull * n);
  return 0;
}
int orc_read_jobs(void* h, uint32_t first, uint32_t n, uint32_t* out) {
  Tree* t = (Tree*)h;
  if ((uint64_t)first + n > std::max<uint32_t>(t->capJobs, 1)) return -1;
  std::memcpy(out, t->job(first), 96ull * n);
  return 0;
}
// Geometry of one part: verts (nv*3 floats), tris (nt*3), edges (ne*8 words)
int orc_read_part_geometry(void* h, uint32_t partIdx, float* verts, uint32_t* tris, uint32_t* edges) {
  Tree* t = (Tree*)h;
  if (partIdx >= t->capParts) return -1;
  uint32_t* pd = t->part(partIdx);
  if (verts) std::memcpy(verts, &t->pool[t->vBase + pd[0]], 12ull * pd[1]);
  if (tris) std::memcpy(tris, &t->pool[t->tBase + pd[2]], 12ull * pd[3]);
  if (edges) std::memcpy(edges, &t->pool[t->eBase + 8ull * pd[4]], 32ull * pd[5]);
  return 0;
}
int orc_read_plane(void* h, uint32_t idx, float* out4) {
  Tree* t = (Tree*)h;
  if (idx >= t->planes.size()) return -1;
  std::memcpy(out4, &t->planes[idx], 16);
  return 0;
}
uint32_t orc_last_items(void* h) { return ((Tree*)h)->lastItems; }

}  // extern "C"
