// cut_kernels.cu — the capped plane cut of the decomposition loop
// (src/cpu/cut.ts:33-315) on the GPU, for a batch of (mesh, plane) cuts.
//
// The result of every cut is bit for bit the host cut's (csrc/plane_cut.cpp):
// the same half meshes, vertices in the same order (numbered by first use in
// each half's triangle list), the same triangles in the same order, the same
// cap triangulation and the same failures. The steps:
//
//   classify   one thread per vertex: signed distance in double, the
//              three-state side (on the plane within 1e-6), whether the
//              plane splits the mesh at all;
//   count      one thread per triangle: how many triangles each half gets
//              (Sutherland-Hodgman on one triangle gives at most a quad) and
//              whether a half's triangles there can hold a cap boundary edge
//              (two vertices on the plane); a device-wide scan turns the
//              counts into each triangle's output positions;
//   surface    one thread per triangle: writes the halves' surface
//              triangles in input order, intersection vertices shared per
//              edge through a hash table keyed on the edge (its coordinates
//              depend only on the edge's lower and higher vertex);
//   cap        one warp per (cut, half): the half's boundary edges in
//              first-seen order, their loops, the loops' classification
//              (outer or hole by signed area, parent by the hole centroid's
//              crossing number) and the caps (ear clipping with holes
//              bridged in, or centroid fans). Steps whose decisions read
//              what earlier iterations wrote (grouping the boundary edges,
//              walking the loops) run on lane 0 while the other lanes wait;
//              sorting and bridging the holes run on every lane with the
//              same data (identical stores) with a warp sync after each
//              step, so no lane writes what another has yet to read;
//              the loops' areas and classification, the edge gathering and
//              the twin search split their work over the lanes, and the ear
//              clipper tests the orientation of the next 32 ring vertices
//              at once (one per lane) and the full ear test only on the
//              survivors, looking at the nodes in the cells of a uniform
//              grid that the ear's bounding box covers. Every loop over a
//              list or ring is bounded by its length;
//   compact    one thread per triangle corner: first use of every vertex
//              (atomicMin), a scan of the first uses numbers the vertices,
//              then the halves are written to the output pools.
//
// The host computes the per-cut constants that involve library functions
// (the normal's length and the cap basis, both from std::hypot), so the
// device only adds, multiplies, divides and compares doubles; this unit
// compiles with --fmad=false and the host cut without contraction, so both
// round every operation the same way.
//
// Boundary edges are looked for among edges with both ends on the plane:
// for a closed input mesh every boundary edge of a half lies there (an edge
// with an end off the plane keeps its reverse in the same half).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "cut_engine.h"
#include "dev_ptr.h"
#include "dev_scan.cuh"

#define CUT_FULL 0xffffffffu
#define CUT_NONE 0xffffffffu

namespace cuacd {
int set_error(int code, const char* msg);

namespace cut {

// ---------------------------------------------------------------------------
// records

struct CutDesc {
  double n[3], d;         // unit normal and offset of the plane
  double u[3], w[3];      // orthonormal basis of the plane for the caps
  uint32_t vOff, nv;      // input mesh: first vertex and count in the vertex pool
  uint32_t tOff, nt;      // first triangle and count in the triangle pool
  uint32_t vBase, tBase;  // this cut's range in the per-vertex / per-triangle scratch
  uint32_t pad[2];
};
static_assert(sizeof(CutDesc) == 112, "CutDesc layout");

// written by the count step
struct CutSizes {
  uint32_t anyPos, anyNeg, straddle, pad;
  uint32_t surf[2];  // surface triangles of each half
  uint32_t cand[2];  // input triangles whose half triangles may hold a boundary edge
};

// set by the host from the sizes
struct CutLayout {
  uint32_t hashOff, hashSize;      // intersection hash (keys, coordinates)
  uint32_t surfOff[2], surfCnt[2];  // surface triangles (vertex ids before compaction)
  uint32_t candOff[2], candCnt[2];  // candidate entries (first half triangle, count)
  uint32_t preOff[2];              // first-use array over the half's vertex ids
  uint32_t capMax[2];              // cap triangles the cap scratch holds
  uint32_t capWord[2], capDbl[2];  // the cap step's scratch in the word and double arenas
  uint32_t mEdge[2];               // bound on the half's plane edges (6 per candidate)
  uint32_t active, pad;
};

// written by the cap and compact steps
struct CutOut {
  int32_t fail[2];   // per half: 0 or a CUT_* failure
  uint32_t cap[2];   // cap triangles of each half
  uint32_t cent[2];  // centroid vertices of each half
  uint32_t nvOut[2];
};

enum { CUT_OK = 0, CUT_NO_SPLIT = 1, CUT_OPEN_CHAIN = 2, CUT_DEAD_END = 3, CUT_CYCLE = 4, CUT_SCRATCH = 5 };

constexpr double ON_PLANE_EPS = 1e-6;  // the host cut's default eps
// ear-clip nodes a cap warp keeps in shared memory (X, Y, their float
// hi/lo copies, index, links, alive flag, grid: 52 bytes each plus the cell
// starts)
constexpr uint32_t CAP_SM_NODES = 2048;
constexpr size_t CAP_SM_RING_BYTES = 16 * CAP_SM_NODES + 4 * 5 * CAP_SM_NODES + 4 * 2 * (CAP_SM_NODES / 2 + 2) +
                                     16 * CAP_SM_NODES;
// a larger ring keeps its links and ear-test memo (12 bytes a node) in
// shared memory up to CAP_SM_LINK_NODES nodes, its coordinates and grid in
// the global scratch: the ear search walks the links node by node, and on
// long degenerate rings that walk is most of the cap's time. One 32-thread
// block per SM fits either way.
constexpr uint32_t CAP_SM_LINK_NODES = 16384;
constexpr size_t CAP_SM_BYTES =
    CAP_SM_RING_BYTES > 12 * (size_t)CAP_SM_LINK_NODES ? CAP_SM_RING_BYTES : 12 * (size_t)CAP_SM_LINK_NODES;
// boundary edges whose walk runs in shared memory: a source hash of up to
// 2 * 2048 entries (key, head, tail) and next, used, source and destination
// per edge, 80 KB, within CAP_SM_BYTES
constexpr uint32_t CAP_SM_WALK_B = 2048;
static_assert(3 * 4 * 2 * CAP_SM_WALK_B + 4 * 4 * CAP_SM_WALK_B <= CAP_SM_BYTES, "walk fits the cap shared memory");
constexpr unsigned long long EMPTY_KEY = ~0ull;

// the cap step's scratch of one half, carved from m = its plane-edge bound
struct CapCarve {
  uint32_t eA, eB;          // plane edges (m each)
  uint32_t eh, ehKey, ehVal;  // edge hash: entries, keys (2 words each), first index
  uint32_t bSrc, bDst, bNext, bUsed;  // boundary edges (m each)
  uint32_t sh, shKey, shHead, shTail;  // source-vertex hash
  uint32_t starts;          // source vertices in first-seen order (m)
  uint32_t loopV, loopS;    // loop vertices (m), loop starts (m + 1)
  uint32_t depth, parent;   // per loop (m)
  uint32_t nd;              // ear-clip node capacity (3 m + 4)
  uint32_t ndI, ndPrev, ndNext, ndAlive;
  uint32_t gId;             // a group's ring: vertex ids (m)
  uint32_t holeL;           // a group's holes: leftmost node (m)
  uint32_t gCnt, gStart, gNodes;  // the ear test's uniform grid: per-cell fill, starts, nodes (nd each)
  uint32_t ndXf, ndYf;      // the nodes' float32 coordinates (nd each)
  uint32_t ndXl, ndYl;      // and their float32 remainders (nd each)
  uint32_t capT;            // cap triangles, 3 words each (capMax)
  uint32_t words;
  uint32_t l2, area, ndX, ndY, gXY, holeX, cent;  // double arena
  uint32_t dbls;
};

__host__ __device__ inline uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 16;
  while (p < x) p <<= 1;
  return p;
}

__host__ __device__ inline CapCarve carve(uint32_t m, uint32_t capMax) {
  CapCarve c;
  uint32_t o = 0;
  c.eh = pow2_at_least(2 * m);
  c.ehKey = o; o += 2 * c.eh;  // first: 8-byte aligned keys
  c.ehVal = o; o += c.eh;
  c.eA = o; o += m;
  c.eB = o; o += m;
  c.bSrc = o; o += m;
  c.bDst = o; o += m;
  c.bNext = o; o += m;
  c.bUsed = o; o += m;
  c.sh = pow2_at_least(2 * m);
  c.shKey = o; o += c.sh;
  c.shHead = o; o += c.sh;
  c.shTail = o; o += c.sh;
  c.starts = o; o += m;
  c.loopV = o; o += m;
  c.loopS = o; o += m + 1;
  c.depth = o; o += m;
  c.parent = o; o += m;
  c.nd = 3 * m + 4;
  c.ndI = o; o += c.nd;
  c.ndPrev = o; o += c.nd;
  c.ndNext = o; o += c.nd;
  c.ndAlive = o; o += c.nd;
  c.gId = o; o += m;
  c.holeL = o; o += m;
  c.gCnt = o; o += c.nd + 1;
  c.gStart = o; o += c.nd + 1;
  c.gNodes = o; o += c.nd;
  c.ndXf = o; o += c.nd;
  c.ndYf = o; o += c.nd;
  c.ndXl = o; o += c.nd;
  c.ndYl = o; o += c.nd;
  c.capT = o; o += 3 * capMax;
  c.words = (o + 1) & ~1u;
  uint32_t d = 0;
  c.l2 = d; d += 2 * m;
  c.area = d; d += m;
  c.ndX = d; d += c.nd;
  c.ndY = d; d += c.nd;
  c.gXY = d; d += 2 * m;
  c.holeX = d; d += m;
  c.cent = d; d += 3 * m;
  c.dbls = d;
  return c;
}

// ---------------------------------------------------------------------------
// helpers

// the segment holding element g: the largest c with pre[c] <= g (pre has
// n + 1 entries, pre[0] = 0, pre[n] > g)
__device__ __forceinline__ uint32_t find_seg(const uint32_t* __restrict__ pre, uint32_t n, uint32_t g) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (pre[mid] <= g) lo = mid;
    else hi = mid;
  }
  return lo;
}

__host__ __device__ __forceinline__ uint32_t mix_key(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return (uint32_t)k;
}

__device__ __forceinline__ int side_of(double v) { return v > ON_PLANE_EPS ? 1 : (v < -ON_PLANE_EPS ? -1 : 0); }

// ---------------------------------------------------------------------------
// classify: signed distance and side of every vertex

__global__ void k_cut_classify(const CutDesc* __restrict__ D, const uint32_t* __restrict__ vPre, uint32_t n,
                               uint32_t totalV, const float* __restrict__ V, double* __restrict__ dist,
                               int8_t* __restrict__ sgn, CutSizes* __restrict__ S) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= totalV) return;
  const uint32_t c = find_seg(vPre, n, g);
  const CutDesc& d = D[c];
  const uint32_t i = g - d.vBase;
  const float* p = V + 3 * ((size_t)d.vOff + i);
  const double x = p[0], y = p[1], z = p[2];
  // n.x x + n.y y + n.z z + d, left to right (the host cut's order)
  double v = d.n[0] * x;
  v = v + d.n[1] * y;
  v = v + d.n[2] * z;
  v = v + d.d;
  const int s = side_of(v);
  dist[g] = v;
  sgn[g] = (int8_t)s;
  if (s > 0 && S[c].anyPos == 0) atomicOr(&S[c].anyPos, 1u);
  if (s < 0 && S[c].anyNeg == 0) atomicOr(&S[c].anyNeg, 1u);
}

// triangles a half gets from one triangle: Sutherland-Hodgman keeps the
// vertices on the kept side or on the plane and adds one vertex per edge
// that crosses the plane strictly; the polygon is fanned
__device__ __forceinline__ uint32_t clip_count(const int s[3], int keep) {
  int np = 0;
  for (int k = 0; k < 3; k++) {
    const int sp = s[k] * keep, sq = s[(k + 1) % 3] * keep;
    if (sp >= 0) np++;
    if (s[k] != 0 && s[(k + 1) % 3] != 0 && sp * sq < 0) np++;
  }
  return np > 2 ? (uint32_t)(np - 2) : 0u;
}

// per triangle: (positive half triangles, negative half triangles, positive
// candidate, negative candidate); a candidate is a triangle whose half
// triangles may hold a boundary edge: two vertices on the plane (a
// straddling triangle always, else one with two vertices of side 0) or an
// edge of the input without a reverse (`open`, a bit per edge)
__device__ __forceinline__ uint4 tri_counts(const int s[3], uint32_t open, bool* straddle) {
  const bool hasPos = s[0] > 0 || s[1] > 0 || s[2] > 0;
  const bool hasNeg = s[0] < 0 || s[1] < 0 || s[2] < 0;
  const int zeros = (s[0] == 0) + (s[1] == 0) + (s[2] == 0);
  *straddle = hasPos && hasNeg;
  const uint32_t cand = (zeros >= 2 || open != 0) ? 1u : 0u;
  if (!hasPos && !hasNeg) return make_uint4(0, 0, 0, 0);
  if (!hasNeg) return make_uint4(1, 0, cand, 0);
  if (!hasPos) return make_uint4(0, 1, 0, cand);
  const uint32_t p = clip_count(s, 1), q = clip_count(s, -1);
  return make_uint4(p, q, p > 0 ? 1 : 0, q > 0 ? 1 : 0);
}

__global__ void k_cut_count(const CutDesc* __restrict__ D, const uint32_t* __restrict__ tPre, uint32_t n,
                            uint32_t totalT, const uint32_t* __restrict__ T, const int8_t* __restrict__ sgn,
                            const uint8_t* __restrict__ openBits, uint4* __restrict__ cnt, CutSizes* __restrict__ S) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= totalT) return;
  const uint32_t c = find_seg(tPre, n, g);
  const CutDesc& d = D[c];
  const uint32_t t = g - d.tBase;
  const uint32_t* tri = T + 3 * ((size_t)d.tOff + t);
  const int s[3] = {sgn[d.vBase + tri[0]], sgn[d.vBase + tri[1]], sgn[d.vBase + tri[2]]};
  bool straddle;
  cnt[g] = tri_counts(s, openBits ? openBits[d.tOff + t] : 0u, &straddle);
  if (straddle) atomicAdd(&S[c].straddle, 1u);
}

__global__ void k_cut_sizes(const CutDesc* __restrict__ D, uint32_t n, const uint4* __restrict__ pre,
                            CutSizes* __restrict__ S) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const uint4 a = pre[D[c].tBase], b = pre[D[c].tBase + D[c].nt];
  S[c].surf[0] = b.x - a.x;
  S[c].surf[1] = b.y - a.y;
  S[c].cand[0] = b.z - a.z;
  S[c].cand[1] = b.w - a.w;
}

// ---------------------------------------------------------------------------
// surface: the halves' triangles in input order

// the intersection vertex of edge (lo, hi): its slot in the cut's hash;
// coordinates p + t (q - p), t = dist[lo] / (dist[lo] - dist[hi])
__device__ uint32_t isect_slot(unsigned long long* __restrict__ keys, double* __restrict__ xyz, uint32_t hashOff,
                               uint32_t hashSize, uint32_t lo, uint32_t hi, const double* __restrict__ dist,
                               const float* __restrict__ V, uint32_t vBase, uint32_t vOff) {
  const unsigned long long key = ((unsigned long long)lo << 32) | hi;
  uint32_t h = mix_key(key) & (hashSize - 1);
  for (uint32_t probe = 0; probe < hashSize; probe++, h = (h + 1) & (hashSize - 1)) {
    const unsigned long long old = atomicCAS(keys + hashOff + h, EMPTY_KEY, key);
    if (old == EMPTY_KEY) {
      const double dl = dist[vBase + lo], dh = dist[vBase + hi];
      const double t = dl / (dl - dh);
      const float* P = V + 3 * ((size_t)vOff + lo);
      const float* Q = V + 3 * ((size_t)vOff + hi);
      double* o = xyz + 3 * ((size_t)hashOff + h);
      for (int a = 0; a < 3; a++) {
        const double pa = P[a], qa = Q[a];
        o[a] = pa + t * (qa - pa);
      }
      return h;
    }
    if (old == key) return h;
  }
  return CUT_NONE;
}

__global__ void k_cut_surface(const CutDesc* __restrict__ D, const CutLayout* __restrict__ L,
                              const uint32_t* __restrict__ tPre, uint32_t n, uint32_t totalT,
                              const uint32_t* __restrict__ T, const float* __restrict__ V,
                              const double* __restrict__ dist, const int8_t* __restrict__ sgn,
                              const uint4* __restrict__ pre, unsigned long long* __restrict__ hashKeys,
                              double* __restrict__ hashXYZ, uint32_t* __restrict__ surfT, uint2* __restrict__ candE,
                              const uint8_t* __restrict__ openBits, CutOut* __restrict__ O) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= totalT) return;
  const uint32_t c = find_seg(tPre, n, g);
  const CutLayout& l = L[c];
  if (!l.active) return;
  const CutDesc& d = D[c];
  const uint32_t* tri = T + 3 * ((size_t)d.tOff + (g - d.tBase));
  const uint32_t ids[3] = {tri[0], tri[1], tri[2]};
  const int s[3] = {sgn[d.vBase + ids[0]], sgn[d.vBase + ids[1]], sgn[d.vBase + ids[2]]};
  bool straddle;
  const uint32_t t = g - d.tBase;
  const uint4 cn = tri_counts(s, openBits ? openBits[d.tOff + t] : 0u, &straddle);
  if (cn.x + cn.y == 0) return;
  // candidate entry: first half triangle, and count | input triangle << 2
  const uint32_t tagT = t << 2;
  const uint4 P = scan::vsub(pre[g], pre[d.tBase]);  // this triangle's positions within the cut
  if (!straddle) {
    const int side = cn.x ? 0 : 1;
    const uint32_t at = side == 0 ? P.x : P.y;
    uint32_t* o = surfT + 3 * ((size_t)l.surfOff[side] + at);
    o[0] = ids[0]; o[1] = ids[1]; o[2] = ids[2];
    if (side == 0 && cn.z) candE[l.candOff[0] + P.z] = make_uint2(at, 1u | tagT);
    if (side == 1 && cn.w) candE[l.candOff[1] + P.w] = make_uint2(at, 1u | tagT);
    return;
  }
  uint32_t ix[3] = {CUT_NONE, CUT_NONE, CUT_NONE};
  for (int k = 0; k < 3; k++) {
    const int k1 = (k + 1) % 3;
    if (s[k] != 0 && s[k1] != 0 && s[k] * s[k1] < 0) {
      const uint32_t lo = min(ids[k], ids[k1]), hi = max(ids[k], ids[k1]);
      const uint32_t h = isect_slot(hashKeys, hashXYZ, l.hashOff, l.hashSize, lo, hi, dist, V, d.vBase, d.vOff);
      if (h == CUT_NONE) {
        O[c].fail[0] = CUT_SCRATCH;
        return;
      }
      ix[k] = d.nv + h;
    }
  }
  for (int side = 0; side < 2; side++) {
    const int keep = side == 0 ? 1 : -1;
    uint32_t poly[4];
    int np = 0;
    for (int k = 0; k < 3; k++) {
      const int sp = s[k] * keep;
      if (sp >= 0) poly[np++] = ids[k];
      if (ix[k] != CUT_NONE) poly[np++] = ix[k];
    }
    const uint32_t at = side == 0 ? P.x : P.y;
    uint32_t* o = surfT + 3 * ((size_t)l.surfOff[side] + at);
    for (int k = 1; k + 1 < np; k++) {
      o[3 * (k - 1)] = poly[0];
      o[3 * (k - 1) + 1] = poly[k];
      o[3 * (k - 1) + 2] = poly[k + 1];
    }
    if (np > 2) candE[l.candOff[side] + (side == 0 ? P.z : P.w)] = make_uint2(at, (uint32_t)(np - 2) | tagT);
  }
}

// ---------------------------------------------------------------------------
// cap: one warp per (cut, half)

struct CapCtx {
  const CutDesc* d;
  uint32_t hashSize, hashOff, nv;
  const double* hashXYZ;
  const float* V;
  // a vertex's coordinates before compaction (an input vertex or an
  // intersection; centroids are never looked up here)
  __device__ void pos(uint32_t q, double& x, double& y, double& z) const {
    if (q < nv) {
      const float* p = V + 3 * ((size_t)d->vOff + q);
      x = p[0];
      y = p[1];
      z = p[2];
    } else {
      const double* p = hashXYZ + 3 * ((size_t)hashOff + (q - nv));
      x = p[0];
      y = p[1];
      z = p[2];
    }
  }
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ double orient2(double ax, double ay, double bx, double by, double cx, double cy) {
  return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

__device__ __forceinline__ int dsgn(double x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); }

// hash of 64-bit keys in the word arena: slot of key, inserting it when
// `insert` (atomic, for the lanes' parallel inserts); CUT_NONE when absent
__device__ uint32_t kh_find(unsigned long long* keys, uint32_t size, unsigned long long key, bool insert) {
  uint32_t h = mix_key(key) & (size - 1);
  for (uint32_t probe = 0; probe < size; probe++, h = (h + 1) & (size - 1)) {
    unsigned long long k = keys[h];
    if (k == key) return h;
    if (k == EMPTY_KEY) {
      if (!insert) return CUT_NONE;
      const unsigned long long old = atomicCAS(keys + h, EMPTY_KEY, key);
      if (old == EMPTY_KEY || old == key) return h;
    }
  }
  return CUT_NONE;
}

// open-addressing hash of 32-bit keys for one lane (the caller's lane 0)
__device__ uint32_t uh_find(uint32_t* keys, uint32_t size, uint32_t key, bool insert, bool* inserted) {
  uint32_t h = mix_key(key) & (size - 1);
  *inserted = false;
  for (uint32_t probe = 0; probe < size; probe++, h = (h + 1) & (size - 1)) {
    const uint32_t k = keys[h];
    if (k == key) return h;
    if (k == CUT_NONE) {
      if (!insert) return CUT_NONE;
      keys[h] = key;
      *inserted = true;
      return h;
    }
  }
  return CUT_NONE;
}

struct Ring {  // ear-clip node arrays of one half (warp-uniform)
  uint32_t *I, *prev, *next, *alive;
  double *X, *Y;
  float *Xf, *Yf;  // the coordinates rounded to float32 (the ear test's prefilter)
  float *Xl, *Yl;  // and the float32 rounding of what that rounding left out
  uint32_t n, cap;
  // uniform grid over the nodes (built once the holes are bridged in), in
  // the float32 coordinates: the ear test looks only at the nodes in the
  // cells its triangle's bounding box covers (rounding is monotonic, so a
  // node inside the box falls in a covered cell), and whether any node lies
  // in the triangle does not depend on the order it looks in
  uint32_t *gCnt, *gStart, *gNodes;
  uint32_t gnx, gny;
  float gx0, gy0, ginvx, ginvy;
  __device__ uint32_t cell_x(float x) const {
    const float f = (x - gx0) * ginvx;
    return f <= 0.0f ? 0u : min(gnx - 1, (uint32_t)f);
  }
  __device__ uint32_t cell_y(float y) const {
    const float f = (y - gy0) * ginvy;
    return f <= 0.0f ? 0u : min(gny - 1, (uint32_t)f);
  }
  __device__ void bridge(uint32_t a, uint32_t b) {
    const uint32_t a2 = n++;
    I[a2] = I[a]; X[a2] = X[a]; Y[a2] = Y[a]; Xf[a2] = Xf[a]; Yf[a2] = Yf[a]; Xl[a2] = Xl[a]; Yl[a2] = Yl[a];
    alive[a2] = 1;
    const uint32_t b2 = n++;
    I[b2] = I[b]; X[b2] = X[b]; Y[b2] = Y[b]; Xf[b2] = Xf[b]; Yf[b2] = Yf[b]; Xl[b2] = Xl[b]; Yl[b2] = Yl[b];
    alive[b2] = 1;
    const uint32_t an = next[a], bp = prev[b];
    next[a] = b;
    prev[b] = a;
    next[a2] = an;
    prev[an] = a2;
    next[b2] = a2;
    prev[a2] = b2;
    next[bp] = b2;
    prev[b2] = bp;
  }
  __device__ bool reflex(uint32_t k) const {
    return orient2(X[prev[k]], Y[prev[k]], X[k], Y[k], X[next[k]], Y[next[k]]) < 0;
  }
};

// ring vertices [s, e) of the group as nodes P.n .. P.n + (e - s) - 1,
// counter-clockwise (ccw) or clockwise, as the host clipper's ring() adds
// them (nodes in creation order, each linked after the previous): the
// signed area's terms in parallel and their sum in order, then every node at
// once; returns the last node
__device__ uint32_t ring_par(Ring& P, const double* gxy, uint32_t s, uint32_t e, bool ccw, int lane) {
  const uint32_t base = P.n, len = e - s;
  double* terms = P.X + base;  // scratch until the nodes are written
  for (uint32_t i = lane; i < len; i += 32) {
    const uint32_t k = s + i, j = k + 1 < e ? k + 1 : s;
    terms[i] = gxy[2 * k] * gxy[2 * j + 1] - gxy[2 * j] * gxy[2 * k + 1];
  }
  __syncwarp();
  double a = 0;
  for (uint32_t i = 0; i < len; i++) a += terms[i];
  __syncwarp();
  const bool fwd = (a > 0) == ccw;
  for (uint32_t i = lane; i < len; i += 32) {
    const uint32_t k = fwd ? s + i : e - 1 - i, nd = base + i;
    P.I[nd] = k;
    P.X[nd] = gxy[2 * k];
    P.Y[nd] = gxy[2 * k + 1];
    const float hx = (float)gxy[2 * k], hy = (float)gxy[2 * k + 1];
    P.Xf[nd] = hx;
    P.Yf[nd] = hy;
    P.Xl[nd] = (float)(gxy[2 * k] - (double)hx);  // exact in double (Sterbenz)
    P.Yl[nd] = (float)(gxy[2 * k + 1] - (double)hy);
    P.alive[nd] = 1;
    P.next[nd] = base + (i + 1 == len ? 0 : i + 1);
    P.prev[nd] = base + (i == 0 ? len - 1 : i - 1);
  }
  __syncwarp();
  P.n = base + len;
  return base + len - 1;
}

// an outer vertex visible from hole vertex h (leftmost of its loop), as the
// host clipper's find_bridge: the nearest crossing of the leftward ray with
// a downward edge of the counter-clockwise outer loop, its endpoint of larger
// x, replaced by the reflex vertex of smallest angle inside the triangle.
// The host walks the ring once for each; here lane 0 lists the ring in order
// from `outer` (order[i], and i in pos[] of each node) and the lanes split
// the edges and nodes by ring position. The host keeps the first crossing in
// ring order among those of largest x (a later one must be strictly larger)
// and the first candidate in ring order from m among those of smallest
// tangent, then largest x (the same strict tests), so each lane keeps its
// own first best and the warp takes the best of the lanes' with the lowest
// ring position. Every value is the host's double expression on the same
// operands. order and pos are scratch (the grid's node list and the alive
// words, both rebuilt before the ear clipping).
__device__ int32_t find_bridge(const Ring& P, uint32_t h, uint32_t outer, uint32_t* order, uint32_t* pos,
                               int lane) {
  uint32_t len = 0;
  if (lane == 0) {
    uint32_t p = outer;
    do {
      if (len >= P.n) {  // more steps than nodes: not a ring
        len = P.n + 1;
        break;
      }
      order[len] = p;
      pos[p] = len;
      len++;
      p = P.next[p];
    } while (p != outer);
  }
  len = __shfl_sync(CUT_FULL, len, 0);
  __syncwarp();
  if (len > P.n) return -1;  // not a ring: never for a well-formed group
  const double hx = P.X[h], hy = P.Y[h];
  // 1. the first crossing of largest x at most hx
  double bx1 = -INFINITY;
  uint32_t bi = CUT_NONE;
  for (uint32_t i = lane; i < len; i += 32) {
    const uint32_t p = order[i], an = P.next[p];
    const double ax = P.X[p], ay = P.Y[p], bx = P.X[an], by = P.Y[an];
    if (hy <= ay && hy >= by && by != ay) {
      const double x = ax + (hy - ay) * (bx - ax) / (by - ay);
      if (x <= hx && x > bx1) {
        bx1 = x;
        bi = i;
      }
    }
  }
  double qx = bx1;
  for (int d = 16; d > 0; d >>= 1) qx = fmax(qx, __shfl_xor_sync(CUT_FULL, qx, d));
  uint32_t first = (bi != CUT_NONE && bx1 == qx) ? bi : CUT_NONE;
  for (int d = 16; d > 0; d >>= 1) first = min(first, __shfl_xor_sync(CUT_FULL, first, d));
  if (first == CUT_NONE) return -1;
  int32_t m;
  {
    const uint32_t p = order[first], an = P.next[p];
    const double ax = P.X[p], ay = P.Y[p], bx = P.X[an], by = P.Y[an];
    if (qx == hx) {
      if (hy == ay) return (int32_t)p;
      if (hy == by) return (int32_t)an;
    }
    m = ax < bx ? (int32_t)an : (int32_t)p;
  }
  if (hx == qx) return m;
  // 2. from m once around: reflex nodes inside the triangle, smallest
  // tangent, then largest x, then first
  const double mx = P.X[m], my = P.Y[m];
  const uint32_t base = pos[m];
  double tBest = INFINITY, cBest = -INFINITY;
  uint32_t jBest = CUT_NONE;
  for (uint32_t j = lane; j < len; j += 32) {
    const uint32_t p = order[base + j < len ? base + j : base + j - len];
    const double cx = P.X[p], cy = P.Y[p];
    if (hx >= cx && cx >= mx && hx != cx) {
      const double d1 = orient2(hx, hy, qx, hy, cx, cy), d2 = orient2(qx, hy, mx, my, cx, cy),
                   d3 = orient2(mx, my, hx, hy, cx, cy);
      const bool inTri = (d1 >= 0 && d2 >= 0 && d3 >= 0) || (d1 <= 0 && d2 <= 0 && d3 <= 0);
      if (inTri && P.reflex(p)) {
        const double tn = fabs(hy - cy) / (hx - cx);
        if (tn < tBest || (tn == tBest && cx > cBest)) {
          tBest = tn;
          cBest = cx;
          jBest = j;
        }
      }
    }
  }
  for (int d = 16; d > 0; d >>= 1) {
    const double t2 = __shfl_xor_sync(CUT_FULL, tBest, d), c2 = __shfl_xor_sync(CUT_FULL, cBest, d);
    const uint32_t j2 = __shfl_xor_sync(CUT_FULL, jBest, d);
    if (t2 < tBest || (t2 == tBest && (c2 > cBest || (c2 == cBest && j2 < jBest)))) {
      tBest = t2;
      cBest = c2;
      jBest = j2;
    }
  }
  if (jBest != CUT_NONE) m = (int32_t)order[base + jBest < len ? base + jBest : base + jBest - len];
  return m;
}

// orient2 of three ring nodes, decided in float32 where the float value is
// clear of its error bound. Each coordinate x is kept as hi = fl(x) and lo =
// fl(x - hi); a difference b - a is (b.hi - a.hi) + (b.lo - a.lo) in float,
// within 2.01 u |b - a| + 6 u^2 S of the exact one (u = 2^-24, S the largest
// |coordinate|), so the float orient2 d1 d2 - d3 d4 is within 6.2 u (|d1 d2|
// + |d3 d4|) + 6.1 u^2 S (|d1| + |d2| + |d3| + |d4|) of the exact value, and
// the double orient2 within 4 2^-53 (|d1 d2| + |d3 d4|) of it. Beyond the sum
// of both (taken as 8 u (...) + 8 u^2 S (...)), the float value has the
// double result's sign; otherwise the double orient2 is computed.
// Returns +1, -1, or 0 for an exact double zero.
__device__ __forceinline__ float ring_diff(const float* h, const float* l, uint32_t b, uint32_t a) {
  return __fadd_rn(__fsub_rn(h[b], h[a]), __fsub_rn(l[b], l[a]));
}

// s + e = a + b exactly (Knuth's two-sum; no overflow in range)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bv = __fsub_rn(s, a), av = __fsub_rn(s, bv);
  e = __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}

// the difference of two ring coordinates as an unevaluated float pair
// (s, r): s + e = hi_b - hi_a exactly, r = fl(e + fl(lo_b - lo_a))
__device__ __forceinline__ void ring_diff2(const float* h, const float* l, uint32_t b, uint32_t a, float& s, float& r) {
  float e;
  two_sum(h[b], -h[a], s, e);
  r = __fadd_rn(e, __fsub_rn(l[b], l[a]));
}

// The second filter: orient2 in float-float arithmetic. With u = 2^-24 and
// S the largest |coordinate|: a coordinate is hi + lo within u^2 |x| (+
// 2^-149), a difference (s, r) is within 9 u^2 S (+ 2^-148) of the exact
// one, with |r| <= u |s| + 2.02 u S; a product is p + q + c with (p, q)
// the exact product s1 s2 (fma) and c = fl(fl(s1 r2 + r1 s2) + r1 r2),
// within 6 u^2 |s1 s2| + 6.1 u^2 S (|s1| + |s2|) + 25 u^3 S^2; the tail sum
// of the two products' low parts and the two-sum error of p1 - p2 adds 12
// u^2 (|p1| + |p2|) + 6.1 u^2 S sum|s|; the host's double orient2 is within
// 0.13 u^2 (|d1 d2| + |d3 d4|) of the exact value. So beyond E = 20 u^2
// (|p1| + |p2|) + 24 u^2 S sum|s| + 128 u^3 S^2 (+ 2^-140 (sum|s| + 1)) the
// float-float value has the double result's sign. Returns +1, -1, or 2
// when undecided.
__device__ int orient_ff(const Ring& P, uint32_t a, uint32_t b, uint32_t c, float S) {
  float s1, r1, s2, r2, s3, r3, s4, r4;
  ring_diff2(P.Xf, P.Xl, b, a, s1, r1);
  ring_diff2(P.Yf, P.Yl, c, a, s2, r2);
  ring_diff2(P.Yf, P.Yl, b, a, s3, r3);
  ring_diff2(P.Xf, P.Xl, c, a, s4, r4);
  const float p1 = __fmul_rn(s1, s2), q1 = __fmaf_rn(s1, s2, -p1);
  const float p2 = __fmul_rn(s3, s4), q2 = __fmaf_rn(s3, s4, -p2);
  const float c1 = __fadd_rn(__fadd_rn(__fmul_rn(s1, r2), __fmul_rn(r1, s2)), __fmul_rn(r1, r2));
  const float c2 = __fadd_rn(__fadd_rn(__fmul_rn(s3, r4), __fmul_rn(r3, s4)), __fmul_rn(r3, r4));
  float h, g;
  two_sum(p1, -p2, h, g);
  const float tail = __fadd_rn(__fadd_rn(__fsub_rn(q1, q2), __fsub_rn(c1, c2)), g);
  const float o = __fadd_rn(h, tail);
  const float u2 = 3.5527137e-15f;  // 2^-48
  const float ss = __fadd_rn(__fadd_rn(fabsf(s1), fabsf(s2)), __fadd_rn(fabsf(s3), fabsf(s4)));
  float E = __fmul_rn(20.0f * u2, __fadd_rn(fabsf(p1), fabsf(p2)));
  E = __fadd_rn(E, __fmul_rn(__fmul_rn(24.0f * u2, S), ss));
  E = __fadd_rn(E, __fmul_rn(__fmul_rn(128.0f * u2 * 5.9604645e-8f, S), S));
  E = __fadd_rn(E, __fmul_rn(7.2e-43f, __fadd_rn(ss, 1.0f)));
  // the bound's own roundings and the rounding of o: a 2 % margin
  E = __fmul_rn(E, 1.02f);
  if (o > E) return 1;
  if (o < -E) return -1;
  return 2;
}

__device__ int orient_sign(const Ring& P, uint32_t a, uint32_t b, uint32_t c) {
  const float d1 = ring_diff(P.Xf, P.Xl, b, a), d2 = ring_diff(P.Yf, P.Yl, c, a);
  const float d3 = ring_diff(P.Yf, P.Yl, b, a), d4 = ring_diff(P.Xf, P.Xl, c, a);
  const float p1 = __fmul_rn(d1, d2), p2 = __fmul_rn(d3, d4);
  const float o = __fsub_rn(p1, p2);
  const float S = fmaxf(fmaxf(fmaxf(fabsf(P.Xf[a]), fabsf(P.Yf[a])), fmaxf(fabsf(P.Xf[b]), fabsf(P.Yf[b]))),
                        fmaxf(fabsf(P.Xf[c]), fabsf(P.Yf[c])));
  if (S < 1e15f) {
    const float u = 5.9604645e-8f;
    const float eb = __fadd_rn(__fmul_rn(8.0f * u, __fadd_rn(fabsf(p1), fabsf(p2))),
                               __fmul_rn(__fmul_rn(8.0f * u * u, S),
                                         __fadd_rn(__fadd_rn(fabsf(d1), fabsf(d2)), __fadd_rn(fabsf(d3), fabsf(d4)))));
    // a bound in the subnormal range is not trusted
    if (eb > 1e-30f) {
      if (o > eb) return 1;
      if (o < -eb) return -1;
    }
    // near-collinear: the float-float filter, then double for what it
    // cannot decide (this GPU's FP64 rate is a small fraction of FP32's)
    const int f = orient_ff(P, a, b, c, S);
    if (f != 2) return f;
  }
  const double r = orient2(P.X[a], P.Y[a], P.X[b], P.Y[b], P.X[c], P.Y[c]);
  return r > 0 ? 1 : (r < 0 ? -1 : 0);
}

// Memo of the ear test, packed with the alive flag in alive[k]: bit 0
// alive, bits 1-2 the sign of orient2(prev, k, next) plus 2 (0: not known),
// bits 3-31 one plus a live node found inside the triangle (prev, k, next)
// (0: none known; node indices stay below 2^28, the 32-bit word arena
// holding more than 16 words per node). Both depend only on k's neighbours and the coordinates,
// so they stay valid until a clip changes k's neighbours, which resets the
// memo of the clipped ear's two neighbours. A retest whose witness is still
// alive fails at once: the host clipper's test on the same triangle finds
// that node inside again. On degenerate rings (long runs of collinear
// vertices, where each pass re-tests the same vertices and their
// orientations need double arithmetic) this removes the repeated tests.
__device__ __forceinline__ int gate_sign(const Ring& P, uint32_t k) {
  const uint32_t m = P.alive[k];
  const uint32_t code = (m >> 1) & 3u;
  if (code) return (int)code - 2;
  const int sg = orient_sign(P, P.prev[k], k, P.next[k]);
  P.alive[k] = (m & ~6u) | ((uint32_t)(sg + 2) << 1);
  return sg;
}

// the orientation gate of the ear test at vertex k (is_ear returns false at
// once when it fails): the triangle (prev, k, next) turns left, or is flat in
// flat mode
__device__ bool ear_gate(const Ring& P, uint32_t k, bool allowFlat) {
  const int sg = gate_sign(P, k);
  return sg > 0 || (sg == 0 && allowFlat);
}

// no other live node inside (or on) the triangle of ear k; the lanes split
// the nodes and vote. Each node test is the host clipper's double test; the
// float copies decide it exactly where they can, and the double arithmetic
// (slow on this GPU) runs only for ties and near-zero orientations
__device__ bool is_ear(const Ring& P, uint32_t k, bool allowFlat, int lane) {
  const uint32_t a = P.prev[k], b = k, c = P.next[k];
  const float axf = P.Xf[a], ayf = P.Yf[a], bxf = P.Xf[b], byf = P.Yf[b], cxf = P.Xf[c], cyf = P.Yf[c];
  // the ear's orientation (arPos: ar > 0; otherwise ar == 0 in flat mode)
  const int sg = gate_sign(P, k);
  if (sg < 0 || (sg == 0 && !allowFlat)) return false;
  const bool arPos = sg > 0;
  {
    // a known witness that is still alive is still inside
    const uint32_t wit = P.alive[k] >> 3;
    if (wit && (P.alive[wit - 1] & 1u)) return false;
  }
  // the node must lie in the triangle's bounding box (as in the host
  // clipper), so only the cells the box covers are looked at; the box's
  // float bounds are the float roundings of its double bounds (rounding is
  // monotonic, so it commutes with min and max)
  const float fbx0 = fminf(fminf(axf, cxf), bxf), fbx1 = fmaxf(fmaxf(axf, cxf), bxf);
  const float fby0 = fminf(fminf(ayf, cyf), byf), fby1 = fmaxf(fmaxf(ayf, cyf), byf);
  const uint32_t x0 = P.cell_x(fbx0), x1 = P.cell_x(fbx1);
  const uint32_t y0 = P.cell_y(fby0), y1 = P.cell_y(fby1);
  // the nodes of one row of covered cells are contiguous in the grid's node
  // list: the lanes take 32 consecutive entries at a time (coalesced, the
  // loads of the whole warp in flight together) and the warp stops at the
  // first batch holding a node inside
  auto inside = [&](uint32_t q) -> bool {
    if (!(P.alive[q] & 1u) || q == a || q == b || q == c) return false;
    const float qxf = P.Xf[q], qyf = P.Yf[q];
    // in the bounding box, exactly: float decides unless it ties
    if (qxf < fbx0 || qxf > fbx1 || qyf < fby0 || qyf > fby1) return false;
    if (qxf == fbx0 || qxf == fbx1 || qyf == fby0 || qyf == fby1) {
      const double qx = P.X[q], qy = P.Y[q];
      const double ax = P.X[a], ay = P.Y[a], bx = P.X[b], by = P.Y[b], cx = P.X[c], cy = P.Y[c];
      if (qx < fmin(fmin(ax, cx), bx) || qx > fmax(fmax(ax, cx), bx) || qy < fmin(fmin(ay, cy), by) ||
          qy > fmax(fmax(ay, cy), by))
        return false;
    }
    // not at a corner's position (equal doubles have equal floats)
    if ((qxf == axf && qyf == ayf && P.X[q] == P.X[a] && P.Y[q] == P.Y[a]) ||
        (qxf == bxf && qyf == byf && P.X[q] == P.X[b] && P.Y[q] == P.Y[b]) ||
        (qxf == cxf && qyf == cyf && P.X[q] == P.X[c] && P.Y[q] == P.Y[c]))
      return false;
    if (orient_sign(P, a, b, q) < 0 || orient_sign(P, b, c, q) < 0 || orient_sign(P, c, a, q) < 0) return false;
    if (!arPos) {
      // a flat ear: only nodes within the box of its two ends count
      const double qx = P.X[q], qy = P.Y[q], ax = P.X[a], ay = P.Y[a], cx = P.X[c], cy = P.Y[c];
      if (!(qx >= fmin(ax, cx) && qx <= fmax(ax, cx) && qy >= fmin(ay, cy) && qy <= fmax(ay, cy))) return false;
    }
    return true;
  };
  bool hit = false;
  uint32_t hitQ = 0;
  for (uint32_t y = y0; y <= y1 && !hit; y++) {
    const uint32_t e0 = P.gStart[y * P.gnx + x0], e1 = P.gStart[y * P.gnx + x1 + 1];
    for (uint32_t base = e0; base < e1; base += 32) {
      const uint32_t e = base + (uint32_t)lane;
      const uint32_t q = e < e1 ? P.gNodes[e] : 0u;
      const bool h = e < e1 && inside(q);
      const uint32_t hb = __ballot_sync(CUT_FULL, h);
      if (hb) {
        hit = true;
        hitQ = __shfl_sync(CUT_FULL, q, __ffs(hb) - 1);
        break;
      }
    }
  }
  if (hit) {
    __syncwarp();
    if (lane == 0) P.alive[k] = (P.alive[k] & 7u) | ((hitQ + 1) << 3);
    __syncwarp();
  }
  return !hit;
}

// the uniform grid of the ring's P.n nodes: about two nodes per cell over
// their bounding box, nodes listed per cell (lanes split the work; the order
// within a cell does not matter)
__device__ void build_grid(Ring& P, int lane) {
  float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
  for (uint32_t q = lane; q < P.n; q += 32) {
    x0 = fminf(x0, P.Xf[q]);
    x1 = fmaxf(x1, P.Xf[q]);
    y0 = fminf(y0, P.Yf[q]);
    y1 = fmaxf(y1, P.Yf[q]);
  }
  for (int d = 16; d > 0; d >>= 1) {
    x0 = fminf(x0, __shfl_xor_sync(CUT_FULL, x0, d));
    x1 = fmaxf(x1, __shfl_xor_sync(CUT_FULL, x1, d));
    y0 = fminf(y0, __shfl_xor_sync(CUT_FULL, y0, d));
    y1 = fmaxf(y1, __shfl_xor_sync(CUT_FULL, y1, d));
  }
  // about two nodes per cell, the cells shaped like the box (a long thin
  // cap gets one row of cells along its length, not a square grid whose
  // few occupied cells each hold many nodes)
  const uint32_t C = max(1u, P.n / 2);
  const float bw = x1 - x0, bh = y1 - y0;
  if (!(bw > 0.0f) && !(bh > 0.0f)) {
    P.gnx = P.gny = 1;
  } else if (!(bh > 0.0f)) {
    P.gnx = C;
    P.gny = 1;
  } else if (!(bw > 0.0f)) {
    P.gnx = 1;
    P.gny = C;
  } else {
    const float gx = sqrtf((float)C * bw / bh);
    P.gnx = gx < 1.0f ? 1u : (gx > (float)C ? C : (uint32_t)gx);
    P.gny = max(1u, C / P.gnx);
  }
  P.gx0 = x0;
  P.gy0 = y0;
  P.ginvx = x1 > x0 ? (float)P.gnx / (x1 - x0) : 0.0f;
  P.ginvy = y1 > y0 ? (float)P.gny / (y1 - y0) : 0.0f;
  const uint32_t cells = P.gnx * P.gny;
  for (uint32_t i = lane; i <= cells; i += 32) P.gCnt[i] = 0;
  __syncwarp();
  for (uint32_t q = lane; q < P.n; q += 32) atomicAdd(P.gCnt + P.cell_y(P.Yf[q]) * P.gnx + P.cell_x(P.Xf[q]), 1u);
  __syncwarp();
  uint32_t run = 0;
  for (uint32_t base = 0; base <= cells; base += 32) {
    const uint32_t i = base + lane;
    const uint32_t v = i < cells ? P.gCnt[i] : 0u;
    uint32_t inc = v;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t u = __shfl_up_sync(CUT_FULL, inc, d);
      if (lane >= d) inc += u;
    }
    if (i <= cells) P.gStart[i] = run + inc - v;
    run += __shfl_sync(CUT_FULL, inc, 31);
  }
  __syncwarp();
  for (uint32_t i = lane; i < cells; i += 32) P.gCnt[i] = P.gStart[i];
  __syncwarp();
  for (uint32_t q = lane; q < P.n; q += 32) {
    const uint32_t cell = P.cell_y(P.Yf[q]) * P.gnx + P.cell_x(P.Xf[q]);
    P.gNodes[atomicAdd(P.gCnt + cell, 1u)] = q;
  }
  __syncwarp();
}

// ear clipping of the group's ring (outer loop [0, outerEnd), holes from
// holeStart); writes ring-index triples to out; returns the triangle count
// (fewer than n + 2 h - 2 when the polygon could not be clipped)
__device__ uint32_t ear_clip(Ring& P, const uint32_t* gid, const double* gxy, uint32_t nAll, const uint32_t* hs,
                             uint32_t nHoles, uint32_t* holeL, double* holeX, uint32_t* out, int lane) {
  P.n = 0;
  const uint32_t outerEnd = nHoles == 0 ? nAll : hs[0];
  if (outerEnd < 3) return 0;
  const uint32_t outer = ring_par(P, gxy, 0, outerEnd, true, lane);
  uint32_t nh = 0;
  for (uint32_t k = 0; k < nHoles; k++) {
    const uint32_t s = hs[k], e = k + 1 < nHoles ? hs[k + 1] : nAll;
    if (e <= s) continue;
    const uint32_t h = ring_par(P, gxy, s, e, false, lane);
    uint32_t left = h, p = h, guard = 0;
    do {
      if (P.X[p] < P.X[left] || (P.X[p] == P.X[left] && P.Y[p] < P.Y[left])) left = p;
      p = P.next[p];
    } while (p != h && ++guard <= P.n);
    // stable insertion by leftmost x
    uint32_t j = nh;
    while (j > 0 && holeX[j - 1] > P.X[left]) {
      holeX[j] = holeX[j - 1];
      holeL[j] = holeL[j - 1];
      j--;
    }
    holeX[j] = P.X[left];
    holeL[j] = left;
    nh++;
    // every lane has finished reading the sorted list before the next hole
    // shifts it (warp-uniform code stays correct only if no lane runs ahead
    // into a write that another lane has not read past)
    __syncwarp();
  }
  for (uint32_t k = 0; k < nh; k++) {
    const int32_t m = find_bridge(P, holeL[k], outer, P.gNodes, P.alive, lane);
    __syncwarp();
    if (m < 0) return 0;
    P.bridge((uint32_t)m, holeL[k]);
    __syncwarp();
  }
  // the alive words held ring positions while the holes were bridged
  if (nh > 0) {
    for (uint32_t q = lane; q < P.n; q += 32) P.alive[q] = 1;
  }
  __syncwarp();
  build_grid(P, lane);
  uint32_t count = 0;
  {
    uint32_t p = outer;
    do {
      count++;
      p = P.next[p];
    } while (p != outer && count <= P.n);
    if (count > P.n) return 0;  // not a ring: never for a well-formed group
  }
  uint32_t nOut = 0;
  uint32_t ear = outer, stop = outer;
  bool flat = false;
  // The host clipper tests ear, next(ear), ... one at a time; most tests
  // fail at the orientation gate (reflex, or flat outside flat mode), and a
  // flat stretch can cost a full pass per clipped ear. Here the warp looks
  // at the next 32 vertices at once: each lane applies the gate to one, and
  // the full test runs on the gate's survivors in ring order; the first
  // that passes is the ear the host finds. Reaching `stop` ends the batch
  // there, where the host switches to flat mode (or gives up).
  __shared__ uint32_t ring33[33];
  // each batch clips an ear, ends a pass, or advances 32 vertices, so
  // 2 n^2 + 16 batches are never reached; the bound keeps a malformed ring
  // finite
  const unsigned long long maxSteps = 2ull * count * count + 16;
  unsigned long long steps = 0;
  while (count > 3) {
    if (++steps > maxSteps) return nOut;
    if (lane == 0) {
      uint32_t cv = ear;
      for (int i = 0; i < 33; i++) {
        ring33[i] = cv;
        cv = P.next[cv];
      }
    }
    __syncwarp();
    // the batch: positions [0, jStop), jStop = first return to `stop`
    uint32_t jStop = 33;
    {
      const bool isStop = lane >= 1 && ring33[lane] == stop;
      const bool isStop32 = ring33[32] == stop;
      const uint32_t bal = __ballot_sync(CUT_FULL, isStop);
      jStop = bal ? (uint32_t)(__ffs(bal) - 1) : (isStop32 ? 32u : 33u);
    }
    const uint32_t nTest = min(jStop, 32u);
    const uint32_t mine = ring33[lane];
    const bool gate = (uint32_t)lane < nTest && ear_gate(P, mine, flat);
    __syncwarp();  // the gates' memo writes before the ear tests read them
    uint32_t cand = __ballot_sync(CUT_FULL, gate);
    int found = -1;
    while (cand) {
      const int i = __ffs(cand) - 1;
      cand &= cand - 1;
      if (is_ear(P, ring33[i], flat, lane)) {
        found = i;
        break;
      }
    }
    if (found >= 0) {
      ear = ring33[found];
      const uint32_t a = P.prev[ear], c = P.next[ear];
      out[3 * nOut] = P.I[a];
      out[3 * nOut + 1] = P.I[ear];
      out[3 * nOut + 2] = P.I[c];
      nOut++;
      __syncwarp();
      P.next[a] = c;
      P.prev[c] = a;
      P.alive[ear] = 0;
      P.alive[a] = 1;  // new neighbours: the memo starts over
      P.alive[c] = 1;
      count--;
      ear = c;
      stop = c;
      flat = false;
      __syncwarp();
      continue;
    }
    if (jStop <= 32) {
      // the walk reached `stop`: the host switches to flat mode or gives up
      ear = stop;
      if (flat) return nOut;
      flat = true;
    } else {
      ear = ring33[32];
    }
    __syncwarp();
  }
  const uint32_t a = P.prev[ear], c = P.next[ear];
  out[3 * nOut] = P.I[a];
  out[3 * nOut + 1] = P.I[ear];
  out[3 * nOut + 2] = P.I[c];
  return nOut + 1;
}

// whether the half edge a -> b of a triangle cut from input triangle tri
// lies on an input edge without a reverse (open bit k of edge tri[k] ->
// tri[k + 1]); an intersection vertex is identified by its edge's key
__device__ __forceinline__ bool on_open_edge(uint32_t a, uint32_t b, const uint32_t* tri, uint32_t bits, uint32_t nv,
                                             const unsigned long long* keys) {
  if (bits == 0) return false;
  uint32_t a0 = a, a1 = a, b0 = b, b1 = b;  // each end's input edge ends
  if (a >= nv) {
    const unsigned long long k = keys[a - nv];
    a0 = (uint32_t)(k >> 32);
    a1 = (uint32_t)k;
  }
  if (b >= nv) {
    const unsigned long long k = keys[b - nv];
    b0 = (uint32_t)(k >> 32);
    b1 = (uint32_t)k;
  }
  for (int k = 0; k < 3; k++) {
    if (!(bits >> k & 1)) continue;
    const uint32_t p = tri[k], q = tri[(k + 1) % 3];
    const bool aOn = a < nv ? (a == p || a == q) : ((a0 == p && a1 == q) || (a0 == q && a1 == p));
    const bool bOn = b < nv ? (b == p || b == q) : ((b0 == p && b1 == q) || (b0 == q && b1 == p));
    // both ends on the edge, not both the same intersection of it
    if (aOn && bOn && !(a >= nv && b >= nv)) return true;
  }
  return false;
}

__global__ void k_cut_cap(const CutDesc* __restrict__ D, const CutLayout* __restrict__ L, CutOut* __restrict__ O,
                          uint32_t n, const uint32_t* __restrict__ surfT, const uint2* __restrict__ candE,
                          const int8_t* __restrict__ sgn, const double* __restrict__ hashXYZ,
                          const float* __restrict__ V, uint32_t* __restrict__ W, double* __restrict__ X,
                          const uint32_t* __restrict__ Tin, const uint8_t* __restrict__ openBits,
                          const unsigned long long* __restrict__ hashKeys) {
  extern __shared__ __align__(16) unsigned char capSm[];
  const uint32_t gw = blockIdx.x;  // one warp per block
  const int lane = threadIdx.x & 31;
  if (gw >= 2 * n) return;
  const uint32_t c = gw >> 1, side = gw & 1;
  const CutLayout& l = L[c];
  if (!l.active || O[c].fail[0] != 0) return;
  const CutDesc& d = D[c];
  const uint32_t nCand = l.candCnt[side];
  if (nCand == 0) return;
  const uint32_t m = l.mEdge[side], capMax = l.capMax[side];
  const CapCarve cv = carve(m, capMax);
  uint32_t* w = W + l.capWord[side];
  double* x = X + l.capDbl[side];
  const uint32_t* st = surfT + 3 * (size_t)l.surfOff[side];
  const uint32_t nv = d.nv;
  CapCtx ctx{&d, l.hashSize, l.hashOff, nv, hashXYZ, V};
  const double dir = side == 0 ? -1.0 : 1.0;
  auto onPlane = [&](uint32_t v) { return v >= nv || sgn[d.vBase + v] == 0; };
  auto failWith = [&](int code) {
    if (lane == 0) O[c].fail[side] = code;
  };

  // 1. the plane edges of the half's candidate triangles, in first-seen
  // order (candidate order, then triangle, then edge)
  uint32_t* eA = w + cv.eA;
  uint32_t* eB = w + cv.eB;
  uint32_t E = 0;
  for (uint32_t base = 0; base < nCand; base += 32) {
    const uint32_t i = base + lane;
    uint32_t ea[6], eb[6];
    uint32_t k = 0;
    if (i < nCand) {
      const uint2 ce = candE[l.candOff[side] + i];
      const uint32_t tIn = ce.y >> 2, nOut = ce.y & 3;
      const uint32_t bits = openBits ? openBits[d.tOff + tIn] : 0u;
      const uint32_t* inTri = Tin + 3 * ((size_t)d.tOff + tIn);
      for (uint32_t tt = 0; tt < nOut && tt < 2; tt++) {
        const uint32_t* tri = st + 3 * (size_t)(ce.x + tt);
        for (int e = 0; e < 3; e++) {
          const uint32_t a = tri[e], b = tri[(e + 1) % 3];
          if ((onPlane(a) && onPlane(b)) || on_open_edge(a, b, inTri, bits, nv, hashKeys + l.hashOff)) {
            ea[k] = a;
            eb[k] = b;
            k++;
          }
        }
      }
    }
    uint32_t inc = k;
    for (int dd = 1; dd < 32; dd <<= 1) {
      const uint32_t u = __shfl_up_sync(CUT_FULL, inc, dd);
      if (lane >= dd) inc += u;
    }
    const uint32_t tot = __shfl_sync(CUT_FULL, inc, 31);
    const uint32_t at = E + inc - k;
    for (uint32_t j = 0; j < k; j++) {
      if (at + j < m) {
        eA[at + j] = ea[j];
        eB[at + j] = eb[j];
      }
    }
    E += tot;
  }
  if (E > m) {
    failWith(CUT_SCRATCH);
    return;
  }
  __syncwarp();
  // 2. first occurrence of every directed edge and its reverse
  unsigned long long* ehKey = reinterpret_cast<unsigned long long*>(w + cv.ehKey);
  uint32_t* ehVal = w + cv.ehVal;
  for (uint32_t i = lane; i < E; i += 32) {
    const unsigned long long key = ((unsigned long long)eA[i] << 32) | eB[i];
    const uint32_t h = kh_find(ehKey, cv.eh, key, true);
    if (h != CUT_NONE) atomicMin(ehVal + h, i);
  }
  __syncwarp();
  uint32_t* bSrc = w + cv.bSrc;
  uint32_t* bDst = w + cv.bDst;
  uint32_t B = 0;
  for (uint32_t base = 0; base < E; base += 32) {
    const uint32_t i = base + lane;
    bool f = false;
    uint32_t a = 0, b = 0;
    if (i < E) {
      a = eA[i];
      b = eB[i];
      const uint32_t h = kh_find(ehKey, cv.eh, ((unsigned long long)a << 32) | b, false);
      const bool first = h != CUT_NONE && ehVal[h] == i;
      const bool twin = kh_find(ehKey, cv.eh, ((unsigned long long)b << 32) | a, false) != CUT_NONE;
      f = first && !twin;
    }
    const uint32_t bal = __ballot_sync(CUT_FULL, f);
    if (f) {
      const uint32_t at = B + __popc(bal & lanemask_lt());
      bSrc[at] = a;
      bDst[at] = b;
    }
    B += __popc(bal);
  }
  __syncwarp();
  if (B == 0) return;

  // ---- from here on the cap's sequential steps: the lanes split the
  // per-edge, per-loop and per-node work, and steps whose decisions read
  // earlier writes run on lane 0 between warp syncs

  // 3. boundary edges grouped by source vertex, in first-seen order. The
  // walk below follows these lists edge by edge, so for up to
  // CAP_SM_WALK_B edges the lists, the source-vertex hash and the edges'
  // ends live in the block's shared memory (free until the ear clipping)
  uint32_t* bNext = w + cv.bNext;
  uint32_t* bUsed = w + cv.bUsed;
  uint32_t* shKey = w + cv.shKey;
  uint32_t* shHead = w + cv.shHead;
  uint32_t* shTail = w + cv.shTail;
  uint32_t* starts = w + cv.starts;
  uint32_t shSize = cv.sh;
  const uint32_t* bSrcW = bSrc;
  const uint32_t* bDstW = bDst;
  if (B <= CAP_SM_WALK_B) {
    uint32_t* su = reinterpret_cast<uint32_t*>(capSm);
    shSize = pow2_at_least(2 * B);
    shKey = su;
    shHead = shKey + shSize;
    shTail = shHead + shSize;
    bNext = shTail + shSize;
    bUsed = bNext + B;
    uint32_t* sSrc = bUsed + B;
    uint32_t* sDst = sSrc + B;
    for (uint32_t i = lane; i < shSize; i += 32) shKey[i] = CUT_NONE;
    for (uint32_t i = lane; i < B; i += 32) {
      sSrc[i] = bSrc[i];
      sDst[i] = bDst[i];
    }
    bSrcW = sSrc;
    bDstW = sDst;
    __syncwarp();
  }
  // Steps 3 and 4 are sequential and each decision reads what earlier
  // iterations wrote (hash inserts, used flags), so they run on lane 0 alone
  // while the other lanes wait; every list walk is bounded.
  uint32_t* loopV = w + cv.loopV;
  uint32_t* loopS = w + cv.loopS;
  uint32_t nLoops = 0, nLV = 0;
  int walkFail = 0;
  if (lane == 0) {
    uint32_t nStarts = 0;
    for (uint32_t i = 0; i < B && !walkFail; i++) {
      bool ins;
      const uint32_t h = uh_find(shKey, shSize, bSrcW[i], true, &ins);
      if (h == CUT_NONE) {
        walkFail = CUT_SCRATCH;
        break;
      }
      bNext[i] = CUT_NONE;
      bUsed[i] = 0;
      if (ins) {
        shHead[h] = i;
        shTail[h] = i;
        starts[nStarts++] = bSrcW[i];
      } else {
        bNext[shTail[h]] = i;
        shTail[h] = i;
      }
    }
    // 4. boundary loops: from each start, each unused out-edge in order,
    // then the first unused out-edge at every vertex
    loopS[0] = 0;
    for (uint32_t si = 0; si < nStarts && !walkFail; si++) {
      const uint32_t start = starts[si];
      bool ins;
      const uint32_t hs = uh_find(shKey, shSize, start, false, &ins);
      uint32_t steps = 0;
      for (uint32_t e = shHead[hs]; e != CUT_NONE && !walkFail; e = bNext[e]) {
        if (++steps > B) {
          walkFail = CUT_CYCLE;
          break;
        }
        if (bUsed[e]) continue;
        if (nLV >= m) {
          walkFail = CUT_SCRATCH;
          break;
        }
        const uint32_t lvStart = nLV;
        loopV[nLV++] = start;
        bUsed[e] = 1;
        uint32_t cur = bDstW[e];
        uint32_t guard = 0;
        while (cur != start) {
          if (nLV >= m) {
            walkFail = CUT_SCRATCH;
            break;
          }
          loopV[nLV++] = cur;
          const uint32_t hc = uh_find(shKey, shSize, cur, false, &ins);
          if (hc == CUT_NONE) {
            walkFail = CUT_OPEN_CHAIN;
            break;
          }
          uint32_t nx = CUT_NONE, n2 = 0;
          for (uint32_t e2 = shHead[hc]; e2 != CUT_NONE && n2 <= B; e2 = bNext[e2], n2++)
            if (!bUsed[e2]) {
              nx = e2;
              break;
            }
          if (nx == CUT_NONE) {
            walkFail = CUT_DEAD_END;
            break;
          }
          bUsed[nx] = 1;
          cur = bDstW[nx];
          if (++guard > B + 1) {
            walkFail = CUT_CYCLE;
            break;
          }
        }
        if (walkFail) break;
        if (nLV - lvStart >= 3) loopS[++nLoops] = nLV;
        else nLV = lvStart;
      }
    }
  }
  __syncwarp();
  walkFail = __shfl_sync(CUT_FULL, walkFail, 0);
  nLoops = __shfl_sync(CUT_FULL, nLoops, 0);
  nLV = __shfl_sync(CUT_FULL, nLV, 0);
  if (walkFail) {
    failWith(walkFail);
    return;
  }
  if (nLoops == 0) return;
  // 5. loop coordinates in the plane's basis (every loop vertex at once) and
  // signed areas: the terms at once, each loop's sum in order by one lane
  double* l2 = x + cv.l2;
  double* area = x + cv.area;
  double* terms = x + cv.gXY;  // scratch until the groups are assembled
  for (uint32_t k = lane; k < nLV; k += 32) {
    double px, py, pz;
    ctx.pos(loopV[k], px, py, pz);
    double a = px * d.u[0];
    a = a + py * d.u[1];
    a = a + pz * d.u[2];
    double b = px * d.w[0];
    b = b + py * d.w[1];
    b = b + pz * d.w[2];
    l2[2 * k] = a;
    l2[2 * k + 1] = b;
  }
  __syncwarp();
  for (uint32_t li = 0; li < nLoops; li++) {
    const uint32_t s0 = loopS[li], e0 = loopS[li + 1];
    for (uint32_t k = s0 + lane; k < e0; k += 32) {
      const uint32_t j = k + 1 < e0 ? k + 1 : s0;
      terms[k] = l2[2 * k] * l2[2 * j + 1] - l2[2 * j] * l2[2 * k + 1];
    }
  }
  __syncwarp();
  for (uint32_t li = lane; li < nLoops; li += 32) {
    double s = 0;
    for (uint32_t k = loopS[li]; k < loopS[li + 1]; k++) s += terms[k];
    area[li] = s / 2;
  }
  __syncwarp();
  // outer loops wind like the largest loop
  int32_t largest = -1;
  for (uint32_t i = 0; i < nLoops; i++)
    if (largest < 0 || fabs(area[i]) > fabs(area[largest])) largest = (int32_t)i;
  const int outerSign = dsgn(area[largest]);
  // 6. a hole's parent: the smallest larger outer loop containing the hole's
  // area centroid (a lane per loop)
  uint32_t* depth = w + cv.depth;
  uint32_t* parent = w + cv.parent;
  for (uint32_t i = lane; i < nLoops; i += 32) {
    depth[i] = 0;
    parent[i] = CUT_NONE;
    if (fabs(area[i]) < 1e-18 || dsgn(area[i]) == outerSign) continue;
    depth[i] = 1;
    double cx, cy;
    {
      const uint32_t s0 = loopS[i], e0 = loopS[i + 1];
      double sx = 0, sy = 0;
      for (uint32_t k = s0; k < e0; k++) {
        const uint32_t j = k + 1 < e0 ? k + 1 : s0;
        const double wv = l2[2 * k] * l2[2 * j + 1] - l2[2 * j] * l2[2 * k + 1];
        sx += (l2[2 * k] + l2[2 * j]) * wv;
        sy += (l2[2 * k + 1] + l2[2 * j + 1]) * wv;
      }
      cx = sx / (6 * area[i]);
      cy = sy / (6 * area[i]);
    }
    double bestArea = INFINITY, fallbackArea = -INFINITY;
    uint32_t fallback = CUT_NONE, par = CUT_NONE;
    for (uint32_t j = 0; j < nLoops; j++) {
      if (i == j || fabs(area[j]) < 1e-18 || dsgn(area[j]) != outerSign) continue;
      if (fabs(area[j]) > fallbackArea) {
        fallbackArea = fabs(area[j]);
        fallback = j;
      }
      if (fabs(area[j]) <= fabs(area[i])) continue;
      bool inside = false;
      const uint32_t s0 = loopS[j], e0 = loopS[j + 1], mm = e0 - s0;
      for (uint32_t a = 0, b = mm - 1; a < mm; b = a++) {
        const double xi = l2[2 * (s0 + a)], yi = l2[2 * (s0 + a) + 1], xj = l2[2 * (s0 + b)], yj = l2[2 * (s0 + b) + 1];
        if ((yi > cy) != (yj > cy) && cx < (xj - xi) * (cy - yi) / (yj - yi) + xi) inside = !inside;
      }
      if (inside && fabs(area[j]) < bestArea) {
        bestArea = fabs(area[j]);
        par = j;
      }
    }
    parent[i] = par != CUT_NONE ? par : fallback;
  }
  __syncwarp();
  // 7. caps, in the host cut's order: fans of zero-area loops, then each
  // outer loop with its holes
  uint32_t* capT = w + cv.capT;
  double* cent = x + cv.cent;
  uint32_t nCap = 0, nCent = 0;
  const uint32_t centBase = nv + l.hashSize;
  auto fan = [&](uint32_t li) -> bool {
    const uint32_t s0 = loopS[li], e0 = loopS[li + 1], len = e0 - s0;
    if (nCap + len > capMax || nCent >= m) return false;
    double sx = 0, sy = 0, sz = 0;
    for (uint32_t k = s0; k < e0; k++) {
      double px, py, pz;
      ctx.pos(loopV[k], px, py, pz);
      sx += px;
      sy += py;
      sz += pz;
    }
    const double dl = (double)len;
    cent[3 * nCent] = sx / dl;
    cent[3 * nCent + 1] = sy / dl;
    cent[3 * nCent + 2] = sz / dl;
    const uint32_t cid = centBase + nCent++;
    for (uint32_t k = 0; k < len; k++) {
      capT[3 * nCap] = cid;
      capT[3 * nCap + 1] = loopV[s0 + (k + 1) % len];
      capT[3 * nCap + 2] = loopV[s0 + k];
      nCap++;
    }
    return true;
  };
  for (uint32_t i = 0; i < nLoops; i++)
    if (fabs(area[i]) < 1e-18 && !fan(i)) {
      failWith(CUT_SCRATCH);
      return;
    }
  // the ear clipper's nodes and grid: in shared memory when the group fits
  // CAP_SM_NODES nodes, else in the global scratch with the links and memo
  // in shared memory up to CAP_SM_LINK_NODES nodes
  Ring Pg;
  Pg.I = w + cv.ndI;
  Pg.prev = w + cv.ndPrev;
  Pg.next = w + cv.ndNext;
  Pg.alive = w + cv.ndAlive;
  Pg.X = x + cv.ndX;
  Pg.Y = x + cv.ndY;
  Pg.cap = cv.nd;
  Pg.n = 0;
  Pg.gCnt = w + cv.gCnt;
  Pg.gStart = w + cv.gStart;
  Pg.gNodes = w + cv.gNodes;
  Pg.Xf = reinterpret_cast<float*>(w + cv.ndXf);
  Pg.Yf = reinterpret_cast<float*>(w + cv.ndYf);
  Pg.Xl = reinterpret_cast<float*>(w + cv.ndXl);
  Pg.Yl = reinterpret_cast<float*>(w + cv.ndYl);
  Ring Ps;
  {
    double* sx = reinterpret_cast<double*>(capSm);
    Ps.X = sx;
    Ps.Y = sx + CAP_SM_NODES;
    uint32_t* su = reinterpret_cast<uint32_t*>(sx + 2 * CAP_SM_NODES);
    Ps.I = su;
    Ps.prev = su + CAP_SM_NODES;
    Ps.next = su + 2 * CAP_SM_NODES;
    Ps.alive = su + 3 * CAP_SM_NODES;
    Ps.gNodes = su + 4 * CAP_SM_NODES;
    Ps.gCnt = su + 5 * CAP_SM_NODES;
    Ps.gStart = Ps.gCnt + CAP_SM_NODES / 2 + 2;
    Ps.Xf = reinterpret_cast<float*>(Ps.gStart + CAP_SM_NODES / 2 + 2);
    Ps.Yf = Ps.Xf + CAP_SM_NODES;
    Ps.Xl = Ps.Yf + CAP_SM_NODES;
    Ps.Yl = Ps.Xl + CAP_SM_NODES;
    Ps.cap = CAP_SM_NODES;
    Ps.n = 0;
  }
  uint32_t* gid = w + cv.gId;
  double* gxy = x + cv.gXY;
  uint32_t* holeL = w + cv.holeL;
  double* holeX = x + cv.holeX;
  for (uint32_t i = 0; i < nLoops; i++) {
    if (fabs(area[i]) < 1e-18 || depth[i] % 2 != 0) continue;
    // the group's ring: the outer loop, then its holes in loop order (hole
    // starts kept in `starts`, free once the loops are walked); the loops'
    // vertices are copied by all lanes at once
    uint32_t nAll = 0, nHoles = 0;
    uint32_t* hs = starts;
    auto append = [&](uint32_t li) {
      const uint32_t s0 = loopS[li], len = loopS[li + 1] - s0;
      for (uint32_t q = lane; q < len; q += 32) {
        gid[nAll + q] = loopV[s0 + q];
        gxy[2 * (nAll + q)] = l2[2 * (s0 + q)];
        gxy[2 * (nAll + q) + 1] = l2[2 * (s0 + q) + 1];
      }
      nAll += len;
    };
    append(i);
    for (uint32_t j = 0; j < nLoops; j++)
      if (parent[j] == i && depth[j] % 2 == 1 && fabs(area[j]) >= 1e-18) {
        hs[nHoles++] = nAll;
        append(j);
      }
    __syncwarp();
    const uint32_t expected = nAll + 2 * nHoles - 2;
    const uint32_t ringNodes = nAll + 2 * nHoles;
    if (ringNodes > Ps.cap && ringNodes <= CAP_SM_LINK_NODES) {
      uint32_t* su = reinterpret_cast<uint32_t*>(capSm);
      Pg.prev = su;
      Pg.next = su + CAP_SM_LINK_NODES;
      Pg.alive = su + 2 * CAP_SM_LINK_NODES;
    } else {
      Pg.prev = w + cv.ndPrev;
      Pg.next = w + cv.ndNext;
      Pg.alive = w + cv.ndAlive;
    }
    Ring& P = ringNodes <= Ps.cap ? Ps : Pg;
    if (nCap + nAll + 2 * nHoles > capMax || nAll + 2 * nHoles > P.cap) {
      failWith(CUT_SCRATCH);
      return;
    }
    __syncwarp();
    const uint32_t got = ear_clip(P, gid, gxy, nAll, hs, nHoles, holeL, holeX, capT + 3 * nCap, lane);
    __syncwarp();
    if (got != expected) {
      if (!fan(i)) {
        failWith(CUT_SCRATCH);
        return;
      }
      for (uint32_t j = 0; j < nLoops; j++)
        if (parent[j] == i && depth[j] % 2 == 1 && fabs(area[j]) >= 1e-18 && !fan(j)) {
          failWith(CUT_SCRATCH);
          return;
        }
      continue;
    }
    // one flip for the whole cap, decided by its largest triangle (the
    // first of the largest |n . normal|, as a sequential scan keeps it)
    double bestAbs = 0, bestDot = 0;
    uint32_t bestK = CUT_NONE;
    for (uint32_t k = lane; k < got; k += 32) {
      const uint32_t* t = capT + 3 * (nCap + k);
      double p0x, p0y, p0z, p1x, p1y, p1z, p2x, p2y, p2z;
      ctx.pos(gid[t[0]], p0x, p0y, p0z);
      ctx.pos(gid[t[1]], p1x, p1y, p1z);
      ctx.pos(gid[t[2]], p2x, p2y, p2z);
      const double ax = p1x - p0x, ay = p1y - p0y, az = p1z - p0z;
      const double bx = p2x - p0x, by = p2y - p0y, bz = p2z - p0z;
      const double qx = ay * bz - az * by, qy = az * bx - ax * bz, qz = ax * by - ay * bx;
      double dd = qx * d.n[0];
      dd = dd + qy * d.n[1];
      dd = dd + qz * d.n[2];
      if (fabs(dd) > bestAbs) {
        bestAbs = fabs(dd);
        bestDot = dd;
        bestK = k;
      }
    }
    for (int dl = 16; dl > 0; dl >>= 1) {
      const double oa = __shfl_xor_sync(CUT_FULL, bestAbs, dl), od = __shfl_xor_sync(CUT_FULL, bestDot, dl);
      const uint32_t ok = __shfl_xor_sync(CUT_FULL, bestK, dl);
      if (oa > bestAbs || (oa == bestAbs && ok < bestK)) {
        bestAbs = oa;
        bestDot = od;
        bestK = ok;
      }
    }
    const bool flip = bestDot * dir < 0;
    __syncwarp();
    for (uint32_t k = lane; k < got; k += 32) {
      uint32_t* t = capT + 3 * (nCap + k);
      const uint32_t a = gid[t[0]], b = gid[t[1]], cc = gid[t[2]];
      t[0] = a;
      t[1] = flip ? cc : b;
      t[2] = flip ? b : cc;
    }
    __syncwarp();
    nCap += got;
    __syncwarp();
  }
  if (lane == 0) {
    O[c].cap[side] = nCap;
    O[c].cent[side] = nCent;
  }
}

// ---------------------------------------------------------------------------
// compact: vertices numbered by first use in each half's triangle list

struct SideRef {
  uint32_t c, side, local, tri;
};

__device__ __forceinline__ SideRef side_of_corner(const uint32_t* cPre, uint32_t n2, uint32_t j) {
  const uint32_t k = find_seg(cPre, n2, j);
  SideRef r;
  r.c = k >> 1;
  r.side = k & 1;
  r.local = j - cPre[k];
  r.tri = r.local / 3;
  return r;
}

// the vertex id at a corner of a half, CUT_NONE past the half's triangles
__device__ __forceinline__ uint32_t corner_id(const CutLayout& l, const CutOut& o, const SideRef& r,
                                              const uint32_t* surfT, const uint32_t* W) {
  if (r.tri < l.surfCnt[r.side]) return surfT[3 * (size_t)l.surfOff[r.side] + r.local];
  const uint32_t ct = r.tri - l.surfCnt[r.side];
  if (ct >= o.cap[r.side]) return CUT_NONE;
  const CapCarve cv = carve(l.mEdge[r.side], l.capMax[r.side]);
  return W[l.capWord[r.side] + cv.capT + 3 * ct + r.local % 3];
}

__global__ void k_cut_first_use(const CutLayout* __restrict__ L, const CutOut* __restrict__ O,
                                const uint32_t* __restrict__ cPre, uint32_t n2, uint32_t total,
                                const uint32_t* __restrict__ surfT, const uint32_t* __restrict__ W,
                                uint32_t* __restrict__ firstPos) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total) return;
  const SideRef r = side_of_corner(cPre, n2, j);
  const CutLayout& l = L[r.c];
  const CutOut& o = O[r.c];
  if (!l.active || o.fail[0] || o.fail[1]) return;
  const uint32_t v = corner_id(l, o, r, surfT, W);
  if (v == CUT_NONE) return;
  atomicMin(firstPos + l.preOff[r.side] + v, r.local);
}

__global__ void k_cut_first_flags(const CutLayout* __restrict__ L, const CutOut* __restrict__ O,
                                  const uint32_t* __restrict__ cPre, uint32_t n2, uint32_t total,
                                  const uint32_t* __restrict__ surfT, const uint32_t* __restrict__ W,
                                  const uint32_t* __restrict__ firstPos, uint32_t* __restrict__ flag) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total) return;
  const SideRef r = side_of_corner(cPre, n2, j);
  const CutLayout& l = L[r.c];
  const CutOut& o = O[r.c];
  uint32_t f = 0;
  if (l.active && !o.fail[0] && !o.fail[1]) {
    const uint32_t v = corner_id(l, o, r, surfT, W);
    f = v != CUT_NONE && firstPos[l.preOff[r.side] + v] == r.local;
  }
  flag[j] = f;
}

__global__ void k_cut_counts(uint32_t n, const uint32_t* __restrict__ cPre, const uint32_t* __restrict__ fpre,
                             CutOut* __restrict__ O) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 2 * n) return;
  O[k >> 1].nvOut[k & 1] = fpre[cPre[k + 1]] - fpre[cPre[k]];
}

__global__ void k_cut_write(const CutDesc* __restrict__ D, const CutLayout* __restrict__ L,
                            const CutOut* __restrict__ O, const uint32_t* __restrict__ cPre, uint32_t n2,
                            uint32_t total, const uint32_t* __restrict__ surfT, const uint32_t* __restrict__ W,
                            const double* __restrict__ X, const uint32_t* __restrict__ firstPos,
                            const uint32_t* __restrict__ fpre, const double* __restrict__ hashXYZ,
                            const float* __restrict__ V, const unsigned long long* __restrict__ outVOff,
                            const unsigned long long* __restrict__ outTOff, float* __restrict__ outV,
                            uint32_t* __restrict__ outT) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total) return;
  const SideRef r = side_of_corner(cPre, n2, j);
  const CutLayout& l = L[r.c];
  const CutOut& o = O[r.c];
  if (!l.active || o.fail[0] || o.fail[1]) return;
  const uint32_t v = corner_id(l, o, r, surfT, W);
  if (v == CUT_NONE) return;
  const uint32_t k = 2 * r.c + r.side;
  const uint32_t fp = firstPos[l.preOff[r.side] + v];
  const uint32_t idx = fpre[cPre[k] + fp] - fpre[cPre[k]];
  outT[outTOff[k] + r.local] = idx;
  if (fp != r.local) return;
  const CutDesc& d = D[r.c];
  float* o3 = outV + 3 * (outVOff[k] + idx);
  if (v < d.nv) {
    const float* p = V + 3 * ((size_t)d.vOff + v);
    o3[0] = p[0];
    o3[1] = p[1];
    o3[2] = p[2];
  } else if (v < d.nv + l.hashSize) {
    const double* p = hashXYZ + 3 * ((size_t)l.hashOff + (v - d.nv));
    o3[0] = (float)p[0];
    o3[1] = (float)p[1];
    o3[2] = (float)p[2];
  } else {
    const CapCarve cv = carve(l.mEdge[r.side], l.capMax[r.side]);
    const double* p = X + l.capDbl[r.side] + cv.cent + 3 * (size_t)(v - d.nv - l.hashSize);
    o3[0] = (float)p[0];
    o3[1] = (float)p[1];
    o3[2] = (float)p[2];
  }
}

// signed volume of every half by the divergence theorem anchored at its
// vertex 0 (mesh.ts:58-72), in two fixed-order steps so that large halves
// spread over many blocks: each chunk of up to VOL_CHUNK triangles is one
// block (every thread sums its strided triangles in order, then a fixed tree
// over the threads), and each half adds its chunks in order (the same value
// on every run; it differs from a sequential sum in the last bits)
constexpr uint32_t VOL_CHUNK = 4096;

__global__ void k_cut_vol_chunks(const uint4* __restrict__ chunks, const unsigned long long* __restrict__ vOff,
                                 const unsigned long long* __restrict__ tOff, const float* __restrict__ outV,
                                 const uint32_t* __restrict__ outT, double* __restrict__ part) {
  __shared__ double ws[32];
  const uint4 ch = chunks[blockIdx.x];  // half, first triangle, end triangle
  const float* v = outV + 3 * vOff[ch.x];
  const uint32_t* t = outT + tOff[ch.x];
  const double ox = v[0], oy = v[1], oz = v[2];
  double s = 0.0;
  for (uint32_t i = ch.y + threadIdx.x; i < ch.z; i += blockDim.x) {
    const uint32_t a = 3 * t[3 * i], b = 3 * t[3 * i + 1], c = 3 * t[3 * i + 2];
    const double ax = v[a] - ox, ay = v[a + 1] - oy, az = v[a + 2] - oz;
    const double bx = v[b] - ox, by = v[b + 1] - oy, bz = v[b + 2] - oz;
    const double cx = v[c] - ox, cy = v[c + 1] - oy, cz = v[c + 2] - oz;
    s += ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
  }
  for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(CUT_FULL, s, d);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (uint32_t w = 0; w < (blockDim.x >> 5); w++) tot += ws[w];
    part[blockIdx.x] = tot;
  }
}

__global__ void k_cut_vol_sum(uint32_t n2, const uint32_t* __restrict__ chunkPre, const double* __restrict__ part,
                              double* __restrict__ vol) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n2) return;
  double s = 0.0;
  for (uint32_t c = chunkPre[k]; c < chunkPre[k + 1]; c++) s += part[c];
  vol[k] = s / 6.0;
}

// open edges of the input meshes (used when the caller does not vouch for
// closed meshes): every directed edge in its mesh's hash, then per triangle a
// bit for each edge whose reverse is absent
__global__ void k_open_insert(const uint32_t* __restrict__ mPre, uint32_t nMeshes, uint32_t totalE,
                              const uint32_t* __restrict__ meshTOff, const uint32_t* __restrict__ hOff,
                              const uint32_t* __restrict__ hSize, const uint32_t* __restrict__ T,
                              unsigned long long* __restrict__ keys) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= totalE) return;
  const uint32_t mi = find_seg(mPre, nMeshes, g);
  const uint32_t e = g - mPre[mi], t = e / 3, k = e % 3;
  const uint32_t* tri = T + 3 * ((size_t)meshTOff[mi] + t);
  const unsigned long long key = ((unsigned long long)tri[k] << 32) | tri[(k + 1) % 3];
  const uint32_t size = hSize[mi];
  unsigned long long* h = keys + hOff[mi];
  uint32_t i = mix_key(key) & (size - 1);
  for (uint32_t probe = 0; probe < size; probe++, i = (i + 1) & (size - 1)) {
    const unsigned long long old = atomicCAS(h + i, EMPTY_KEY, key);
    if (old == EMPTY_KEY || old == key) return;
  }
}

__global__ void k_open_bits(const uint32_t* __restrict__ mtPre, uint32_t nMeshes, uint32_t totalT,
                            const uint32_t* __restrict__ meshTOff, const uint32_t* __restrict__ hOff,
                            const uint32_t* __restrict__ hSize, const uint32_t* __restrict__ T,
                            const unsigned long long* __restrict__ keys, uint8_t* __restrict__ bits) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= totalT) return;
  const uint32_t mi = find_seg(mtPre, nMeshes, g);
  const uint32_t t = g - mtPre[mi];
  const uint32_t* tri = T + 3 * ((size_t)meshTOff[mi] + t);
  const uint32_t size = hSize[mi];
  const unsigned long long* h = keys + hOff[mi];
  uint32_t b = 0;
  for (int k = 0; k < 3; k++) {
    const unsigned long long rev = ((unsigned long long)tri[(k + 1) % 3] << 32) | tri[k];
    uint32_t i = mix_key(rev) & (size - 1);
    bool found = false;
    for (uint32_t probe = 0; probe < size; probe++, i = (i + 1) & (size - 1)) {
      const unsigned long long kk = h[i];
      if (kk == rev) {
        found = true;
        break;
      }
      if (kk == EMPTY_KEY) break;
    }
    if (!found) b |= 1u << k;
  }
  bits[meshTOff[mi] + t] = (uint8_t)b;
}

// ---------------------------------------------------------------------------
// host side

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t need) {
    if (need <= bytes) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    need = std::max<size_t>(need, 256);
    if (cudaMalloc(&p, need) != cudaSuccess) return set_error(CUACD_E_CUDA, "cut: device allocation failed");
    bytes = need;
    return 0;
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
  ~Buf() {
    if (p) cudaFree(p);
  }
};

struct Engine {
  Buf inV, inT, desc, vPre, tPre, sizes, layout, out, cPre, dist, sgn, cnt, pre, tiles, hashKeys, hashXYZ, surfT,
      candE, firstPos, flag, fpre, words, dbls, outVOff, outTOff, outV, outT, vol, openBits, openKeys, openMeta,
      volChunks, volPre, volPart;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  void* stage = nullptr;  // pinned staging of the halves' readback
  size_t stageBytes = 0;
  ~Engine() {
    if (stage) cudaFreeHost(stage);
  }
};

Engine* engine_create() {
  Engine* e = new Engine();
  if (cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess) {
    delete e;
    return nullptr;
  }
  return e;
}

void engine_destroy(Engine* e) {
  if (!e) return;
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  delete e;
}

size_t engine_device_bytes(const Engine* e) {
  if (!e) return 0;
  size_t n = 0;
  for (const Buf* b : {&e->inV, &e->inT, &e->desc, &e->vPre, &e->tPre, &e->sizes, &e->layout, &e->out, &e->cPre,
                       &e->dist, &e->sgn, &e->cnt, &e->pre, &e->tiles, &e->hashKeys, &e->hashXYZ, &e->surfT, &e->candE,
                       &e->firstPos, &e->flag, &e->fpre, &e->words, &e->dbls, &e->outVOff, &e->outTOff, &e->outV,
                       &e->outT, &e->vol, &e->openBits, &e->openKeys, &e->openMeta, &e->volChunks, &e->volPre,
                       &e->volPart})
    n += b->bytes;
  return n;
}

#define CUTCK(x)                                                                             \
  do {                                                                                       \
    cudaError_t err_ = (x);                                                                  \
    if (err_ != cudaSuccess) return set_error(CUACD_E_CUDA, (std::string("cut: ") + #x + ": " + \
                                                             cudaGetErrorString(err_)).c_str()); \
  } while (0)

template <typename T>
static int scan(Engine* e, const T* in, uint32_t n, T* out, cudaStream_t s) {
  if (int rc = e->tiles.ensure(sizeof(T) * (scan::tiles_for(n) + 1))) return rc;
  scan::exclusive<T>(in, n, out, e->tiles.as<T>(), s);
  return 0;
}

static inline uint32_t blocks(uint64_t n, uint32_t t) { return (uint32_t)std::max<uint64_t>(1, (n + t - 1) / t); }

int engine_run(Engine* e, cudaStream_t s, const cuacd_mesh* meshes, int nMeshes, const CutSpec* cuts, int nCuts,
               bool closed, Halves* out) {
  if (!e || !out || nCuts < 0 || nMeshes < 0 || (nCuts > 0 && (!meshes || !cuts)))
    return set_error(CUACD_E_INVALID, "cut: invalid argument");
  out->status.assign(nCuts, 0);
  out->vOff.assign(2 * (size_t)nCuts, 0);
  out->tOff.assign(2 * (size_t)nCuts, 0);
  out->nv.assign(2 * (size_t)nCuts, 0);
  out->nt.assign(2 * (size_t)nCuts, 0);
  out->gpuMs = 0;
  if (nCuts == 0) return CUACD_OK;
  // ---- inputs: every mesh once, cut descriptors
  std::vector<uint64_t> mv(nMeshes + 1, 0), mt(nMeshes + 1, 0);
  for (int i = 0; i < nMeshes; i++) {
    const cuacd_mesh& m = meshes[i];
    if ((m.nv && !m.verts) || (m.nt && !m.tris)) return set_error(CUACD_E_INVALID, "cut: null mesh buffer");
    // a device mesh (both buffers in device memory) is copied on the device
    // and its indices are the caller's to vouch for; a host mesh is checked
    const bool dv = is_device_ptr(m.verts), dt = is_device_ptr(m.tris);
    if ((m.nv && m.nt && dv != dt) || (!m.nv && dt) || (!m.nt && dv))
      return set_error(CUACD_E_INVALID, "cut: a mesh's buffers must both be host or both be device memory");
    if (!dt)
      for (uint64_t k = 0; k < 3ull * m.nt; k++)
        if (m.tris[k] >= m.nv) return set_error(CUACD_E_INVALID, "cut: triangle index out of range");
    mv[i + 1] = mv[i] + m.nv;
    mt[i + 1] = mt[i] + m.nt;
  }
  const uint32_t n = (uint32_t)nCuts;
  std::vector<CutDesc> desc(n);
  std::vector<uint32_t> vPre(n + 1, 0), tPre(n + 1, 0);
  uint64_t totV = 0, totT = 0;
  for (uint32_t c = 0; c < n; c++) {
    const CutSpec& cs = cuts[c];
    if (cs.mesh < 0 || cs.mesh >= nMeshes) return set_error(CUACD_E_INVALID, "cut: mesh index out of range");
    CutDesc& d = desc[c];
    std::memset(&d, 0, sizeof(d));
    for (int a = 0; a < 3; a++) {
      d.n[a] = cs.n[a];
      d.u[a] = cs.u[a];
      d.w[a] = cs.v[a];
    }
    d.d = cs.d;
    d.vOff = (uint32_t)mv[cs.mesh];
    d.nv = meshes[cs.mesh].nv;
    d.tOff = (uint32_t)mt[cs.mesh];
    d.nt = meshes[cs.mesh].nt;
    d.vBase = (uint32_t)totV;
    d.tBase = (uint32_t)totT;
    totV += d.nv;
    totT += d.nt;
    vPre[c + 1] = (uint32_t)totV;
    tPre[c + 1] = (uint32_t)totT;
  }
  if (totV >= (1ull << 31) || totT >= (1ull << 30) || mv[nMeshes] >= (1ull << 31))
    return set_error(CUACD_E_CAPACITY, "cut: batch too large");
  int rc;
  if ((rc = e->inV.ensure(12 * mv[nMeshes])) || (rc = e->inT.ensure(12 * mt[nMeshes])) ||
      (rc = e->desc.ensure(sizeof(CutDesc) * n)) || (rc = e->vPre.ensure(4 * (n + 1))) ||
      (rc = e->tPre.ensure(4 * (n + 1))) || (rc = e->sizes.ensure(sizeof(CutSizes) * n)) ||
      (rc = e->layout.ensure(sizeof(CutLayout) * n)) || (rc = e->out.ensure(sizeof(CutOut) * n)) ||
      (rc = e->dist.ensure(8 * totV)) || (rc = e->sgn.ensure(totV)) || (rc = e->cnt.ensure(16 * totT)) ||
      (rc = e->pre.ensure(16 * (totT + 1))))
    return rc;
  CUTCK(cudaEventRecord(e->ev0, s));
  for (int i = 0; i < nMeshes; i++) {
    const cuacd_mesh& m = meshes[i];
    if (m.nv) CUTCK(cudaMemcpyAsync(e->inV.as<float>() + 3 * mv[i], m.verts, 12ull * m.nv, cudaMemcpyDefault, s));
    if (m.nt) CUTCK(cudaMemcpyAsync(e->inT.as<uint32_t>() + 3 * mt[i], m.tris, 12ull * m.nt, cudaMemcpyDefault, s));
  }
  CUTCK(cudaMemcpyAsync(e->desc.p, desc.data(), sizeof(CutDesc) * n, cudaMemcpyHostToDevice, s));
  CUTCK(cudaMemcpyAsync(e->vPre.p, vPre.data(), 4 * (n + 1), cudaMemcpyHostToDevice, s));
  CUTCK(cudaMemcpyAsync(e->tPre.p, tPre.data(), 4 * (n + 1), cudaMemcpyHostToDevice, s));
  CUTCK(cudaMemsetAsync(e->sizes.p, 0, sizeof(CutSizes) * n, s));
  // open input edges, unless the caller vouches for closed meshes
  const uint8_t* dOpen = nullptr;
  if (!closed && mt[nMeshes] > 0) {
    const uint32_t nm = (uint32_t)nMeshes;
    // edge prefix, triangle prefix, tOff, hash offset; the hash sizes follow
    std::vector<uint32_t> meta(4 * (size_t)nm + 2, 0);
    uint32_t* ePreH = meta.data();
    uint32_t* mtPreH = ePreH + nm + 1;
    uint32_t* tOffH = mtPreH + nm + 1;
    uint32_t* hOffH = tOffH + nm;
    std::vector<uint32_t> hs(nm);
    uint64_t hTot = 0;
    for (uint32_t i = 0; i < nm; i++) {
      ePreH[i + 1] = ePreH[i] + 3 * meshes[i].nt;
      mtPreH[i + 1] = mtPreH[i] + meshes[i].nt;
      tOffH[i] = (uint32_t)mt[i];
      hOffH[i] = (uint32_t)hTot;
      hs[i] = pow2_at_least(std::max<uint32_t>(16, 6 * meshes[i].nt));
      hTot += hs[i];
    }
    std::vector<uint32_t> metaAll(meta);
    metaAll.insert(metaAll.end(), hs.begin(), hs.end());
    if ((rc = e->openBits.ensure(mt[nMeshes])) || (rc = e->openKeys.ensure(8 * hTot)) ||
        (rc = e->openMeta.ensure(4 * metaAll.size())))
      return rc;
    CUTCK(cudaMemcpyAsync(e->openMeta.p, metaAll.data(), 4 * metaAll.size(), cudaMemcpyHostToDevice, s));
    CUTCK(cudaMemsetAsync(e->openKeys.p, 0xff, 8 * hTot, s));
    const uint32_t* dm = e->openMeta.as<uint32_t>();
    const uint32_t* dePre = dm;
    const uint32_t* dmtPre = dm + nm + 1;
    const uint32_t* dtOff = dm + 2 * (nm + 1);
    const uint32_t* dhOff = dtOff + nm;
    const uint32_t* dhSize = dhOff + nm;
    k_open_insert<<<blocks(3 * mt[nMeshes], 256), 256, 0, s>>>(dePre, nm, (uint32_t)(3 * mt[nMeshes]), dtOff, dhOff,
                                                              dhSize, e->inT.as<uint32_t>(),
                                                              e->openKeys.as<unsigned long long>());
    k_open_bits<<<blocks(mt[nMeshes], 256), 256, 0, s>>>(dmtPre, nm, (uint32_t)mt[nMeshes], dtOff, dhOff, dhSize,
                                                        e->inT.as<uint32_t>(), e->openKeys.as<unsigned long long>(),
                                                        e->openBits.as<uint8_t>());
    dOpen = e->openBits.as<uint8_t>();
  }
  const CutDesc* dD = e->desc.as<CutDesc>();
  CutSizes* dS = e->sizes.as<CutSizes>();
  if (totV) k_cut_classify<<<blocks(totV, 256), 256, 0, s>>>(dD, e->vPre.as<uint32_t>(), n, (uint32_t)totV,
                                                               e->inV.as<float>(), e->dist.as<double>(),
                                                               e->sgn.as<int8_t>(), dS);
  if (totT) k_cut_count<<<blocks(totT, 256), 256, 0, s>>>(dD, e->tPre.as<uint32_t>(), n, (uint32_t)totT,
                                                            e->inT.as<uint32_t>(), e->sgn.as<int8_t>(), dOpen,
                                                            e->cnt.as<uint4>(), dS);
  if ((rc = scan<uint4>(e, e->cnt.as<uint4>(), (uint32_t)totT, e->pre.as<uint4>(), s))) return rc;
  k_cut_sizes<<<blocks(n, 128), 128, 0, s>>>(dD, n, e->pre.as<uint4>(), dS);
  std::vector<CutSizes> sz(n);
  CUTCK(cudaMemcpyAsync(sz.data(), dS, sizeof(CutSizes) * n, cudaMemcpyDeviceToHost, s));
  CUTCK(cudaStreamSynchronize(s));

  // ---- layout
  std::vector<CutLayout> lay(n);
  std::vector<CutOut> outRec(n);
  std::vector<uint32_t> cPre(2 * n + 1, 0);
  uint64_t hashTot = 0, surfTot = 0, candTot = 0, preTot = 0, corners = 0, wordTot = 0, dblTot = 0;
  for (uint32_t c = 0; c < n; c++) {
    CutLayout& l = lay[c];
    std::memset(&l, 0, sizeof(l));
    std::memset(&outRec[c], 0, sizeof(CutOut));
    const bool split = sz[c].anyPos && sz[c].anyNeg;
    l.active = split ? 1 : 0;
    if (!split) {
      out->status[c] = CUT_NO_SPLIT;
      outRec[c].fail[0] = CUT_NO_SPLIT;
      cPre[2 * c + 1] = (uint32_t)corners;
      cPre[2 * c + 2] = (uint32_t)corners;
      continue;
    }
    l.hashSize = pow2_at_least(std::max<uint32_t>(16, 4 * sz[c].straddle));
    l.hashOff = (uint32_t)hashTot;
    hashTot += l.hashSize;
    for (int sd = 0; sd < 2; sd++) {
      l.surfOff[sd] = (uint32_t)surfTot;
      l.surfCnt[sd] = sz[c].surf[sd];
      surfTot += sz[c].surf[sd];
      l.candOff[sd] = (uint32_t)candTot;
      l.candCnt[sd] = sz[c].cand[sd];
      candTot += sz[c].cand[sd];
      const uint32_t m = 6 * sz[c].cand[sd] + 6;
      l.mEdge[sd] = m;
      l.capMax[sd] = 3 * m;
      l.preOff[sd] = (uint32_t)preTot;
      preTot += (uint64_t)desc[c].nv + l.hashSize + m;
      const CapCarve cv = carve(m, l.capMax[sd]);
      l.capWord[sd] = (uint32_t)wordTot;
      wordTot += cv.words;
      l.capDbl[sd] = (uint32_t)dblTot;
      dblTot += cv.dbls;
      corners += 3ull * (l.surfCnt[sd] + l.capMax[sd]);
      cPre[2 * c + sd + 1] = (uint32_t)corners;
    }
  }
  if (corners >= (1ull << 31) || preTot >= (1ull << 31) || wordTot >= (1ull << 32) || dblTot >= (1ull << 31) ||
      hashTot >= (1ull << 30))
    return set_error(CUACD_E_CAPACITY, "cut: batch too large");
  if ((rc = e->hashKeys.ensure(8 * hashTot)) || (rc = e->hashXYZ.ensure(24 * hashTot)) ||
      (rc = e->surfT.ensure(12 * surfTot)) || (rc = e->candE.ensure(8 * candTot)) ||
      (rc = e->firstPos.ensure(4 * preTot)) || (rc = e->flag.ensure(4 * corners)) ||
      (rc = e->fpre.ensure(4 * (corners + 1))) || (rc = e->words.ensure(4 * wordTot)) ||
      (rc = e->dbls.ensure(8 * dblTot)) || (rc = e->cPre.ensure(4 * (2 * n + 1))) ||
      (rc = e->outVOff.ensure(8 * 2 * n)) || (rc = e->outTOff.ensure(8 * 2 * n)))
    return rc;
  CUTCK(cudaMemcpyAsync(e->layout.p, lay.data(), sizeof(CutLayout) * n, cudaMemcpyHostToDevice, s));
  CUTCK(cudaMemcpyAsync(e->out.p, outRec.data(), sizeof(CutOut) * n, cudaMemcpyHostToDevice, s));
  CUTCK(cudaMemcpyAsync(e->cPre.p, cPre.data(), 4 * (2 * n + 1), cudaMemcpyHostToDevice, s));
  if (hashTot) CUTCK(cudaMemsetAsync(e->hashKeys.p, 0xff, 8 * hashTot, s));
  if (preTot) CUTCK(cudaMemsetAsync(e->firstPos.p, 0xff, 4 * preTot, s));
  if (wordTot) CUTCK(cudaMemsetAsync(e->words.p, 0xff, 4 * wordTot, s));
  const CutLayout* dL = e->layout.as<CutLayout>();
  CutOut* dO = e->out.as<CutOut>();
  if (totT)
    k_cut_surface<<<blocks(totT, 256), 256, 0, s>>>(dD, dL, e->tPre.as<uint32_t>(), n, (uint32_t)totT,
                                                      e->inT.as<uint32_t>(), e->inV.as<float>(), e->dist.as<double>(),
                                                      e->sgn.as<int8_t>(), e->pre.as<uint4>(),
                                                      e->hashKeys.as<unsigned long long>(), e->hashXYZ.as<double>(),
                                                      e->surfT.as<uint32_t>(), e->candE.as<uint2>(), dOpen, dO);
  // the cap warps' shared ring (above the 48 KB default); set on every run,
  // so it holds on whichever device is current
  CUTCK(cudaFuncSetAttribute(k_cut_cap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CAP_SM_BYTES));
  k_cut_cap<<<2 * n, 32, CAP_SM_BYTES, s>>>(dD, dL, dO, n, e->surfT.as<uint32_t>(), e->candE.as<uint2>(),
                                                       e->sgn.as<int8_t>(), e->hashXYZ.as<double>(),
                                                       e->inV.as<float>(), e->words.as<uint32_t>(),
                                                       e->dbls.as<double>(), e->inT.as<uint32_t>(), dOpen,
                                                       e->hashKeys.as<unsigned long long>());
  if (corners) {
    k_cut_first_use<<<blocks(corners, 256), 256, 0, s>>>(dL, dO, e->cPre.as<uint32_t>(), 2 * n, (uint32_t)corners,
                                                         e->surfT.as<uint32_t>(), e->words.as<uint32_t>(),
                                                         e->firstPos.as<uint32_t>());
    k_cut_first_flags<<<blocks(corners, 256), 256, 0, s>>>(dL, dO, e->cPre.as<uint32_t>(), 2 * n, (uint32_t)corners,
                                                           e->surfT.as<uint32_t>(), e->words.as<uint32_t>(),
                                                           e->firstPos.as<uint32_t>(), e->flag.as<uint32_t>());
  }
  if ((rc = scan<uint32_t>(e, e->flag.as<uint32_t>(), (uint32_t)corners, e->fpre.as<uint32_t>(), s))) return rc;
  k_cut_counts<<<blocks(2ull * n, 128), 128, 0, s>>>(n, e->cPre.as<uint32_t>(), e->fpre.as<uint32_t>(), dO);
  CUTCK(cudaMemcpyAsync(outRec.data(), dO, sizeof(CutOut) * n, cudaMemcpyDeviceToHost, s));
  CUTCK(cudaStreamSynchronize(s));

  // ---- outputs
  std::vector<unsigned long long> vo(2 * n, 0), to(2 * n, 0);
  uint64_t outVTot = 0, outTTot = 0;
  for (uint32_t c = 0; c < n; c++) {
    const CutOut& o = outRec[c];
    int st = out->status[c];
    if (st == 0) st = o.fail[0] ? o.fail[0] : o.fail[1];
    out->status[c] = st;
    for (int sd = 0; sd < 2; sd++) {
      const size_t k = 2 * (size_t)c + sd;
      vo[k] = outVTot;
      to[k] = outTTot;
      if (st != 0) continue;
      out->nv[k] = o.nvOut[sd];
      out->nt[k] = lay[c].surfCnt[sd] + o.cap[sd];
      out->vOff[k] = outVTot;
      out->tOff[k] = outTTot;
      outVTot += out->nv[k];
      outTTot += out->nt[k];
    }
  }
  if ((rc = e->outV.ensure(12 * outVTot)) || (rc = e->outT.ensure(12 * outTTot)) ||
      (rc = e->vol.ensure(8 * 2 * n)))
    return rc;
  for (auto& x : to) x *= 3;  // corner offsets
  CUTCK(cudaMemcpyAsync(e->outVOff.p, vo.data(), 8 * 2 * n, cudaMemcpyHostToDevice, s));
  CUTCK(cudaMemcpyAsync(e->outTOff.p, to.data(), 8 * 2 * n, cudaMemcpyHostToDevice, s));
  if (corners)
    k_cut_write<<<blocks(corners, 256), 256, 0, s>>>(dD, dL, dO, e->cPre.as<uint32_t>(), 2 * n, (uint32_t)corners,
                                                     e->surfT.as<uint32_t>(), e->words.as<uint32_t>(),
                                                     e->dbls.as<double>(), e->firstPos.as<uint32_t>(),
                                                     e->fpre.as<uint32_t>(), e->hashXYZ.as<double>(),
                                                     e->inV.as<float>(), e->outVOff.as<unsigned long long>(),
                                                     e->outTOff.as<unsigned long long>(), e->outV.as<float>(),
                                                     e->outT.as<uint32_t>());
  {
    // chunks of the halves' triangles for the volume sums
    std::vector<uint4> chunks;
    std::vector<uint32_t> chunkPre(2 * (size_t)n + 1, 0);
    for (uint32_t k = 0; k < 2 * n; k++) {
      for (uint32_t t0 = 0; t0 < out->nt[k]; t0 += VOL_CHUNK)
        chunks.push_back(make_uint4(k, t0, std::min<uint32_t>(out->nt[k], t0 + VOL_CHUNK), 0));
      chunkPre[k + 1] = (uint32_t)chunks.size();
    }
    if ((rc = e->volChunks.ensure(16 * std::max<size_t>(chunks.size(), 1))) ||
        (rc = e->volPre.ensure(4 * chunkPre.size())) || (rc = e->volPart.ensure(8 * std::max<size_t>(chunks.size(), 1))))
      return rc;
    if (!chunks.empty()) {
      CUTCK(cudaMemcpyAsync(e->volChunks.p, chunks.data(), 16 * chunks.size(), cudaMemcpyHostToDevice, s));
      k_cut_vol_chunks<<<(uint32_t)chunks.size(), 256, 0, s>>>(e->volChunks.as<uint4>(),
                                                              e->outVOff.as<unsigned long long>(),
                                                              e->outTOff.as<unsigned long long>(), e->outV.as<float>(),
                                                              e->outT.as<uint32_t>(), e->volPart.as<double>());
    }
    CUTCK(cudaMemcpyAsync(e->volPre.p, chunkPre.data(), 4 * chunkPre.size(), cudaMemcpyHostToDevice, s));
    k_cut_vol_sum<<<blocks(2ull * n, 128), 128, 0, s>>>(2 * n, e->volPre.as<uint32_t>(), e->volPart.as<double>(),
                                                        e->vol.as<double>());
  }
  CUTCK(cudaGetLastError());
  out->vol.assign(2 * (size_t)n, 0.0);
  CUTCK(cudaMemcpyAsync(out->vol.data(), e->vol.p, 8 * 2 * n, cudaMemcpyDeviceToHost, s));
  // the halves come back into the engine's pinned staging buffer (grown,
  // never shrunk) and are copied into the result's own host arrays
  const size_t need = 12 * outVTot + 12 * outTTot + 16;
  if (e->stageBytes < need) {
    if (e->stage) cudaFreeHost(e->stage);
    e->stage = nullptr;
    e->stageBytes = 0;
    CUTCK(cudaMallocHost(&e->stage, std::max<size_t>(need, 1 << 20)));
    e->stageBytes = std::max<size_t>(need, 1 << 20);
  }
  out->host.resize((need + 3) / 4);
  out->V = reinterpret_cast<float*>(out->host.data());
  out->T = out->host.data() + 3 * outVTot;
  float* stV = static_cast<float*>(e->stage);
  uint32_t* stT = reinterpret_cast<uint32_t*>(static_cast<uint8_t*>(e->stage) + 12 * outVTot);
  if (outVTot) CUTCK(cudaMemcpyAsync(stV, e->outV.p, 12 * outVTot, cudaMemcpyDeviceToHost, s));
  if (outTTot) CUTCK(cudaMemcpyAsync(stT, e->outT.p, 12 * outTTot, cudaMemcpyDeviceToHost, s));
  CUTCK(cudaEventRecord(e->ev1, s));
  CUTCK(cudaStreamSynchronize(s));
  std::memcpy(out->V, stV, 12 * outVTot);
  std::memcpy(out->T, stT, 12 * outTTot);
  // the halves stay in the engine's output buffers until its next batch
  out->dV = e->outV.as<float>();
  out->dT = e->outT.as<uint32_t>();
  cudaEventElapsedTime(&out->gpuMs, e->ev0, e->ev1);
  return CUACD_OK;
}

}  // namespace cut
}  // namespace cuacd
