// hull_kernel.cu — exact incremental convex hulls of the tree's child parts
// (the reference's hull kernel, src/gpu/shaders.ts:752-1401), on sm_103a.
//
// Per part: quantise to a 2^21 grid across the largest bbox extent, take the
// extremes along 40 fixed axes as 80 seeds, build a simplex, insert the
// seeds farthest-first, then every point still outside, farthest-first.
// Orientation signs come from a float32 determinant when it clears a
// rigorous rounding bound and from an exact 64/128-bit integer determinant
// otherwise (the reference uses three 32-bit limbs; the sign is the same).
//
// GB300 design:
//   * one group per part: a warp for parts up to smallNv points, a block of
//     256, 512 or 1024 threads above; persistent groups walk the level's parts, each
//     with its own scratch slab (owner, dist, candidates, faces, visible list)
//   * visible faces are listed in slot order and new faces are created in
//     horizon-edge order with group prefix sums, so the face sets are
//     deterministic (the reference uses atomicAdd order); the most visible
//     face and the next point break ties by the lowest index
//   * the hull volume is an exact 128-bit sum of integer determinants
//
// Compiled with --fmad=false: face ranking values match the CPU oracle bit
// for bit, and with them the insertion order and the face sets.
#include <type_traits>

#include "cuacd_dev.cuh"

namespace cuacd {

#define HULL_VIS_MAX 2048u
#define ALIVE 0x80000000u
// points a warp group keeps in shared memory (3 floats each)
#define QC_MAX 256u

// k-DOP seed axes (shaders.ts:769-810): the same table, so the seeds are the
// same extreme points as the reference picks
__constant__ float c_kdop[40][3] = {
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

struct HullSm {
  uint32_t seed[80];
  uint32_t nf, nalive, fail, compacted;
  uint32_t ncand, ok, nvis;
  uint32_t nfRef;    // register hull: the slot count the slot-array form would have
  uint32_t remapN;   // candidates cand[0, remapN) whose owner slots a compaction renumbers
  uint32_t newBase;  // first slot of the faces the last insertion created
  uint32_t pad[2];
};

// Register hull (one warp, up to TINY_FACES faces, face k in lane k): the
// staging area for the faces an insertion creates and the horizon maps.
#define TINY_FACES 32u
// parts whose distinct seeds exceed this go straight to the slot-array form
// (a hull with F <= 32 faces has at most 18 vertices)
#define TINY_SEEDS 24u
struct TinySm {
  uint32_t stage[3 * TINY_FACES];  // new face j: a, b, old lane of the face across (a, b)
  uint8_t hA[QC_MAX];              // per point: lane of the new face starting there
  uint8_t hB[QC_MAX];              // per point: lane of the new face ending there
};

// exact sign of det[e1; e2; d] for integer vectors below 2^23 (shaders.ts:868-876)
__device__ __noinline__ int orient_exact(f3 e1f, f3 e2f, f3 df) {
  long long e1x = (long long)e1f.x, e1y = (long long)e1f.y, e1z = (long long)e1f.z;
  long long e2x = (long long)e2f.x, e2y = (long long)e2f.y, e2z = (long long)e2f.z;
  long long dx = (long long)df.x, dy = (long long)df.y, dz = (long long)df.z;
  long long cx = e1y * e2z - e1z * e2y;
  long long cy = e1z * e2x - e1x * e2z;
  long long cz = e1x * e2y - e1y * e2x;
  __int128 det = (__int128)cx * dx + (__int128)cy * dy + (__int128)cz * dz;
  return det > 0 ? 1 : (det < 0 ? -1 : 0);
}
// filtered orientation (shaders.ts:878-884)
__device__ __forceinline__ int orient_filtered(f3 n, f3 e1, f3 e2, f3 d) {
  float det = dot(n, d);
  float bound = ((1e-6f * l1(e1)) * l1(e2)) * l1(d);
  if (det > bound) return 1;
  if (det < -bound) return -1;
  return orient_exact(e1, e2, d);
}

struct HullCtx {
  const float* V;
  uint32_t vOff, nv;
  f3 qlo;
  float qs;
  uint32_t fmax;
  uint32_t* owner;
  float* dist;
  uint32_t* cand;
  uint32_t* F;     // face records, 16 words each
  uint32_t* vis;   // visible face slots in slot order (HULL_VIS_MAX)
  uint32_t* q;     // walk queue (HULL_VIS_MAX)
  uint32_t* nbr;   // 4 words per face slot: the faces across its 3 edges
  uint32_t* bm;    // one bit per face slot
  uint32_t* wp;    // compaction: alive faces before each bitmap word
  uint32_t* hA;    // per point: new face whose horizon edge starts there
  uint32_t* hB;    // per point: new face whose horizon edge ends there
  const float* qc;  // quantised points in shared memory, or null

  __device__ __forceinline__ f3 qvert(uint32_t i) const {
    if (qc) return mk3(qc[3 * i], qc[3 * i + 1], qc[3 * i + 2]);
    f3 v = ldv(V, (size_t)vOff + 3 * (size_t)i) - qlo;
    return mk3(rintf(v.x * qs), rintf(v.y * qs), rintf(v.z * qs));
  }
  __device__ __forceinline__ uint4* rec(uint32_t f) const { return reinterpret_cast<uint4*>(F + 16 * (size_t)f); }
  __device__ __forceinline__ bool alive(uint32_t f) const { return (F[16 * (size_t)f] & ALIVE) != 0; }
  __device__ __forceinline__ void abc(uint32_t f, uint32_t& a, uint32_t& b, uint32_t& c) const {
    uint4 w = rec(f)[0];
    a = w.x & 0x7fffffffu; b = w.y; c = w.z;
  }
  // face record (16-word slots):
  //   ia|alive ib ic kb | nx ny nz s | ax ay az Nx.lo | Ny.lo Nz.lo Nx.hi|Ny.hi<<16 Nz.hi
  // kb = 1e-6 * |e1|_1 * |e2|_1 is the rounding-bound factor of the filtered
  // predicate and s = max(|n|, 1e-30) the ranking divisor, both rounded
  // exactly as the predicate rounds them when it forms them itself. N is the
  // exact integer normal e1 x e2: grid differences are at most 2^21, so each
  // component is below 2^43 and splits into a low word and a 16-bit high part.
  __device__ __forceinline__ void face_make(uint32_t a, uint32_t b, uint32_t c, uint4& w0, uint4& w1, uint4& w2,
                                            uint4& w3) const {
    face_make_q(a, b, c, qvert(c), w0, w1, w2, w3);
  }
  // face_make with the grid point of corner c given
  __device__ __forceinline__ void face_make_q(uint32_t a, uint32_t b, uint32_t c, f3 pc, uint4& w0, uint4& w1,
                                              uint4& w2, uint4& w3) const {
    f3 pa = qvert(a), pb = qvert(b);
    f3 e1 = pb - pa, e2 = pc - pa;
    f3 n = cross(e1, e2);
    const float kb = 1e-6f * (l1(e1) * l1(e2));
    const float s = fmaxf(sqrtf(dot(n, n)), 1e-30f);
    const long long e1x = (long long)e1.x, e1y = (long long)e1.y, e1z = (long long)e1.z;
    const long long e2x = (long long)e2.x, e2y = (long long)e2.y, e2z = (long long)e2.z;
    const long long Nx = e1y * e2z - e1z * e2y, Ny = e1z * e2x - e1x * e2z, Nz = e1x * e2y - e1y * e2x;
    const uint32_t hx = (uint32_t)(Nx >> 32) & 0xffffu, hy = (uint32_t)(Ny >> 32) & 0xffffu;
    w0 = make_uint4(a | ALIVE, b, c, __float_as_uint(kb));
    w1 = make_uint4(__float_as_uint(n.x), __float_as_uint(n.y), __float_as_uint(n.z), __float_as_uint(s));
    w2 = make_uint4(__float_as_uint(pa.x), __float_as_uint(pa.y), __float_as_uint(pa.z), (uint32_t)Nx);
    w3 = make_uint4((uint32_t)Ny, (uint32_t)Nz, hx | (hy << 16), (uint32_t)(Nz >> 32));
  }
  __device__ __forceinline__ void face_write(uint32_t f, uint32_t a, uint32_t b, uint32_t c) const {
    uint4 w0, w1, w2, w3;
    face_make(a, b, c, w0, w1, w2, w3);
    uint4* w = rec(f);
    w[0] = w0; w[1] = w1; w[2] = w2; w[3] = w3;
  }
  // the float32 filter on loaded record words: the ranking value det/|n|
  // when the point is visible beyond the rounding bound, -1 when it is
  // behind it, 0 when the sign needs the exact determinant. Grid
  // coordinates are integers, so a nonzero det is at least 1 and det/|n|
  // is above 2^-46: the exact test's 1e-30 is below every filtered value.
  // A corner of the face itself (point index pi) is never visible: its
  // determinant is exactly zero, and the float32 one stays inside the bound
  // (its rounding error is below 5 * 2^-24 * |e1|_1^2 * |e2|_1), so the
  // filter would hand it to the exact test, which returns zero.
  __device__ __forceinline__ float face_filter(uint4 w0, uint4 w1, uint4 w2, f3 p, uint32_t pi) const {
    const f3 n = mk3(__uint_as_float(w1.x), __uint_as_float(w1.y), __uint_as_float(w1.z));
    const f3 d = p - mk3(__uint_as_float(w2.x), __uint_as_float(w2.y), __uint_as_float(w2.z));
    const float det = dot(n, d);
    const float bound = __uint_as_float(w0.w) * l1(d);
    if (det > bound) return det / __uint_as_float(w1.w);
    if (det < -bound) return -1.0f;
    return ((w0.x & 0x7fffffffu) == pi || w0.y == pi || w0.z == pi) ? -1.0f : 0.0f;
  }
  // exact visibility of p from the face (shaders.ts:868-876): the sign of
  // N . (p - a) with the stored integer normal. With N = 2^32 h + l (l the
  // unsigned low word) the determinant is 2^32 A + B, A = h . d below 2^37
  // and B = l . d below 2^57; folding B's high part into A leaves
  // 2^32 A' + r with 0 <= r < 2^32, whose sign is A''s, or r's when A' = 0.
  __device__ __forceinline__ bool face_exact(uint4 w2, uint4 w3, f3 p) const {
    const long long dx = (long long)(p.x - __uint_as_float(w2.x));
    const long long dy = (long long)(p.y - __uint_as_float(w2.y));
    const long long dz = (long long)(p.z - __uint_as_float(w2.z));
    const long long hx = (short)(w3.z & 0xffffu), hy = (short)(w3.z >> 16), hz = (short)w3.w;
    const long long A = hx * dx + hy * dy + hz * dz;
    const long long B = (long long)w2.w * dx + (long long)w3.x * dy + (long long)w3.y * dz;
    const long long A2 = A + (B >> 32);
    return A2 > 0 || (A2 == 0 && (uint32_t)B != 0u);
  }
  // the predicate (shaders.ts:906-921): positive = visible (ranking value),
  // negative = not visible
  __device__ __forceinline__ float face_eval(uint32_t f, f3 p, uint32_t pi) const {
    const uint4* w = rec(f);
    const uint4 w0 = w[0];
    if ((w0.x & ALIVE) == 0) return -1e30f;
    const uint4 w2 = w[2];
    const float v = face_filter(w0, w[1], w2, p, pi);
    return v != 0.0f ? v : (face_exact(w2, w[3], p) ? 1e-30f : -1.0f);
  }
  // the most visible face of [f0, f1) for point i (first slot on ties;
  // distance 0 when none). An exact-visible face ranks 1e-30, below every
  // filtered value, so the exact test only runs while no face is visible.
  __device__ __forceinline__ void best_face(uint32_t i, uint32_t f0, uint32_t f1, uint32_t& bestF, float& bestD) const {
    const f3 pt = qvert(i);
    bestF = CUACD_NONE;
    bestD = 0.0f;
    for (uint32_t f = f0; f < f1; f++) {
      const uint4* w = rec(f);
      const uint4 w0 = w[0];
      if ((w0.x & ALIVE) == 0) continue;
      const uint4 w2 = w[2];
      const float dd = face_filter(w0, w[1], w2, pt, i);
      if (dd > bestD) { bestD = dd; bestF = f; }
      if (dd == 0.0f && bestF == CUACD_NONE && face_exact(w2, w[3], pt)) { bestD = 1e-30f; bestF = f; }
    }
  }
  __device__ __forceinline__ void assign(uint32_t i, uint32_t f0, uint32_t f1) const {
    uint32_t bestF;
    float bestD;
    best_face(i, f0, f1, bestF, bestD);
    owner[i] = bestF;
    dist[i] = bestD;
  }
};

__device__ __forceinline__ bool shares_edge(uint32_t f0, uint32_t f1, uint32_t f2, uint32_t g0, uint32_t g1, uint32_t g2) {
  uint32_t f[3] = {f0, f1, f2};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    uint32_t a = f[k], b = f[k == 2 ? 0 : k + 1];
    if ((g0 == b && g1 == a) || (g1 == b && g2 == a) || (g2 == b && g0 == a)) return true;
  }
  return false;
}

// Adjacency: nbr[4 f + k] is the face across edge k of face f, edges being
// (a, b), (b, c), (c, a). The bitmap bm marks the faces visible from the
// point being inserted (and, during a compaction, the alive faces).
__device__ __forceinline__ bool bm_test(const uint32_t* bm, uint32_t f) { return (bm[f >> 5] >> (f & 31)) & 1u; }

// remove dead face slots, keeping slot order (shaders.ts:946-969). Face
// f's new slot is its rank among alive faces: the alive bitmap's word
// prefix plus the bits below f in its word. Neighbour slots are renumbered
// the same way. Returns the new slot of `track`.
template <int G>
__device__ __noinline__ uint32_t hull_compact(const HullCtx& h, HullSm& hs, GrpSmem& sm, uint32_t track,
                                              uint32_t* slotOwn = nullptr, uint32_t nSlots = 0) {
  const int lid = Grp<G>::lid();
  const uint32_t nf = hs.nf;
  const uint32_t nw = (nf + 31) / 32;
  // alive bitmap, one ballot per 32 slots
  for (uint32_t c = 0; c * G < nf; c++) {
    const uint32_t f = c * G + lid;
    const bool al = f < nf && h.alive(f);
    const unsigned m = __ballot_sync(FULLMASK, al);
    if ((threadIdx.x & 31) == 0 && (f >> 5) < nw) h.bm[f >> 5] = m;
  }
  Grp<G>::sync();
  uint32_t run = 0;
  for (uint32_t c = 0; c * G < nw; c++) {
    const uint32_t w = c * G + lid;
    const uint32_t cnt = w < nw ? __popc(h.bm[w]) : 0u;
    uint32_t tot;
    const uint32_t pre = grp_scan_u<G>(cnt, &tot, sm);
    if (w < nw) h.wp[w] = run + pre;
    run += tot;
  }
  Grp<G>::sync();
  auto rank = [&](uint32_t f) { return h.wp[f >> 5] + __popc(h.bm[f >> 5] & ((1u << (f & 31)) - 1u)); };
  // the candidates' owners (alive faces) move with their faces
  for (uint32_t k = lid; k < hs.remapN; k += G) {
    const uint32_t i = h.cand[k];
    const uint32_t o = h.owner[i];
    if (o < nf && bm_test(h.bm, o)) h.owner[i] = rank(o);
  }
  // owners kept per candidate slot (the block path)
  for (uint32_t k = lid; k < nSlots; k += G) {
    const uint32_t o = slotOwn[k];
    if (o < nf && bm_test(h.bm, o)) slotOwn[k] = rank(o);
  }
  for (uint32_t c = 0; c * G < nf; c++) {
    const uint32_t f = c * G + lid;
    uint4 w0 = make_uint4(0, 0, 0, 0), w1 = w0, w2 = w0, w3 = w0, nb = w0;
    bool al = false;
    if (f < nf) {
      const uint4* r = h.rec(f);
      w0 = r[0];
      al = (w0.x & ALIVE) != 0;
      if (al) {
        w1 = r[1]; w2 = r[2]; w3 = r[3];
        nb = *reinterpret_cast<const uint4*>(h.nbr + 4 * (size_t)f);
        if (nb.x < nf) nb.x = rank(nb.x);
        if (nb.y < nf) nb.y = rank(nb.y);
        if (nb.z < nf) nb.z = rank(nb.z);
      }
    }
    Grp<G>::sync();
    if (al) {
      const uint32_t r0 = rank(f);
      uint4* r = h.rec(r0);
      r[0] = w0; r[1] = w1; r[2] = w2; r[3] = w3;
      *reinterpret_cast<uint4*>(h.nbr + 4 * (size_t)r0) = nb;
    }
    Grp<G>::sync();
  }
  const uint32_t tracked = track < nf ? rank(track) : track;
  Grp<G>::sync();
  for (uint32_t w = lid; w < nw; w += G) h.bm[w] = 0;
  if (lid == 0) { hs.nf = run; hs.compacted = 1; }
  Grp<G>::sync();
  return tracked;
}

// Insert point pIdx (shaders.ts:975-1055). The reference scans every face
// slot for visible faces and keeps the edge-connected component of the
// most visible one; with exact predicates the visible faces of a convex
// hull form one connected patch, so here the patch is walked from the
// point's owner face (a visible face) across neighbours, and the bitmap of
// the patch is then listed in slot order: the visible list, the horizon
// order and the new face slots are the reference's deterministic ones.
// The bitmap stays set for hull_grow's reassignment and is cleared there.
template <int G>
__device__ __noinline__ void hull_insert(const HullCtx& h, HullSm& hs, GrpSmem& sm, uint32_t pIdx, uint32_t start) {
  const int lid = Grp<G>::lid();
  const f3 p = h.qvert(pIdx);
  uint32_t nf = hs.nf;
  const uint32_t nalive = hs.nalive;
  if (nf + 3 * HULL_VIS_MAX > h.fmax || nf > 2 * nalive + 512) {
    start = hull_compact<G>(h, hs, sm, start);
    nf = hs.nf;
  }
  // breadth-first walk over visible neighbours, claiming faces in bm
  if (lid == 0) {
    h.q[0] = start;
    h.bm[start >> 5] |= 1u << (start & 31);
  }
  Grp<G>::sync();
  uint32_t head = 0, qn = 1;
  bool overflow = false;
  while (head < qn) {
    const uint32_t tasks = 3 * (qn - head);
    uint32_t added = 0;
    for (uint32_t t0 = 0; t0 < tasks; t0 += G) {
      const uint32_t t = t0 + lid;
      uint32_t g = 0;
      bool claimed = false;
      if (t < tasks) {
        g = h.nbr[4 * (size_t)h.q[head + t / 3] + t % 3];
        if (g < nf && !bm_test(h.bm, g) && h.face_eval(g, p, pIdx) > 0.0f) {
          const uint32_t bit = 1u << (g & 31);
          claimed = (atomicOr(h.bm + (g >> 5), bit) & bit) == 0;
        }
      }
      uint32_t tot;
      const uint32_t pre = grp_scan_bit<G>(claimed, &tot, sm);
      if (claimed && qn + added + pre < HULL_VIS_MAX) h.q[qn + added + pre] = g;
      added += tot;
    }
    Grp<G>::sync();
    head = qn;
    qn += added;
    if (qn > HULL_VIS_MAX) { overflow = true; break; }
  }
  const uint32_t nw = (nf + 31) / 32;
  if (overflow || nf + 3 * qn > h.fmax) {
    // visible-set overflow (code 1) or face slots exhausted (code 2)
    for (uint32_t w = lid; w < nw; w += G) h.bm[w] = 0;
    if (lid == 0) hs.fail = overflow ? 1u : 2u;
    Grp<G>::sync();
    return;
  }
  const uint32_t nvis = qn;
  // the visible faces in slot order
  uint32_t pos = 0;
  for (uint32_t c = 0; c * G < nw; c++) {
    const uint32_t w = c * G + lid;
    uint32_t bits = w < nw ? h.bm[w] : 0u;
    uint32_t tot;
    uint32_t at = pos + grp_scan_u<G>(__popc(bits), &tot, sm);
    while (bits) {
      const uint32_t b = __ffs(bits) - 1;
      h.vis[at++] = 32 * w + b;
      bits &= bits - 1;
    }
    pos += tot;
  }
  Grp<G>::sync();
  // horizon edges in order e = 3 * listPos + k become new faces (a, b, p):
  // an edge is on the horizon when the face across it is not visible
  uint32_t nnew = 0;
  for (uint32_t c = 0; c * G < 3 * nvis; c++) {
    const uint32_t e = c * G + lid;
    bool isNew = false;
    uint32_t a = 0, b = 0, f = 0, twin = 0;
    if (e < 3 * nvis) {
      const uint32_t vi = e / 3, k = e % 3;
      f = h.vis[vi];
      twin = h.nbr[4 * (size_t)f + k];
      if (twin >= nf || !bm_test(h.bm, twin)) {
        isNew = true;
        uint32_t fa, fb, fc;
        h.abc(f, fa, fb, fc);
        a = k == 0 ? fa : (k == 1 ? fb : fc);
        b = k == 0 ? fb : (k == 1 ? fc : fa);
      }
    }
    uint32_t tot;
    const uint32_t pre = grp_scan_bit<G>(isNew, &tot, sm);
    if (isNew) {
      const uint32_t s = nf + nnew + pre;
      h.face_write(s, a, b, pIdx);
      h.nbr[4 * (size_t)s] = twin;
      if (twin < nf) {
        uint32_t* tn = h.nbr + 4 * (size_t)twin;
        for (int j = 0; j < 3; j++) if (tn[j] == f) tn[j] = s;
      }
      h.hA[a] = s;
      h.hB[b] = s;
    }
    nnew += tot;
  }
  Grp<G>::sync();
  // new faces around the horizon loop: (b, p) borders the face starting at
  // b, (p, a) the face ending at a
  for (uint32_t s = nf + lid; s < nf + nnew; s += G) {
    uint32_t a, b, c;
    h.abc(s, a, b, c);
    h.nbr[4 * (size_t)s + 1] = h.hA[b];
    h.nbr[4 * (size_t)s + 2] = h.hB[a];
  }
  for (uint32_t vi = lid; vi < nvis; vi += G) h.F[16 * (size_t)h.vis[vi]] &= 0x7fffffffu;
  if (lid == 0) {
    hs.newBase = nf;
    hs.nf = nf + nnew;
    hs.nalive = nalive + nnew - nvis;
    hs.nvis = nvis;
  }
  Grp<G>::sync();
}

// hull_grow for a warp whose candidate list fits its lanes: lane k holds
// candidate k (point ci, owner co, distance cd) in registers. The pick (the
// largest distance, lowest point index on ties) is two redux operations and
// reassignment is per lane; dropping inside points from the list is not
// needed because the pick does not depend on list order. Same result as
// hull_grow; the owner and distance arrays are not kept up to date.
__device__ __noinline__ uint32_t hull_grow_lanes(const HullCtx& h, HullSm& hs, GrpSmem& sm, uint32_t nfPrev,
                                                 uint32_t maxIter, uint32_t ci, uint32_t co, float cd) {
  const int lane = threadIdx.x & 31;
  uint32_t nIns = 0;
  for (uint32_t iter = 0; iter < maxIter; iter++) {
    const uint32_t key = co != CUACD_NONE ? __float_as_uint(cd) : 0u;
    const uint32_t mk = __reduce_max_sync(FULLMASK, key);
    if (mk == 0u) break;
    const uint32_t pick = __reduce_min_sync(FULLMASK, key == mk ? ci : CUACD_NONE);
    const unsigned holder = __ballot_sync(FULLMASK, key == mk && ci == pick);
    const uint32_t start = __shfl_sync(FULLMASK, co, __ffs(holder) - 1);
    if (lane == 0) hs.compacted = 0;
    __syncwarp();
    hull_insert<32>(h, hs, sm, pick, start);
    nIns++;
    if (hs.fail) break;
    const uint32_t nfNow = hs.nf;
    const bool compacted = hs.compacted != 0;
    if (ci == pick) co = CUACD_NONE;
    if (co != CUACD_NONE && (compacted || bm_test(h.bm, co))) h.best_face(ci, compacted ? 0 : nfPrev, nfNow, co, cd);
    __syncwarp();
    for (uint32_t vi = lane; vi < hs.nvis; vi += 32) h.bm[h.vis[vi] >> 5] = 0;
    __syncwarp();
    nfPrev = nfNow;
  }
  __syncwarp();
  return nIns;
}

// ---------------------------------------------------------------------------
// Register hull: the same insertion sequence as hull_grow_lanes + hull_insert
// for a hull of at most 32 alive faces, with face k held by lane k. The
// lanes keep the alive faces in slot order (survivors in order, then the new
// faces in horizon order), which is all the slot order decides: the first
// slot on ranking ties and the visible-list order. The slot counter of the
// slot-array form (nfRef) is carried along because it decides when that
// form compacts, which makes the next reassignment scan every face, and the
// face-slot failure. The faces live in the slot array densely (slots 0 ..
// nalive-1) before and after each call.

struct TinyFace {
  uint4 w0, w1, w2, w3;    // face record words
  uint32_t nb0, nb1, nb2;  // lanes across edges (a, b), (b, c), (c, a)
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
// bit position of the (k+1)-th set bit of m, for k < popc(m)
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t k) {
  uint32_t pos = 0;
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1) {
    const uint32_t c = __popc(m & ((1u << w) - 1u));
    if (k >= c) { k -= c; m >>= w; pos += w; }
  }
  return pos;
}
__device__ __forceinline__ float tiny_eval(const HullCtx& h, const TinyFace& F, f3 p, uint32_t pi) {
  const float v = h.face_filter(F.w0, F.w1, F.w2, p, pi);
  return v != 0.0f ? v : (h.face_exact(F.w2, F.w3, p) ? 1e-30f : -1.0f);
}
__device__ __forceinline__ uint4 shfl4(uint4 v, uint32_t src) {
  v.x = __shfl_sync(FULLMASK, v.x, src);
  v.y = __shfl_sync(FULLMASK, v.y, src);
  v.z = __shfl_sync(FULLMASK, v.z, src);
  v.w = __shfl_sync(FULLMASK, v.w, src);
  return v;
}

// Returns the number of insertions, or CUACD_NONE when the hull outgrows
// the warp (the caller then builds it again in the slot-array form). A
// face-slot failure sets hs.fail = 2 as hull_insert does.
// Candidates on lanes below nInit start without an owner and are assigned
// over every face first (the seed phase's assignment over the simplex).
__device__ __noinline__ uint32_t hull_tiny_grow(const HullCtx& h, HullSm& hs, TinySm& ts, uint32_t maxIter,
                                                uint32_t ci, uint32_t co, float cd, uint32_t nInit) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt = lanemask_lt();
  uint32_t nalive = hs.nalive, nfRef = hs.nfRef;
  TinyFace F;
  F.w0 = F.w1 = F.w2 = F.w3 = make_uint4(0, 0, 0, 0);
  F.nb0 = F.nb1 = F.nb2 = 0;
  if (lane < nalive) {
    const uint4* r = h.rec(lane);
    F.w0 = r[0]; F.w1 = r[1]; F.w2 = r[2]; F.w3 = r[3];
    const uint4 nb = *reinterpret_cast<const uint4*>(h.nbr + 4 * lane);
    F.nb0 = nb.x; F.nb1 = nb.y; F.nb2 = nb.z;
  }
  uint32_t nIns = 0;
  bool outgrown = false;
  // candidates waiting for a (re)assignment over faces [lo, nalive)
  uint32_t R = __ballot_sync(FULLMASK, lane < nInit);
  uint32_t lo = 0;
  for (uint32_t iter = 0;; iter++) {
    // reassign the candidates whose owner died in the last insertion (all of
    // them after a compaction) over its new faces (every face after a
    // compaction); a face ranks first in slot order on ties
    while (R) {
      const uint32_t r = __ffs(R) - 1;
      R &= R - 1;
      const uint32_t pr = __shfl_sync(FULLMASK, ci, r);
      float v = -1.0f;
      if (lane >= lo && lane < nalive) v = tiny_eval(h, F, h.qvert(pr), pr);
      const uint32_t vk = v > 0.0f ? __float_as_uint(v) : 0u;
      const uint32_t best = __reduce_max_sync(FULLMASK, vk);
      const unsigned at = __ballot_sync(FULLMASK, best != 0u && vk == best);
      if (lane == r) {
        co = best != 0u ? (uint32_t)(__ffs(at) - 1) : CUACD_NONE;
        cd = best != 0u ? __uint_as_float(best) : 0.0f;
      }
    }
    if (iter == maxIter) break;
    // the farthest candidate, lowest point index on ties
    const uint32_t key = co != CUACD_NONE ? __float_as_uint(cd) : 0u;
    const uint32_t mk = __reduce_max_sync(FULLMASK, key);
    if (mk == 0u) break;
    const uint32_t pick = __reduce_min_sync(FULLMASK, key == mk ? ci : CUACD_NONE);
    const unsigned holder = __ballot_sync(FULLMASK, key == mk && ci == pick);
    const uint32_t start = __shfl_sync(FULLMASK, co, __ffs(holder) - 1);
    const f3 pp = h.qvert(pick);
    nIns++;
    // the slot-array form compacts here (hull_insert's condition)
    bool compacted = false;
    if (nfRef + 3 * HULL_VIS_MAX > h.fmax || nfRef > 2 * nalive + 512) {
      nfRef = nalive;
      compacted = true;
    }
    // visible faces, and the edge-connected patch of the start face
    const bool live = lane < nalive;
    const uint32_t V = __ballot_sync(FULLMASK, live && tiny_eval(h, F, pp, pick) > 0.0f);
    uint32_t C = 1u << start;
    for (uint32_t it = 0; it < TINY_FACES; it++) {
      const bool nin = (((C >> (F.nb0 & 31u)) | (C >> (F.nb1 & 31u)) | (C >> (F.nb2 & 31u))) & 1u) != 0;
      const uint32_t C2 = C | __ballot_sync(FULLMASK, ((V >> lane) & 1u) && nin);
      if (C2 == C) break;
      C = C2;
    }
    const uint32_t qn = __popc(C);
    if (nfRef + 3 * qn > h.fmax) {
      if (lane == 0) hs.fail = 2;
      break;
    }
    // horizon edges in order 3 * listPos + k become new faces (a, b, pick)
    const bool inC = ((C >> lane) & 1u) != 0;
    const bool e0 = inC && !((C >> (F.nb0 & 31u)) & 1u);
    const bool e1 = inC && !((C >> (F.nb1 & 31u)) & 1u);
    const bool e2 = inC && !((C >> (F.nb2 & 31u)) & 1u);
    const uint32_t cnt = (uint32_t)e0 + (uint32_t)e1 + (uint32_t)e2;
    const uint32_t B0 = __ballot_sync(FULLMASK, cnt & 1u), B1 = __ballot_sync(FULLMASK, (cnt & 2u) != 0);
    const uint32_t nnew = __popc(B0) + 2 * __popc(B1);
    const uint32_t alive = nalive >= 32 ? FULLMASK : ((1u << nalive) - 1u);
    const uint32_t S = alive & ~C;
    const uint32_t nS = __popc(S);
    if (nS + nnew > TINY_FACES) {
      outgrown = true;
      break;
    }
    if (inC) {
      uint32_t j = __popc(B0 & lt) + 2 * __popc(B1 & lt);
      const uint32_t a = F.w0.x & 0x7fffffffu, b = F.w0.y, c = F.w0.z;
      if (e0) { ts.stage[3 * j] = a; ts.stage[3 * j + 1] = b; ts.stage[3 * j + 2] = F.nb0; ts.hA[a] = (uint8_t)(nS + j); ts.hB[b] = (uint8_t)(nS + j); j++; }
      if (e1) { ts.stage[3 * j] = b; ts.stage[3 * j + 1] = c; ts.stage[3 * j + 2] = F.nb1; ts.hA[b] = (uint8_t)(nS + j); ts.hB[c] = (uint8_t)(nS + j); j++; }
      if (e2) { ts.stage[3 * j] = c; ts.stage[3 * j + 1] = a; ts.stage[3 * j + 2] = F.nb2; ts.hA[c] = (uint8_t)(nS + j); ts.hB[a] = (uint8_t)(nS + j); }
    }
    __syncwarp();
    // survivors move down in order, new faces follow
    const uint32_t src = lane < nS ? nth_set_bit(S, lane) : lane;
    F.w0 = shfl4(F.w0, src); F.w1 = shfl4(F.w1, src); F.w2 = shfl4(F.w2, src); F.w3 = shfl4(F.w3, src);
    F.nb0 = __shfl_sync(FULLMASK, F.nb0, src);
    F.nb1 = __shfl_sync(FULLMASK, F.nb1, src);
    F.nb2 = __shfl_sync(FULLMASK, F.nb2, src);
    if (lane < nS) {
      // a neighbour that died is replaced by the new face on that edge,
      // which starts at this edge's end point
      const uint32_t a = F.w0.x & 0x7fffffffu, b = F.w0.y, c = F.w0.z;
      F.nb0 = ((C >> F.nb0) & 1u) ? ts.hA[b] : __popc(S & ((1u << F.nb0) - 1u));
      F.nb1 = ((C >> F.nb1) & 1u) ? ts.hA[c] : __popc(S & ((1u << F.nb1) - 1u));
      F.nb2 = ((C >> F.nb2) & 1u) ? ts.hA[a] : __popc(S & ((1u << F.nb2) - 1u));
    } else if (lane < nS + nnew) {
      const uint32_t j = lane - nS;
      const uint32_t a = ts.stage[3 * j], b = ts.stage[3 * j + 1], tw = ts.stage[3 * j + 2];
      h.face_make(a, b, pick, F.w0, F.w1, F.w2, F.w3);
      F.nb0 = __popc(S & ((1u << tw) - 1u));
      F.nb1 = ts.hA[b];
      F.nb2 = ts.hB[a];
    }
    __syncwarp();
    // owners that survived move down with their faces; the others wait for
    // the reassignment at the top of the next pass
    if (ci == pick) co = CUACD_NONE;
    bool need = false;
    if (co != CUACD_NONE) {
      if (compacted || ((C >> co) & 1u)) need = true;
      else co = __popc(S & ((1u << co) - 1u));
    }
    R = __ballot_sync(FULLMASK, need);
    lo = compacted ? 0u : nS;
    nalive = nS + nnew;
    nfRef += nnew;
  }
  __syncwarp();
  if (outgrown) return CUACD_NONE;
  // back to the slot array, densely
  if (lane < nalive) {
    uint4* r = h.rec(lane);
    r[0] = F.w0; r[1] = F.w1; r[2] = F.w2; r[3] = F.w3;
    *reinterpret_cast<uint4*>(h.nbr + 4 * lane) = make_uint4(F.nb0, F.nb1, F.nb2, 0u);
  }
  if (lane == 0) {
    hs.nf = nalive;
    hs.nalive = nalive;
    hs.nfRef = nfRef;
  }
  __syncwarp();
  return nIns;
}

// Reassignment of candidate i over every face [0, nf1), as the reference
// does after a compaction (shaders.ts:1090-1101), without scanning every
// face: the faces visible from a point form one edge-connected patch, so the
// patch is walked from one visible face and the most visible face of the
// patch (first slot on ties) is the most visible face of all. The walk
// starts at the point's owner when it survived the insertion (an alive face
// keeps its record, so it still sees the point), else at the first new face
// that sees the point; a point outside a dead owner and outside the new hull
// is outside one of the new faces (the cone faces cover what the dead faces
// saw), so when no new face sees it the point is inside. A patch larger than
// PATCH_CAP falls back to the scan.
#define PATCH_CAP 64u
__device__ __noinline__ void patch_best(const HullCtx& h, uint32_t i, uint32_t own, bool dead, uint32_t nb0,
                                        uint32_t nf1, uint32_t& outF, float& outD) {
  const f3 pt = h.qvert(i);
  uint32_t q[PATCH_CAP];
  uint32_t n = 0;
  uint32_t bestF = CUACD_NONE;
  float bestD = 0.0f;
  if (!dead) {
    const float v = h.face_eval(own, pt, i);
    if (!(v > 0.0f)) {
      h.best_face(i, 0, nf1, outF, outD);
      return;
    }
    q[n++] = own;
    bestF = own;
    bestD = v;
  } else {
    for (uint32_t f = nb0; f < nf1; f++) {
      const float v = h.face_eval(f, pt, i);
      if (v > 0.0f) {
        q[n++] = f;
        bestF = f;
        bestD = v;
        break;
      }
    }
  }
  for (uint32_t head = 0; head < n; head++) {
    const uint32_t f = q[head];
    for (int k = 0; k < 3; k++) {
      const uint32_t g = h.nbr[4 * (size_t)f + k];
      if (g >= nf1) continue;
      bool seen = false;
      for (uint32_t j = 0; j < n; j++) seen |= q[j] == g;
      if (seen) continue;
      const float v = h.face_eval(g, pt, i);
      if (!(v > 0.0f)) continue;
      if (n == PATCH_CAP) {
        h.best_face(i, 0, nf1, outF, outD);
        return;
      }
      q[n++] = g;
      if (v > bestD || (v == bestD && g < bestF)) {
        bestD = v;
        bestF = g;
      }
    }
  }
  outF = bestF;
  outD = bestF != CUACD_NONE ? bestD : 0.0f;
}
__device__ __forceinline__ void reassign_patch(const HullCtx& h, uint32_t i, uint32_t own, bool dead, uint32_t nb0,
                                               uint32_t nf1) {
  uint32_t f;
  float d;
  patch_best(h, i, own, dead, nb0, nf1, f, d);
  h.owner[i] = f;
  h.dist[i] = d;
}

// farthest-first insertion of the candidate list (shaders.ts:1060-1129)
template <int G>
__device__ __noinline__ uint32_t hull_grow(const HullCtx& h, HullSm& hs, GrpSmem& sm, uint32_t nfPrev, uint32_t maxIter) {
  const int lid = Grp<G>::lid();
  uint32_t ncand = hs.ncand;
  uint32_t sinceCompact = 0, nIns = 0;
  for (uint32_t iter = 0; iter < maxIter; iter++) {
    if (ncand == 0) break;
    float md = -1.0f;
    uint32_t mi = CUACD_NONE;
    for (uint32_t k = lid; k < ncand; k += G) {
      uint32_t i = h.cand[k];
      if (h.owner[i] != CUACD_NONE) am_merge(md, mi, h.dist[i], i);
    }
    grp_argmax_pos<G>(md, mi, sm);
    if (md < 0.0f) break;
    const uint32_t pick = mi;
    if (lid == 0) {
      hs.compacted = 0;
      hs.remapN = ncand;
    }
    Grp<G>::sync();
    if (G > 32) {
      // a visible patch is a few faces: the insertion's walk, horizon and
      // linking run on the first warp with warp-level scans, the block
      // meets once afterwards instead of at every step
      if (threadIdx.x < 32) hull_insert<32>(h, hs, sm, pick, h.owner[pick]);
      Grp<G>::sync();
    } else {
      hull_insert<G>(h, hs, sm, pick, h.owner[pick]);
    }
    nIns++;
    if (hs.fail) break;
    const uint32_t nfNow = hs.nf;
    const bool compacted = hs.compacted != 0;
    const uint32_t newBase = hs.newBase;
    Grp<G>::sync();
    if (lid == 0) { h.owner[pick] = CUACD_NONE; h.dist[pick] = 0.0f; hs.remapN = 0; }
    Grp<G>::sync();
    // an owner face died in this insertion exactly when it was visible;
    // after a compaction every candidate is reassigned over every face
    for (uint32_t k = lid; k < ncand; k += G) {
      uint32_t i = h.cand[k];
      uint32_t own = h.owner[i];
      if (own == CUACD_NONE) continue;
      if (compacted) {
        reassign_patch(h, i, own, bm_test(h.bm, own), newBase, nfNow);
        continue;
      }
      if (!bm_test(h.bm, own)) continue;
      h.assign(i, nfPrev, nfNow);
    }
    Grp<G>::sync();
    for (uint32_t vi = lid; vi < hs.nvis; vi += G) h.bm[h.vis[vi] >> 5] = 0;
    Grp<G>::sync();
    nfPrev = nfNow;
    if (++sinceCompact >= 4) {
      sinceCompact = 0;
      uint32_t nc = 0;
      for (uint32_t c = 0; c * G < ncand; c++) {
        const uint32_t k = c * G + lid;
        uint32_t keep = 0, i = 0;
        if (k < ncand) { i = h.cand[k]; keep = h.owner[i] != CUACD_NONE ? 1u : 0u; }
        uint32_t tot;
        uint32_t pre = grp_scan_bit<G>(keep != 0, &tot, sm);
        Grp<G>::sync();
        if (keep) h.cand[nc + pre] = i;
        nc += tot;
        Grp<G>::sync();
      }
      ncand = nc;
    }
  }
  if (lid == 0) hs.ncand = ncand;
  Grp<G>::sync();
  return nIns;
}

// ---------------------------------------------------------------------------
// Block path (parts above smallNv points, 256, 512 or 1024 threads). The same insertion
// sequence and face slots as hull_grow + hull_insert, laid out for latency:
//   * the insertion (warp 0) keeps the visible patch in shared memory: a
//     hash set of its faces, their corners and the faces across their
//     edges, read once during the walk; the slot order is a rank sort of the
//     patch and the horizon loop is matched in shared memory. A patch of more
//     than BIG_VIS faces falls back to hull_insert (nothing global has been
//     written by then).
//   * the candidates are kept per candidate slot k (point cand[k], owner
//     and distance in the owner and dist words at k), so one coalesced pass
//     after each insertion drops the inserted point, reassigns the points of
//     dead faces and finds the next pick (largest distance, lowest point
//     index); dead slots are squeezed out when they reach a quarter.
#ifndef BIG_VIS
#define BIG_VIS 128u
#endif
#define BIG_HASH 256u
#define BIG_NREC 32u
struct BigSm {
  uint32_t key[BIG_HASH];     // patch face + 1; 0 = empty
  uint32_t f[BIG_VIS];        // patch faces in walk order
  uint32_t nb[BIG_VIS][3];    // faces across their edges
  uint32_t vabc[BIG_VIS][3];  // their corners
  uint32_t ord[BIG_VIS];      // walk index of the patch's k-th face in slot order
  uint32_t hzA[3 * BIG_VIS];  // new face j: start and end of its horizon edge
  uint32_t hzB[3 * BIG_VIS];
  uint4 nrec[BIG_NREC][4];    // records of the first new faces, for the reassignment
  uint32_t fast, ntodo;
};

// Batched rounds. A round takes the next picks in key order c_0, c_1, ...,
// walks their visible patches on the current hull in parallel (one warp
// each) and inserts the longest prefix whose insertions, one after
// another, give the hull the single-pick loop gives:
//   * the patches are disjoint and no face of a later patch borders a face
//     of an earlier one. A new face of c_i borders only c_i's other new
//     faces and the faces across c_i's horizon, so c_j's visible faces,
//     horizon and new faces are the ones found on the current hull, and
//     c_j's orphans (the points its patch owns) are the current ones;
//   * c_j still holds the largest key once c_0 .. c_(j-1) are in: the
//     orphans of each earlier patch get their new keys over that patch's
//     new faces, and all of them are below c_j's key;
//   * neither the compaction rule nor the slot limit fires at any of the
//     steps (a round whose first step would compact runs the single-pick
//     step).
// c_j's new faces take the slots the single-pick loop gives them, right
// after c_(j-1)'s, so face slots, owners and insertion order are the
// single-pick loop's.
// picks per round: one per warp of the block (NW warps)
#define BAT_FACES 32u   // faces of a batched patch, one per lane
#define BAT_NEW 36u     // its horizon edges (a connected patch of n faces has at most n + 2)
#define BAT_HASH_BITS 6u
// the faces of every whole walked patch: at most NW * BAT_FACES, so the set
// is never more than half full
#ifndef KMAX_CAP
#define KMAX_CAP 16u
#endif
template <int NW>
struct BatDims {
  static constexpr uint32_t BLK_BITS = NW <= 8 ? 9u : (NW <= 16 ? 10u : 11u);
  static constexpr uint32_t NRC = NW <= 8 ? 16u : 8u;  // new-face records per step kept in shared memory
  // picks per round: one per warp, at most KMAX_CAP (the merge of the
  // warps' lists is serial in the picks, and later picks rarely pass the
  // checks: on 15-28k-point blob hulls 12 and 16 measured the same, 20
  // 1-2 % slower, 28 4-6 % slower)
  static constexpr uint32_t KMAX = NW < KMAX_CAP ? (uint32_t)NW : KMAX_CAP;
};
#define BAT_LIST 8u  // keys per warp list
// candidate slots per thread in flight in the batched round's slot pass
#ifndef SCAN_U
#define SCAN_U 4
#endif
// dead candidate slots are squeezed out above 1 / SQZ_DIV of the list
#ifndef SQZ_DIV
#define SQZ_DIV 8u
#endif
// orphans listed per round (six words each in the visible list's and walk
// queue's words); a round with more inserts its first step alone
#ifndef TODO_CAP
#define TODO_CAP (HULL_VIS_MAX / 3)
#endif
struct BatWalk {
  uint32_t key[1u << BAT_HASH_BITS];  // patch face + 1; 0 = empty
  uint32_t f[BAT_FACES];              // patch faces in walk order
  uint32_t nb[BAT_FACES][3];          // faces across their edges
  uint32_t vabc[BAT_FACES][3];        // their corners
  uint32_t ord[BAT_FACES];            // walk index of the k-th face in slot order
  uint32_t hA[BAT_NEW], hB[BAT_NEW];  // new face q: its horizon edge (a, b)
  uint32_t tw[BAT_NEW], df[BAT_NEW];  // the face across that edge and the patch face inside it
  uint32_t n, nnew, ok, pick;
};
template <int NW>
struct BatSm {
  static constexpr uint32_t BLK_BITS = BatDims<NW>::BLK_BITS, NRC = BatDims<NW>::NRC;
  union {
    BigSm big;  // the single-pick step
    BatWalk w[NW];
  } u;
  // per warp: its largest candidate keys in descending order with their
  // slots and owners, their count, whether keys below the last one may be
  // missing, and the warp's count of dead slots
  unsigned long long wk[NW][BAT_LIST];
  uint32_t ws[NW][BAT_LIST], wo[NW][BAT_LIST];
  uint32_t wn[NW], wt[NW], wdead[NW];
  // faces of the whole walked patches (face + 1, 0 = empty) with the bit
  // mask of the walks (warps) that hold them
  uint2 btab[1u << BLK_BITS];
  // words 0-2 of the first NRC new faces of each step
  uint4 nrc[NW][NRC][3];
  unsigned long long selKey[NW], maxOrph[NW];
  uint32_t selSlot[NW], selOwn[NW];
  uint32_t nfj[NW + 1], nalj[NW + 1];  // slot and alive counts before step j
  uint32_t cf[NW];                     // patch j meets an earlier patch
  uint32_t nsel, ntodo, totDead;
};

// open-addressing face sets in shared memory (face + 1 stored, 0 = empty)
template <uint32_t BITS>
__device__ __forceinline__ uint32_t tab_hash(uint32_t f) { return (f * 2654435761u) >> (32 - BITS); }
template <uint32_t BITS>
__device__ __forceinline__ bool tab_has(const uint32_t* key, uint32_t f) {
  constexpr uint32_t N = 1u << BITS;
  uint32_t s = tab_hash<BITS>(f);
  for (uint32_t n = 0; n < N; n++) {
    const uint32_t k = *reinterpret_cast<const volatile uint32_t*>(key + s);
    if (k == f + 1) return true;
    if (k == 0) return false;
    s = (s + 1) & (N - 1);
  }
  return false;
}
// 1: inserted, 0: already present, 2: set full; *at = its entry
template <uint32_t BITS>
__device__ __forceinline__ uint32_t tab_add(uint32_t* key, uint32_t f, uint32_t& at) {
  constexpr uint32_t N = 1u << BITS;
  uint32_t s = tab_hash<BITS>(f);
  for (uint32_t n = 0; n < N; n++) {
    const uint32_t old = atomicCAS(key + s, 0u, f + 1);
    at = s;
    if (old == 0) return 1;
    if (old == f + 1) return 0;
    s = (s + 1) & (N - 1);
  }
  return 2;
}

// the block's set of whole walked patches' faces: add f with a walk's bit
// (the set never fills: at most half its entries are used)
template <int NW>
__device__ __forceinline__ void btab_add(BatSm<NW>& B, uint32_t f, uint32_t bit) {
  constexpr uint32_t N = 1u << BatSm<NW>::BLK_BITS;
  uint32_t s = tab_hash<BatSm<NW>::BLK_BITS>(f);
  for (uint32_t n = 0; n < N; n++) {
    const uint32_t old = atomicCAS(&B.btab[s].x, 0u, f + 1);
    if (old == 0 || old == f + 1) {
      atomicOr(&B.btab[s].y, bit);
      return;
    }
    s = (s + 1) & (N - 1);
  }
}
// the mask of the walks holding face f, 0 when none (the set is not changing)
template <int NW>
__device__ __forceinline__ uint32_t btab_mask(const BatSm<NW>& B, uint32_t f) {
  constexpr uint32_t N = 1u << BatSm<NW>::BLK_BITS;
  uint32_t s = tab_hash<BatSm<NW>::BLK_BITS>(f);
  for (uint32_t n = 0; n < N; n++) {
    const uint2 e = B.btab[s];
    if (e.x == f + 1) return e.y;
    if (e.x == 0) return 0;
    s = (s + 1) & (N - 1);
  }
  return 0;
}

// the single-pick step's patch set (BIG_HASH = 2^8 entries)
static_assert(BIG_HASH == (1u << 8), "the single-pick patch set has 2^8 entries");
__device__ __forceinline__ bool big_has(const BigSm& bs, uint32_t f) { return tab_has<8>(bs.key, f); }
// 1: inserted, 0: already present, 2: table full
__device__ __forceinline__ uint32_t big_add(BigSm& bs, uint32_t f) {
  uint32_t at;
  return tab_add<8>(bs.key, f, at);
}

// hull_insert for warp 0 with the patch in shared memory; false when the
// patch exceeds BIG_VIS faces (nothing changed: the caller runs hull_insert)
__device__ __noinline__ bool big_insert(const HullCtx& h, HullSm& hs, BigSm& bs, uint32_t pIdx, uint32_t start) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt = lanemask_lt();
  const f3 p = h.qvert(pIdx);
  const uint32_t nf = hs.nf, nalive = hs.nalive;
  for (uint32_t j = lane; j < BIG_HASH; j += 32) bs.key[j] = 0;
  __syncwarp();
  if (lane == 0) {
    big_add(bs, start);
    bs.f[0] = start;
    const uint4 w0 = h.rec(start)[0];
    const uint4 nb = *reinterpret_cast<const uint4*>(h.nbr + 4 * (size_t)start);
    bs.vabc[0][0] = w0.x & 0x7fffffffu; bs.vabc[0][1] = w0.y; bs.vabc[0][2] = w0.z;
    bs.nb[0][0] = nb.x; bs.nb[0][1] = nb.y; bs.nb[0][2] = nb.z;
  }
  __syncwarp();
  // breadth-first walk over visible neighbours; a face's record and its
  // neighbours are read together, once
  uint32_t head = 0, qn = 1;
  for (;;) {
    const uint32_t tasks = 3 * (qn - head);
    uint32_t added = 0;
    bool over = false;
    for (uint32_t t0 = 0; t0 < tasks; t0 += 32) {
      const uint32_t t = t0 + lane;
      bool claimed = false;
      uint32_t g = 0;
      uint4 w0 = make_uint4(0, 0, 0, 0), nb = w0;
      if (t < tasks) {
        g = bs.nb[head + t / 3][t % 3];
        if (g < nf && !big_has(bs, g)) {
          const uint4* r = h.rec(g);
          w0 = r[0];
          const uint4 w1 = r[1], w2 = r[2];
          nb = *reinterpret_cast<const uint4*>(h.nbr + 4 * (size_t)g);
          if (w0.x & ALIVE) {
            const float v = h.face_filter(w0, w1, w2, p, pIdx);
            if (v > 0.0f || (v == 0.0f && h.face_exact(w2, r[3], p))) {
              const uint32_t rr = big_add(bs, g);
              claimed = rr == 1;
              over = rr == 2;
            }
          }
        }
      }
      const unsigned m = __ballot_sync(FULLMASK, claimed);
      const uint32_t at = qn + added + __popc(m & lt);
      if (claimed && at < BIG_VIS) {
        bs.f[at] = g;
        bs.vabc[at][0] = w0.x & 0x7fffffffu; bs.vabc[at][1] = w0.y; bs.vabc[at][2] = w0.z;
        bs.nb[at][0] = nb.x; bs.nb[at][1] = nb.y; bs.nb[at][2] = nb.z;
      }
      added += __popc(m);
    }
    __syncwarp();
    head = qn;
    qn += added;
    if (__any_sync(FULLMASK, over) || qn > BIG_VIS) return false;
    if (head == qn) break;
  }
  const uint32_t n = qn;
  if (nf + 3 * n > h.fmax) {
    // face slots exhausted (hull_insert's code 2)
    if (lane == 0) hs.fail = 2u;
    __syncwarp();
    return true;
  }
  // the patch in slot order
  for (uint32_t i = lane; i < n; i += 32) {
    const uint32_t fi = bs.f[i];
    uint32_t r = 0;
    for (uint32_t j = 0; j < n; j++) r += bs.f[j] < fi ? 1u : 0u;
    bs.ord[r] = i;
  }
  __syncwarp();
  // horizon edges in order e = 3 * listPos + k become new faces (a, b, p)
  uint32_t nnew = 0;
  for (uint32_t c = 0; c * 32 < 3 * n; c++) {
    const uint32_t e = c * 32 + lane;
    bool isNew = false;
    uint32_t a = 0, b = 0, f = 0, twin = 0;
    if (e < 3 * n) {
      const uint32_t vi = bs.ord[e / 3], k = e % 3;
      f = bs.f[vi];
      twin = bs.nb[vi][k];
      if (twin >= nf || !big_has(bs, twin)) {
        isNew = true;
        a = bs.vabc[vi][k];
        b = bs.vabc[vi][k == 2 ? 0 : k + 1];
      }
    }
    const unsigned m = __ballot_sync(FULLMASK, isNew);
    if (isNew) {
      const uint32_t j = nnew + __popc(m & lt);
      const uint32_t s = nf + j;
      // the twin's neighbours are read before the new record is stored
      uint4 tn = make_uint4(0, 0, 0, 0);
      if (twin < nf) tn = *reinterpret_cast<const uint4*>(h.nbr + 4 * (size_t)twin);
      uint4 w0, w1, w2, w3;
      h.face_make_q(a, b, pIdx, p, w0, w1, w2, w3);
      uint4* w = h.rec(s);
      w[0] = w0; w[1] = w1; w[2] = w2; w[3] = w3;
      if (j < BIG_NREC) {
        bs.nrec[j][0] = w0; bs.nrec[j][1] = w1; bs.nrec[j][2] = w2; bs.nrec[j][3] = w3;
      }
      h.nbr[4 * (size_t)s] = twin;
      if (twin < nf) {
        uint32_t* tq = h.nbr + 4 * (size_t)twin;
        if (tn.x == f) tq[0] = s;
        if (tn.y == f) tq[1] = s;
        if (tn.z == f) tq[2] = s;
      }
      bs.hzA[j] = a;
      bs.hzB[j] = b;
    }
    nnew += __popc(m);
  }
  __syncwarp();
  // around the horizon loop: (b, p) borders the new face starting at b,
  // (p, a) the new face ending at a
  for (uint32_t j = lane; j < nnew; j += 32) {
    const uint32_t a = bs.hzA[j], b = bs.hzB[j];
    uint32_t j1 = 0, j2 = 0;
    for (uint32_t q = 0; q < nnew; q++) {
      if (bs.hzA[q] == b) j1 = q;
      if (bs.hzB[q] == a) j2 = q;
    }
    h.nbr[4 * (size_t)(nf + j) + 1] = nf + j1;
    h.nbr[4 * (size_t)(nf + j) + 2] = nf + j2;
  }
  for (uint32_t i = lane; i < n; i += 32) h.F[16 * (size_t)bs.f[i]] &= 0x7fffffffu;
  if (lane == 0) {
    hs.newBase = nf;
    hs.nf = nf + nnew;
    hs.nalive = nalive + nnew - n;
    hs.nvis = n;
  }
  __syncwarp();
  return true;
}

// a candidate's new owner: over every face after a compaction (patch walk),
// else over the new faces when its owner died
// (best_face over the new faces, the first BIG_NREC read from shared memory
// when nrec is given)
__device__ __noinline__ void slot_reassign(const HullCtx& h, uint32_t i, uint32_t own, bool gone, bool compacted,
                                           uint32_t newBase, uint32_t nfNow, const uint4 (*nrec)[4], uint32_t& outF,
                                           float& outD) {
  if (compacted) {
    patch_best(h, i, own, gone, newBase, nfNow, outF, outD);
    return;
  }
  const f3 pt = h.qvert(i);
  uint32_t bestF = CUACD_NONE;
  float bestD = 0.0f;
  for (uint32_t f = newBase; f < nfNow; f++) {
    const uint32_t j = f - newBase;
    const bool sh = nrec != nullptr && j < BIG_NREC;
    const uint4* w = sh ? nrec[j] : h.rec(f);
    const uint4 w0 = w[0];
    if ((w0.x & ALIVE) == 0) continue;
    const uint4 w2 = w[2];
    const float dd = h.face_filter(w0, w[1], w2, pt, i);
    if (dd > bestD) { bestD = dd; bestF = f; }
    if (dd == 0.0f && bestF == CUACD_NONE && h.face_exact(w2, w[3], pt)) { bestD = 1e-30f; bestF = f; }
  }
  outF = bestF;
  outD = bestD;
}

__device__ __forceinline__ unsigned long long cand_key(float d, uint32_t i) {
  return ((unsigned long long)__float_as_uint(d) << 32) | (unsigned long long)(0xffffffffu - i);
}
// a thread's two largest candidate keys (0 = none) with slots and owners
struct Top2 {
  unsigned long long k1, k2;
  uint32_t s1, o1, s2, o2;
  __device__ __forceinline__ void clear() {
    k1 = k2 = 0;
    s1 = o1 = s2 = o2 = 0;
  }
  __device__ __forceinline__ void add(unsigned long long k, uint32_t s, uint32_t o) {
    if (k <= k2) return;
    if (k > k1) {
      k2 = k1; s2 = s1; o2 = o1;
      k1 = k; s1 = s; o1 = o;
    } else {
      k2 = k; s2 = s; o2 = o;
    }
  }
};
// every thread of the block: the warp's largest keys from its threads' two
// largest, in descending order, for as long as the order is certain (once a
// thread's second key is taken its third could come next, and keys below
// the BAT_LIST-th may be missing: the list is marked truncated), and the
// warp's count of dead slots
template <int NW>
__device__ __forceinline__ void top2_publish(BatSm<NW>& B, const Top2& t, uint32_t dead) {
  const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long cur = t.k1;
  bool first = true;
  uint32_t n = 0, trunc = 1;
  const uint32_t dn = warp_sum_u(dead);
  for (; n < BAT_LIST; n++) {
    // the largest key: high words, then low words among the lanes holding
    // the largest high word (a live key has a nonzero high word)
    const uint32_t hi = __reduce_max_sync(FULLMASK, (uint32_t)(cur >> 32));
    if (hi == 0) {
      trunc = 0;
      break;
    }
    const uint32_t lo = __reduce_max_sync(FULLMASK, (uint32_t)(cur >> 32) == hi ? (uint32_t)cur : 0u);
    const unsigned long long m = ((unsigned long long)hi << 32) | lo;
    bool sec = false;
    if (cur == m) {
      B.wk[w][n] = m;
      B.ws[w][n] = first ? t.s1 : t.s2;
      B.wo[w][n] = first ? t.o1 : t.o2;
      sec = !first;
      cur = first ? t.k2 : 0ull;
      first = false;
    }
    if (__any_sync(FULLMASK, sec)) {
      n++;
      break;
    }
  }
  if (lane == 0) {
    B.wn[w] = n;
    B.wt[w] = trunc;
    B.wdead[w] = dn;
  }
}

// warp 0: the block's largest keys in descending order, at most kmax, by
// merging the warps' lists (lane w holds list w's next key). Every key of a
// warp above the last key of its truncated list is in the list, so the
// merge stops after taking such a last key; and the total of the dead-slot
// counts
template <int NW>
__device__ __noinline__ void bat_select(BatSm<NW>& B, uint32_t kmax) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t wn = lane < NW ? B.wn[lane] : 0u;
  const bool wt = lane < NW && B.wt[lane] != 0;
  const uint32_t dn = warp_sum_u(lane < NW ? B.wdead[lane] : 0u);
  uint32_t pos = 0;
  unsigned long long cur = wn > 0 ? B.wk[lane][0] : 0ull;
  uint32_t n = 0;
  while (n < kmax) {
    const uint32_t hi = __reduce_max_sync(FULLMASK, (uint32_t)(cur >> 32));
    if (hi == 0) break;
    const uint32_t lo = __reduce_max_sync(FULLMASK, (uint32_t)(cur >> 32) == hi ? (uint32_t)cur : 0u);
    const unsigned long long m = ((unsigned long long)hi << 32) | lo;
    bool stop = false;
    if (cur == m) {
      B.selKey[n] = m;
      B.selSlot[n] = B.ws[lane][pos];
      B.selOwn[n] = B.wo[lane][pos];
      pos++;
      stop = pos == wn && wt;
      cur = pos < wn ? B.wk[lane][pos] : 0ull;
    }
    n++;
    if (__any_sync(FULLMASK, stop)) break;
  }
  if (lane == 0) {
    B.nsel = n;
    B.totDead = dn;
  }
  __syncwarp();
}

// one warp: the visible patch of point pIdx on the current hull, walked
// from its owner face `start` as big_insert walks it, in slot order, and
// its horizon edges in the insertion's order (e = 3 * listPos + k); the
// patch's faces also go into the block's set with the warp's bit. W.ok = 0
// when the patch has more than BAT_FACES faces.
template <int NW>
__device__ __noinline__ void bat_walk(const HullCtx& h, uint32_t nf, BatSm<NW>& B, uint32_t pIdx, uint32_t start) {
  constexpr uint32_t HB = BAT_HASH_BITS;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BatWalk& W = B.u.w[warp];
  const uint32_t lt = lanemask_lt();
  const f3 p = h.qvert(pIdx);
  for (uint32_t j = lane; j < (1u << HB); j += 32) W.key[j] = 0;
  __syncwarp();
  if (lane == 0) {
    uint32_t at;
    tab_add<HB>(W.key, start, at);
    W.f[0] = start;
    const uint4 w0 = h.rec(start)[0];
    const uint4 nb = *reinterpret_cast<const uint4*>(h.nbr + 4 * (size_t)start);
    W.vabc[0][0] = w0.x & 0x7fffffffu; W.vabc[0][1] = w0.y; W.vabc[0][2] = w0.z;
    W.nb[0][0] = nb.x; W.nb[0][1] = nb.y; W.nb[0][2] = nb.z;
  }
  __syncwarp();
  uint32_t head = 0, qn = 1;
  bool bad = false;
  for (;;) {
    const uint32_t tasks = 3 * (qn - head);
    uint32_t added = 0;
    bool over = false;
    for (uint32_t t0 = 0; t0 < tasks; t0 += 32) {
      const uint32_t t = t0 + lane;
      bool claimed = false;
      uint32_t g = 0;
      uint4 w0 = make_uint4(0, 0, 0, 0), nb = w0;
      if (t < tasks) {
        g = W.nb[head + t / 3][t % 3];
        if (g < nf && !tab_has<HB>(W.key, g)) {
          const uint4* r = h.rec(g);
          w0 = r[0];
          const uint4 w1 = r[1], w2 = r[2];
          nb = *reinterpret_cast<const uint4*>(h.nbr + 4 * (size_t)g);
          if (w0.x & ALIVE) {
            const float v = h.face_filter(w0, w1, w2, p, pIdx);
            if (v > 0.0f || (v == 0.0f && h.face_exact(w2, r[3], p))) {
              uint32_t at;
              const uint32_t rr = tab_add<HB>(W.key, g, at);
              claimed = rr == 1;
              over = rr == 2;
            }
          }
        }
      }
      const unsigned m = __ballot_sync(FULLMASK, claimed);
      const uint32_t at = qn + added + __popc(m & lt);
      if (claimed && at < BAT_FACES) {
        W.f[at] = g;
        W.vabc[at][0] = w0.x & 0x7fffffffu; W.vabc[at][1] = w0.y; W.vabc[at][2] = w0.z;
        W.nb[at][0] = nb.x; W.nb[at][1] = nb.y; W.nb[at][2] = nb.z;
      }
      added += __popc(m);
    }
    __syncwarp();
    head = qn;
    qn += added;
    if (__any_sync(FULLMASK, over) || qn > BAT_FACES) {
      bad = true;
      break;
    }
    if (head == qn) break;
  }
  if (bad) {
    if (lane == 0) W.ok = 0;
    __syncwarp();
    return;
  }
  const uint32_t n = qn;
  if (lane < n) {
    const uint32_t fi = W.f[lane];
    uint32_t r = 0;
    for (uint32_t j = 0; j < n; j++) r += W.f[j] < fi ? 1u : 0u;
    W.ord[r] = lane;
    btab_add(B, fi, 1u << warp);
  }
  __syncwarp();
  uint32_t nnew = 0;
  for (uint32_t c = 0; c * 32 < 3 * n; c++) {
    const uint32_t e = c * 32 + lane;
    bool isNew = false;
    uint32_t a = 0, b = 0, f = 0, twin = 0;
    if (e < 3 * n) {
      const uint32_t vi = W.ord[e / 3], k = e % 3;
      f = W.f[vi];
      twin = W.nb[vi][k];
      if (twin >= nf || !tab_has<HB>(W.key, twin)) {
        isNew = true;
        a = W.vabc[vi][k];
        b = W.vabc[vi][k == 2 ? 0 : k + 1];
      }
    }
    const unsigned m = __ballot_sync(FULLMASK, isNew);
    const uint32_t q = nnew + __popc(m & lt);
    if (isNew && q < BAT_NEW) {
      W.hA[q] = a; W.hB[q] = b;
      W.tw[q] = twin; W.df[q] = f;
    }
    nnew += __popc(m);
  }
  if (lane == 0) {
    W.n = n;
    W.nnew = nnew;
    W.ok = nnew <= BAT_NEW ? 1u : 0u;
    W.pick = pIdx;
  }
  __syncwarp();
}

// warp j < K: whether patch j meets an earlier walked patch (a face of
// patch j, or a face across one of its edges, was claimed by a walk i < j);
// the round's counters are reset
template <int NW>
__device__ __noinline__ void bat_conflicts(BatSm<NW>& B, uint32_t K) {
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) B.ntodo = 0;
  if (threadIdx.x < NW) B.maxOrph[threadIdx.x] = 0;
  if (warp >= K) return;
  const BatWalk& W = B.u.w[warp];
  const uint32_t below = (1u << warp) - 1u;
  bool hit = false;
  if (W.ok && lane < W.n) {
    const uint32_t g[4] = {W.f[lane], W.nb[lane][0], W.nb[lane][1], W.nb[lane][2]};
#pragma unroll
    for (int k = 0; k < 4; k++) hit = hit || (btab_mask(B, g[k]) & below) != 0;
  }
  hit = __any_sync(FULLMASK, hit);
  if (lane == 0) B.cf[warp] = hit ? 1u : 0u;
}

// every thread: the number of accepted steps ms, the longest prefix of the
// walked picks whose patches are whole, disjoint and not adjacent, with
// neither the compaction rule (steps after the first) nor the slot limit
// firing; *base = the first new-face slot of the thread's warp's step.
// Thread 0 stores the slot and alive counts before each step.
template <int NW>
__device__ __noinline__ uint32_t bat_prefix(const HullCtx& h, const HullSm& hs, BatSm<NW>& B, uint32_t K,
                                            uint32_t* base) {
  const uint32_t warp = threadIdx.x >> 5;
  uint32_t nfc = hs.nf, nalc = hs.nalive, ms = 0;
  *base = nfc;
  for (uint32_t j = 0; j < K; j++) {
    const BatWalk& W = B.u.w[j];
    if (!W.ok || B.cf[j]) break;
    if (j > 0 && (nfc + 3 * HULL_VIS_MAX > h.fmax || nfc > 2 * nalc + 512)) break;
    if (nfc + 3 * W.n > h.fmax) break;
    if (threadIdx.x == 0) {
      B.nfj[j] = nfc;
      B.nalj[j] = nalc;
    }
    if (j == warp) *base = nfc;
    nfc += W.nnew;
    nalc = nalc + W.nnew - W.n;
    ms = j + 1;
  }
  if (threadIdx.x == 0) {
    B.nfj[ms] = nfc;
    B.nalj[ms] = nalc;
  }
  return ms;
}

// squeeze dead slots out of the candidate list (slot order kept); returns
// the new count and publishes the threads' keys
template <int NW>
__device__ __noinline__ uint32_t big_squeeze(const HullCtx& h, GrpSmem& sm, BatSm<NW>& B, uint32_t ncand) {
  constexpr int G = 32 * NW;
  const uint32_t lid = threadIdx.x;
  uint32_t nc = 0;
  Top2 t;
  t.clear();
  for (uint32_t c = 0; c * G < ncand; c++) {
    const uint32_t k = c * G + lid;
    uint32_t o = CUACD_NONE, i = 0;
    float d = 0.0f;
    if (k < ncand) {
      o = h.owner[k];
      i = h.cand[k];
      d = h.dist[k];
    }
    uint32_t tot;
    const uint32_t pre = grp_scan_bit<G>(o != CUACD_NONE, &tot, sm);
    __syncthreads();
    if (o != CUACD_NONE) {
      const uint32_t at = nc + pre;
      h.cand[at] = i;
      h.owner[at] = o;
      h.dist[at] = d;
      t.add(cand_key(d, i), at, o);
    }
    nc += tot;
    __syncthreads();
  }
  top2_publish(B, t, 0);
  __syncthreads();
  return nc;
}

// the single-pick step for the selection's first pick: hull_insert's
// compaction by the whole block, big_insert (hull_insert for a patch above
// BIG_VIS faces) by warp 0, then one pass over the candidate slots: the
// inserted point leaves, points of dead faces (all points after a
// compaction) are reassigned, and the threads' keys are published
template <int NW>
__device__ __noinline__ void big_seq_step(const HullCtx& h, HullSm& hs, GrpSmem& sm, BatSm<NW>& B, uint32_t ncand) {
  constexpr int G = 32 * NW;
  BigSm& bs = B.u.big;
  const uint32_t lid = threadIdx.x;
  uint32_t* cown = h.owner;
  float* cdist = h.dist;
  const uint32_t pick = 0xffffffffu - (uint32_t)(B.selKey[0] & 0xffffffffu);
  const uint32_t pickSlot = B.selSlot[0];
  uint32_t start = B.selOwn[0];
  {
    if (lid == 0) {
      hs.compacted = 0;
      hs.remapN = 0;
      bs.ntodo = 0;
    }
    __syncthreads();
    if (hs.nf + 3 * HULL_VIS_MAX > h.fmax || hs.nf > 2 * hs.nalive + 512) {
      start = hull_compact<G>(h, hs, sm, start, cown, ncand);
    }
    if (threadIdx.x < 32) {
      const bool fast = big_insert(h, hs, bs, pick, start);
      if (!fast) hull_insert<32>(h, hs, sm, pick, start);
      if (threadIdx.x == 0) bs.fast = fast ? 1u : 0u;
    }
    __syncthreads();
    if (hs.fail) return;
    const uint32_t nfNow = hs.nf, newBase = hs.newBase;
    const bool compacted = hs.compacted != 0, fast = bs.fast != 0;
    Top2 top;
    top.clear();
    uint32_t dead = 0;
    bool sweep = compacted;
    if (!compacted) {
      // scan, four slots per thread in flight; the slots whose owner died
      // are listed (in the walk queue's words, free after an insertion) and
      // reassigned by the whole block afterwards
      uint32_t* todo = h.q;
      for (uint32_t k0 = lid; k0 < ncand; k0 += 4 * G) {
        uint32_t ow[4], ci[4];
        float cd[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const uint32_t k = k0 + u * G;
          const bool in = k < ncand;
          ow[u] = in ? cown[k] : CUACD_NONE;
          ci[u] = in ? h.cand[k] : 0u;
          cd[u] = in ? cdist[k] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const uint32_t k = k0 + u * G;
          if (k >= ncand) break;
          const uint32_t own = ow[u];
          if (own == CUACD_NONE) {
            dead++;
            continue;
          }
          if (k == pickSlot) {
            cown[k] = CUACD_NONE;
            dead++;
            continue;
          }
          if (fast ? big_has(bs, own) : bm_test(h.bm, own)) {
            const uint32_t t = atomicAdd(&bs.ntodo, 1u);
            if (t < HULL_VIS_MAX) todo[t] = k;
            continue;
          }
          const unsigned long long key = cand_key(cd[u], ci[u]);
          top.add(key, k, own);
        }
      }
      __syncthreads();
      const uint32_t nt = bs.ntodo;
      for (uint32_t t = lid; t < min(nt, HULL_VIS_MAX); t += G) {
        const uint32_t k = todo[t], i = h.cand[k];
        uint32_t own;
        float d;
        slot_reassign(h, i, cown[k], true, false, newBase, nfNow, fast ? bs.nrec : nullptr, own, d);
        cown[k] = own;
        cdist[k] = d;
        if (own == CUACD_NONE) {
          dead++;
        } else {
          const unsigned long long key = cand_key(d, i);
          top.add(key, k, own);
        }
      }
      // more than the list holds: the rest is found by a sweep
      sweep = nt > HULL_VIS_MAX;
      __syncthreads();
    }
    if (sweep) {
      for (uint32_t k = lid; k < ncand; k += G) {
        uint32_t own = cown[k];
        if (own == CUACD_NONE) {
          if (compacted) dead++;
          continue;
        }
        if (compacted && k == pickSlot) {
          cown[k] = CUACD_NONE;
          dead++;
          continue;
        }
        const bool gone = fast ? big_has(bs, own) : bm_test(h.bm, own);
        if (!compacted && !gone) continue;
        const uint32_t i = h.cand[k];
        float d;
        slot_reassign(h, i, own, gone, compacted, newBase, nfNow, fast ? bs.nrec : nullptr, own, d);
        cown[k] = own;
        cdist[k] = d;
        if (own == CUACD_NONE) {
          dead++;
        } else {
          const unsigned long long key = cand_key(d, i);
          top.add(key, k, own);
        }
      }
    }
    __syncthreads();
    if (!fast) {
      for (uint32_t vi = lid; vi < hs.nvis; vi += G) h.bm[h.vis[vi] >> 5] = 0;
    }
    top2_publish(B, top, dead);
    __syncthreads();
  }
}

// best_face over the new faces [f0, f1) of one step (all alive), the first
// NRC records read from shared memory
template <uint32_t NRC>
__device__ __forceinline__ void bat_best(const HullCtx& h, uint32_t i, uint32_t f0, uint32_t f1, const uint4 (*nrc)[3],
                                         uint32_t& outF, float& outD) {
  const f3 pt = h.qvert(i);
  uint32_t bestF = CUACD_NONE;
  float bestD = 0.0f;
  for (uint32_t f = f0; f < f1; f++) {
    const uint32_t q = f - f0;
    uint4 w0, w1, w2;
    if (q < NRC) {
      w0 = nrc[q][0]; w1 = nrc[q][1]; w2 = nrc[q][2];
    } else {
      const uint4* w = h.rec(f);
      w0 = w[0]; w1 = w[1]; w2 = w[2];
    }
    const float dd = h.face_filter(w0, w1, w2, pt, i);
    if (dd > bestD) { bestD = dd; bestF = f; }
    if (dd == 0.0f && bestF == CUACD_NONE && h.face_exact(w2, h.rec(f)[3], pt)) { bestD = 1e-30f; bestF = f; }
  }
  outF = bestF;
  outD = bestD;
}

// A batched round after validation (ms >= 1 steps): the new faces of every
// validated step at their slots while one pass over the candidate slots
// lists the orphans of the validated patches (six words each in the
// visible list's and walk queue's words: slot, point, owner, then new
// owner, new distance, step), the orphans' new owners over their step's
// new faces and the largest new key per step, the accepted prefix, then its
// commit (twin links, dead faces, counts) and the orphans' new owners.
// Returns the number of insertions.
template <int NW>
__device__ __noinline__ uint32_t bat_step(const HullCtx& h, HullSm& hs, BatSm<NW>& B, uint32_t ncand, uint32_t ms,
                                          uint32_t myBase) {
  constexpr int G = 32 * NW;
  constexpr uint32_t NRC = BatSm<NW>::NRC;
  const uint32_t lid = threadIdx.x, warp = lid >> 5, lane = lid & 31;
  const uint32_t nf0 = hs.nf;
  uint32_t* tK = h.vis;
  uint32_t* tI = h.vis + TODO_CAP;
  uint32_t* tO = h.vis + 2 * TODO_CAP;
  uint32_t* tNO = h.q;
  uint32_t* tND = h.q + TODO_CAP;
  uint32_t* tJ = h.q + 2 * TODO_CAP;
  // new faces (a, b, pick) and the links among them and to the twins;
  // records of steps that are not accepted lie above the slot count and
  // are overwritten later
  if (warp < ms) {
    const BatWalk& W = B.u.w[warp];
    const uint32_t base = myBase, nnew = W.nnew, pIdx = W.pick;
    const f3 p = h.qvert(pIdx);
    for (uint32_t q = lane; q < nnew; q += 32) {
      const uint32_t a = W.hA[q], b = W.hB[q], s = base + q;
      uint4 w0, w1, w2, w3;
      h.face_make_q(a, b, pIdx, p, w0, w1, w2, w3);
      uint4* w = h.rec(s);
      w[0] = w0; w[1] = w1; w[2] = w2; w[3] = w3;
      if (q < NRC) {
        B.nrc[warp][q][0] = w0; B.nrc[warp][q][1] = w1; B.nrc[warp][q][2] = w2;
      }
      // around the horizon loop: (b, p) borders the new face starting at
      // b, (p, a) the new face ending at a
      uint32_t j1 = 0, j2 = 0;
      for (uint32_t r = 0; r < nnew; r++) {
        if (W.hA[r] == b) j1 = r;
        if (W.hB[r] == a) j2 = r;
      }
      uint32_t* nq = h.nbr + 4 * (size_t)s;
      nq[0] = W.tw[q];
      nq[1] = base + j1;
      nq[2] = base + j2;
    }
  }
  // one pass over the slots, SCAN_U per thread in flight
  Top2 top;
  top.clear();
  uint32_t dead = 0;
  for (uint32_t k0 = lid; k0 < ncand; k0 += SCAN_U * G) {
    uint32_t ow[SCAN_U], ci[SCAN_U];
    float cd[SCAN_U];
#pragma unroll
    for (int u = 0; u < SCAN_U; u++) {
      const uint32_t k = k0 + u * G;
      const bool in = k < ncand;
      ow[u] = in ? h.owner[k] : CUACD_NONE;
      ci[u] = in ? h.cand[k] : 0u;
      cd[u] = in ? h.dist[k] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < SCAN_U; u++) {
      const uint32_t k = k0 + u * G;
      if (k >= ncand) break;
      const uint32_t own = ow[u];
      if (own == CUACD_NONE) {
        dead++;
        continue;
      }
      // the first walk holding the owner: an earlier step's patch when two
      // hold it, and then only that step can be accepted
      const uint32_t j = __ffs(btab_mask(B, own)) - 1u;
      if (j < ms) {
        const uint32_t t = atomicAdd(&B.ntodo, 1u);
        if (t < TODO_CAP) {
          tK[t] = k;
          tI[t] = ci[u];
          tO[t] = own;
          tJ[t] = j;
        }
        continue;
      }
      top.add(cand_key(cd[u], ci[u]), k, own);
    }
  }
  __syncthreads();
  const uint32_t nt = B.ntodo;
  uint32_t m = 1;
  if (nt <= TODO_CAP) {
    for (uint32_t t = lid; t < nt; t += G) {
      const uint32_t k = tK[t], i = tI[t], j = tJ[t];
      uint32_t no = CUACD_NONE;
      float nd = 0.0f;
      if (k != B.selSlot[j]) {
        bat_best<NRC>(h, i, B.nfj[j], B.nfj[j + 1], B.nrc[j], no, nd);
        if (no != CUACD_NONE) atomicMax(&B.maxOrph[j], cand_key(nd, i));
      }
      tNO[t] = no;
      tND[t] = __float_as_uint(nd);
    }
    __syncthreads();
    // pick j is next while every earlier step's orphans stay below its key
    unsigned long long run = B.maxOrph[0];
    for (uint32_t j = 1; j < ms; j++) {
      if (!(run < B.selKey[j])) break;
      run = B.maxOrph[j] > run ? B.maxOrph[j] : run;
      m++;
    }
  }
  // commit: the twins link to the new faces, the patches die
  if (warp < m) {
    const BatWalk& W = B.u.w[warp];
    const uint32_t base = B.nfj[warp];
    for (uint32_t q = lane; q < W.nnew; q += 32) {
      const uint32_t twin = W.tw[q], f = W.df[q], s = base + q;
      if (twin < nf0) {
        uint32_t* tq = h.nbr + 4 * (size_t)twin;
        const uint4 tn = *reinterpret_cast<const uint4*>(tq);
        if (tn.x == f) tq[0] = s;
        if (tn.y == f) tq[1] = s;
        if (tn.z == f) tq[2] = s;
      }
    }
    for (uint32_t i = lane; i < W.n; i += 32) h.F[16 * (size_t)W.f[i]] &= 0x7fffffffu;
  }
  if (lid == 0) {
    hs.newBase = nf0;
    hs.nf = B.nfj[m];
    hs.nalive = B.nalj[m];
  }
  if (nt <= TODO_CAP) {
    // accepted steps' orphans take their new owners (the picks leave);
    // the others keep theirs
    for (uint32_t t = lid; t < nt; t += G) {
      const uint32_t k = tK[t], i = tI[t], j = tJ[t];
      if (j < m) {
        const uint32_t no = tNO[t];
        const float nd = __uint_as_float(tND[t]);
        h.owner[k] = no;
        h.dist[k] = nd;
        if (no == CUACD_NONE) dead++;
        else top.add(cand_key(nd, i), k, no);
      } else {
        top.add(cand_key(h.dist[k], i), k, tO[t]);
      }
    }
  } else {
    // more orphans than the list holds: the first step alone, its orphans
    // reassigned by a sweep
    for (uint32_t k = lid; k < ncand; k += G) {
      const uint32_t own = h.owner[k];
      if (own == CUACD_NONE) continue;
      const uint32_t j = __ffs(btab_mask(B, own)) - 1u;
      if (j >= ms) continue;
      const uint32_t i = h.cand[k];
      if (j != 0) {
        top.add(cand_key(h.dist[k], i), k, own);
        continue;
      }
      uint32_t no = CUACD_NONE;
      float nd = 0.0f;
      if (k != B.selSlot[0]) bat_best<NRC>(h, i, B.nfj[0], B.nfj[1], B.nrc[0], no, nd);
      h.owner[k] = no;
      h.dist[k] = nd;
      if (no == CUACD_NONE) dead++;
      else top.add(cand_key(nd, i), k, no);
    }
  }
  top2_publish(B, top, dead);
  __syncthreads();
  return m;
}

template <int NW>
__device__ __noinline__ uint32_t hull_grow_big(const HullCtx& h, HullSm& hs, GrpSmem& sm, BatSm<NW>& B,
                                               uint32_t maxIter) {
  constexpr int G = 32 * NW;
  const uint32_t lid = threadIdx.x, warp = lid >> 5;
  uint32_t ncand = hs.ncand;
  // owner and distance to candidate-slot order, in place: each chunk is read
  // before it is written, and a later chunk reads only points cand[k] >= k
  // (the assignment pass lists points in index order; the seed list fits
  // one chunk)
  Top2 top;
  top.clear();
  uint32_t dead = 0;
  for (uint32_t c = 0; c * G < ncand; c++) {
    const uint32_t k = c * G + lid;
    uint32_t o = CUACD_NONE, i = 0;
    float d = 0.0f;
    if (k < ncand) {
      i = h.cand[k];
      o = h.owner[i];
      d = h.dist[i];
    }
    __syncthreads();
    if (k < ncand) {
      h.owner[k] = o;
      h.dist[k] = d;
      if (o != CUACD_NONE) top.add(cand_key(d, i), k, o);
      else dead++;
    }
    __syncthreads();
  }
  top2_publish(B, top, dead);
  __syncthreads();
  uint32_t nIns = 0;
  while (nIns < maxIter) {
    for (uint32_t e = lid; e < (1u << BatSm<NW>::BLK_BITS); e += G) B.btab[e] = make_uint2(0u, 0u);
    if (warp == 0) bat_select(B, min(BatDims<NW>::KMAX, maxIter - nIns));
    __syncthreads();
    // squeeze dead slots out when they pass 1 / SQZ_DIV of the list
    if (SQZ_DIV * B.totDead > ncand) {
      ncand = big_squeeze(h, sm, B, ncand);
      continue;
    }
    const uint32_t K = B.nsel;
    if (K == 0) break;
    uint32_t ms = 0, myBase = 0;
    if (hs.nf + 3 * HULL_VIS_MAX <= h.fmax && hs.nf <= 2 * hs.nalive + 512) {
      if (warp < K) bat_walk(h, hs.nf, B, 0xffffffffu - (uint32_t)(B.selKey[warp] & 0xffffffffu), B.selOwn[warp]);
      __syncthreads();
      bat_conflicts(B, K);
      __syncthreads();
      // the same on every thread; the slot pass reads the block's set of
      // claimed faces, which no thread writes until the next round
      ms = bat_prefix(h, hs, B, K, &myBase);
    }
    if (ms == 0) {
      // the single-pick step's shared words overlay the walks' words
      __syncthreads();
      big_seq_step(h, hs, sm, B, ncand);
      nIns++;
      if (hs.fail) break;
    } else {
      nIns += bat_step(h, hs, B, ncand, ms, myBase);
    }
  }
  if (lid == 0) hs.ncand = ncand;
  __syncthreads();
  return nIns;
}

// Every point against the face slots [0, nf) (shaders.ts:1332-1354): owner =
// the first slot of largest positive ranking value, candidates = the points
// with an owner, in index order. Each thread holds up to ASSIGN_K points in
// registers and the slots are read once per ASSIGN_K * G points, the next
// slot's record loading while the current one is evaluated. Warp groups
// hold one point per thread: their kernel is limited by instruction fetch,
// and the smaller loop measured 4 % faster on the staircase tree than two.
template <int G>
__device__ __noinline__ uint32_t hull_assign_all(const HullCtx& h, GrpSmem& sm, uint32_t nf) {
  constexpr int ASSIGN_K = G == 32 ? 1 : 2;
  const int lid = Grp<G>::lid();
  const uint32_t nv = h.nv;
  uint32_t ncand = 0;
  for (uint32_t base = 0; base < nv; base += ASSIGN_K * G) {
    f3 p[ASSIGN_K];
    float bd[ASSIGN_K];
    uint32_t bo[ASSIGN_K];
#pragma unroll
    for (int k = 0; k < ASSIGN_K; k++) {
      const uint32_t i = base + k * G + lid;
      p[k] = h.qvert(i < nv ? i : 0u);
      bd[k] = 0.0f;
      bo[k] = CUACD_NONE;
    }
    uint4 n0 = nf > 0 ? h.rec(0)[0] : make_uint4(0, 0, 0, 0);
    for (uint32_t f = 0; f < nf; f++) {
      const uint4 w0 = n0;
      if (f + 1 < nf) n0 = h.rec(f + 1)[0];
      if ((w0.x & ALIVE) == 0) continue;
      const uint4* w = h.rec(f);
      const uint4 w1 = w[1], w2 = w[2];
#pragma unroll
      for (int k = 0; k < ASSIGN_K; k++) {
        if (base + k * G < nv) {
          const float dd = h.face_filter(w0, w1, w2, p[k], base + k * G + lid);
          if (dd > bd[k]) { bd[k] = dd; bo[k] = f; }
          // an exact-visible face ranks 1e-30, below every filtered value:
          // it only matters while the point has no owner
          if (dd == 0.0f && bo[k] == CUACD_NONE && h.face_exact(w2, w[3], p[k])) { bd[k] = 1e-30f; bo[k] = f; }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < ASSIGN_K; k++) {
      if (base + k * G < nv) {
        const uint32_t i = base + k * G + lid;
        const bool outside = i < nv && bo[k] != CUACD_NONE;
        if (i < nv) {
          h.owner[i] = bo[k];
          h.dist[i] = bd[k];
        }
        uint32_t tot;
        const uint32_t pre = grp_scan_bit<G>(outside, &tot, sm);
        if (outside) h.cand[ncand + pre] = i;
        ncand += tot;
      }
    }
  }
  return ncand;
}

// exact volume of the alive faces, in grid units
template <int G>
__device__ __noinline__ double hull_volume_grid(const HullCtx& h, HullSm& hs, GrpSmem& sm) {
  const int lid = Grp<G>::lid();
  uint32_t a0, b0, c0;
  h.abc(0, a0, b0, c0);
  const f3 of = h.qvert(a0);
  const long long ox = (long long)of.x, oy = (long long)of.y, oz = (long long)of.z;
  __int128 v6 = 0;
  const uint32_t nf = hs.nf;
  for (uint32_t f = lid; f < nf; f += G) {
    if (!h.alive(f)) continue;
    uint32_t a, b, c;
    h.abc(f, a, b, c);
    f3 pa = h.qvert(a), pb = h.qvert(b), pc = h.qvert(c);
    long long ax = (long long)pa.x - ox, ay = (long long)pa.y - oy, az = (long long)pa.z - oz;
    long long bx = (long long)pb.x - ox, by = (long long)pb.y - oy, bz = (long long)pb.z - oz;
    long long cx = (long long)pc.x - ox, cy = (long long)pc.y - oy, cz = (long long)pc.z - oz;
    long long nx = by * cz - bz * cy, ny = bz * cx - bx * cz, nz = bx * cy - by * cx;
    v6 += (__int128)ax * nx + (__int128)ay * ny + (__int128)az * nz;
  }
  // group sum of the 128-bit partials
  unsigned long long lo = (unsigned long long)v6;
  long long hi = (long long)(v6 >> 64);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long lo2 = __shfl_xor_sync(FULLMASK, lo, o);
    long long hi2 = __shfl_xor_sync(FULLMASK, hi, o);
    __int128 s = ((__int128)hi << 64 | (__int128)lo) + ((__int128)hi2 << 64 | (__int128)lo2);
    lo = (unsigned long long)s;
    hi = (long long)(s >> 64);
  }
  __int128 tot = (__int128)hi << 64 | (__int128)lo;
  if (G > 32) {
    __shared__ unsigned long long vs[G / 32][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) { vs[w][0] = lo; vs[w][1] = (unsigned long long)hi; }
    __syncthreads();
    tot = 0;
    for (int i = 0; i < G / 32; i++) tot += ((__int128)(long long)vs[i][1] << 64) | (__int128)vs[i][0];
    __syncthreads();
  }
  if (tot < 0) tot = -tot;
  long long th = (long long)(tot >> 32);
  uint32_t tl = (uint32_t)(tot & 0xffffffffu);
  return ((double)th * 4294967296.0 + (double)tl) / 6.0;
}

template <int G>
__device__ void hull_one(const Level& P, const Dev& D, uint32_t idx, uint32_t* slab, HullSm& hs, GrpSmem& sm,
                         float* qcache, TinySm* ts, BatSm<(G >= 256 ? G / 32 : 8)>* bs) {
  const int lid = Grp<G>::lid();
  const uint32_t partIdx = P.partBase + idx;
  PartDesc* pdp = D.parts + partIdx;
  const uint32_t nv = pdp->nv, nt = pdp->nt, vOff = pdp->vOff, flags = pdp->flags;
  const float meshVol = pdp->meshVol;
  if (!(nv >= 4 && (nt > 0 || (flags & 2) != 0))) {
    if (lid == 0) pdp->hullVol = 0.0f;
    return;
  }
  const uint32_t fb = (2 * nv + max(nv, 80u) + 7) & ~7u;
  const uint32_t fmax = P.hullSlabWords > fb ? (P.hullSlabWords - fb) / 16 : 0;
  if (fmax < 64) {
    if (lid == 0) { pdp->hullVol = -1.0f; pdp->flags = 3; atomicAdd(D.ctr + CTR_HULLFAIL, 1u); }
    return;
  }
  // the walk's arrays after the reference's slab words must fit the slab
  // (always true for hull_slab_stride; checked so a slab is never overrun)
  if ((uint64_t)P.hullSlabWords + 2 * HULL_VIS_MAX + 4ull * fmax + 2 * ((fmax + 31) / 32) + 2ull * nv > P.slabStride) {
    if (lid == 0) { pdp->hullVol = -1.0f; pdp->flags = 3; atomicAdd(D.ctr + CTR_HULLFAIL, 1u); }
    return;
  }
  if (lid == 0) add_bytes(D.ctr, CTR_BYTES_HULL, 12ull * nv);
  HullCtx h;
  h.qc = nullptr;
  h.V = D.V; h.vOff = vOff; h.nv = nv; h.fmax = fmax;
  h.owner = slab;
  h.dist = reinterpret_cast<float*>(slab + nv);
  h.cand = slab + 2 * nv;
  h.F = slab + fb;
  // after the reference's slab words (which fix fmax): visible list, walk
  // queue, adjacency, bitmap, word prefix, horizon maps (hull_slab_stride)
  h.vis = slab + P.hullSlabWords;
  h.q = h.vis + HULL_VIS_MAX;
  h.nbr = h.q + HULL_VIS_MAX;
  const uint32_t nw = (fmax + 31) / 32;
  h.bm = h.nbr + 4 * (size_t)fmax;
  h.wp = h.bm + nw;
  h.hA = h.wp + nw;
  h.hB = h.hA + nv;
  for (uint32_t w = lid; w < nw; w += G) h.bm[w] = 0;
  // quantisation grid: 2^21 cells across the largest extent
  f3 lo = mk3(1e30f, 1e30f, 1e30f), hi = mk3(-1e30f, -1e30f, -1e30f);
  for (uint32_t i = lid; i < nv; i += G) {
    f3 p = ldv(D.V, (size_t)vOff + 3 * (size_t)i);
    lo = vmin3(lo, p);
    hi = vmax3(hi, p);
  }
  lo.x = grp_min_f<G>(lo.x, sm); lo.y = grp_min_f<G>(lo.y, sm); lo.z = grp_min_f<G>(lo.z, sm);
  hi.x = grp_max_f<G>(hi.x, sm); hi.y = grp_max_f<G>(hi.y, sm); hi.z = grp_max_f<G>(hi.z, sm);
  const f3 ext = hi - lo;
  const float scale = fmaxf(fmaxf(fmaxf(ext.x, ext.y), ext.z), 1e-30f);
  h.qlo = lo;
  h.qs = 2097152.0f / scale;
  const float cell = scale / 2097152.0f;
  const float volScale = (cell * cell) * cell;
  // small parts keep their quantised points in shared memory
  if (G == 32 && qcache != nullptr && nv <= QC_MAX) {
    for (uint32_t i = lid; i < nv; i += G) {
      f3 v = ldv(D.V, (size_t)vOff + 3 * (size_t)i) - lo;
      qcache[3 * i] = rintf(v.x * h.qs);
      qcache[3 * i + 1] = rintf(v.y * h.qs);
      qcache[3 * i + 2] = rintf(v.z * h.qs);
    }
    h.qc = qcache;
    Grp<G>::sync();
  }
  // 80 seeds: max and min along 40 axes, lowest index on ties; seed 2a is
  // the maximum along axis a, seed 2a + 1 the minimum
  if (h.qc != nullptr) {
    // one lane per axis, each scanning every point in index order
    for (uint32_t a = lid; a < 40; a += G) {
      const f3 ax = mk3(c_kdop[a][0], c_kdop[a][1], c_kdop[a][2]);
      float mx = -1e30f, mn = 1e30f;
      uint32_t ix = 0, in = 0;
      for (uint32_t i = 0; i < nv; i++) {
        const float d = dot(ax, h.qvert(i));
        if (d > mx) { mx = d; ix = i; }
        if (d < mn) { mn = d; in = i; }
      }
      hs.seed[2 * a] = ix;
      hs.seed[2 * a + 1] = in;
    }
  } else
  for (int ps = 0; ps < 20; ps++) {
    const f3 a0 = mk3(c_kdop[2 * ps][0], c_kdop[2 * ps][1], c_kdop[2 * ps][2]);
    const f3 a1 = mk3(c_kdop[2 * ps + 1][0], c_kdop[2 * ps + 1][1], c_kdop[2 * ps + 1][2]);
    float mx0 = -1e30f, mx1 = -1e30f, mn0 = -1e30f, mn1 = -1e30f;  // mins stored negated
    uint32_t ix0 = CUACD_NONE, ix1 = CUACD_NONE, in0 = CUACD_NONE, in1 = CUACD_NONE;
    for (uint32_t i = lid; i < nv; i += G) {
      f3 v = h.qvert(i);
      float d0 = dot(a0, v), d1 = dot(a1, v);
      am_merge(mx0, ix0, d0, i);
      am_merge(mn0, in0, -d0, i);
      am_merge(mx1, ix1, d1, i);
      am_merge(mn1, in1, -d1, i);
    }
    grp_argmax<G>(mx0, ix0, sm);
    grp_argmax<G>(mn0, in0, sm);
    grp_argmax<G>(mx1, ix1, sm);
    grp_argmax<G>(mn1, in1, sm);
    if (lid == 0) { hs.seed[4 * ps] = ix0; hs.seed[4 * ps + 1] = in0; hs.seed[4 * ps + 2] = ix1; hs.seed[4 * ps + 3] = in1; }
  }
  Grp<G>::sync();
  if (P.hullStage == 1) {
    if (lid == 0) pdp->hullVol = 0.0f;
    return;
  }
  // the register hull first when the part's points are in shared memory; a
  // hull that outgrows the warp is built again from the simplex in the
  // slot-array form (the same sequence, so the same result)
  bool tiny = G == 32 && ts != nullptr && h.qc != nullptr;
restart:
  // initial simplex (shaders.ts:1227-1263). The reference scans the 80 seeds
  // serially with strict comparisons, so each choice is the first seed
  // position reaching the maximum: here every lane scans its positions in
  // order and the group argmax breaks ties by the lowest position.
  {
    const uint32_t i0 = hs.seed[1], i1 = hs.seed[0];
    const f3 p0 = h.qvert(i0), p1 = h.qvert(i1);
    const f3 d01 = p1 - p0;
    float best = 0.0f;
    uint32_t bk = CUACD_NONE;
    for (uint32_t k = lid; k < 80; k += G) {
      const f3 c = cross(d01, h.qvert(hs.seed[k]) - p0);
      const float v = dot(c, c);
      if (v > best) { best = v; bk = k; }
    }
    grp_argmax<G>(best, bk, sm);
    uint32_t i3 = CUACD_NONE, i2 = CUACD_NONE;
    int bs = 0;
    if (bk != CUACD_NONE) {
      i2 = hs.seed[bk];
      const f3 e2 = h.qvert(i2) - p0;
      const f3 n = cross(d01, e2);
      float bd = 0.0f;
      uint32_t k3 = CUACD_NONE;
      for (uint32_t k = lid; k < 80; k += G) {
        const f3 dk = h.qvert(hs.seed[k]) - p0;
        const float v = fabsf(dot(n, dk));
        if (v > bd && orient_filtered(n, d01, e2, dk) != 0) { bd = v; k3 = k; }
      }
      grp_argmax<G>(bd, k3, sm);
      if (k3 != CUACD_NONE) {
        i3 = hs.seed[k3];
        bs = orient_filtered(n, d01, e2, h.qvert(i3) - p0);
      }
    }
    if (lid < 4 && i3 != CUACD_NONE) {
      uint32_t a = i0, b = i1, c = i2;
      if (bs > 0) { b = i2; c = i1; }
      if (lid == 0) h.face_write(0, a, b, c);
      if (lid == 1) h.face_write(1, a, i3, b);
      if (lid == 2) h.face_write(2, b, i3, c);
      if (lid == 3) h.face_write(3, c, i3, a);
      // faces across each edge of the tetrahedron
      const uint4 nb[4] = {make_uint4(1, 2, 3, 0), make_uint4(3, 2, 0, 0), make_uint4(1, 3, 0, 0), make_uint4(2, 1, 0, 0)};
      *reinterpret_cast<uint4*>(h.nbr + 4 * lid) = nb[lid];
    }
    if (lid == 0) {
      hs.fail = 0;
      hs.ok = i3 != CUACD_NONE ? 1u : 0u;
      hs.nf = 4;
      hs.nalive = 4;
      hs.remapN = 0;
    }
  }
  Grp<G>::sync();
  if (!hs.ok) {
    if (lid == 0) pdp->hullVol = 0.0f;
    return;
  }
  // seeds first. A point can be the extreme of several axes; its repeats in
  // the list have the same distance and index, so they never change a pick
  // or an owner, and the list keeps first occurrences only.
  uint32_t nuniq = 0;
  for (uint32_t c = 0; c * G < 80; c++) {
    const uint32_t k = c * G + lid;
    bool keep = false;
    uint32_t s = 0;
    if (k < 80) {
      s = hs.seed[k];
      keep = true;
      for (uint32_t j = 0; j < k; j++) if (hs.seed[j] == s) { keep = false; break; }
    }
    uint32_t tot;
    const uint32_t pre = grp_scan_bit<G>(keep, &tot, sm);
    if (keep) h.cand[nuniq + pre] = s;
    nuniq += tot;
  }
  Grp<G>::sync();
  uint32_t nIns;
  bool tinyUsed = false;
  if (tiny && nuniq <= TINY_SEEDS) {
    const uint32_t ci = (uint32_t)lid < nuniq ? h.cand[lid] : 0u;
    if (lid == 0) hs.nfRef = 4;
    __syncwarp();
    nIns = hull_tiny_grow(h, hs, *ts, 80, ci, CUACD_NONE, 0.0f, nuniq);
    if (nIns == CUACD_NONE) {
      tiny = false;
      goto restart;
    }
    tinyUsed = true;
  } else if (G == 32 && nuniq <= 32) {
    uint32_t ci = 0, co = CUACD_NONE;
    float cd = 0.0f;
    if ((uint32_t)lid < nuniq) {
      ci = h.cand[lid];
      h.best_face(ci, 0, 4, co, cd);
    }
    nIns = hull_grow_lanes(h, hs, sm, 4, 80, ci, co, cd);
  } else {
    for (uint32_t k = lid; k < nuniq; k += G) h.assign(h.cand[k], 0, 4);
    if (lid == 0) hs.ncand = nuniq;
    Grp<G>::sync();
    if constexpr (G >= 256) nIns = hull_grow_big<G / 32>(h, hs, sm, *bs, 80);
    else nIns = hull_grow<G>(h, hs, sm, 4, 80);
  }
  const uint32_t fail0 = hs.fail;
  const uint32_t nfPrev = hs.nf;
  // last-level branch and bound (shaders.ts:1300-1331)
  if (P.lastLevel == 1 && P.level > 0 && P.nSeeds > 0 && P.exportStride == 0 && fail0 == 0) {
    const Job* jb = D.jobs + P.jobBase + idx / 2;
    const ItemDesc* pit = D.items + P.itemsInBase + jb->parentItem;
    float ssum = 0.0f;
    for (uint32_t l = 0; l < pit->nLevels; l++) ssum += pit->levelCosts[l];
    // the seed's best completed-path upper bound (k_seed_bound)
    const float ub = D.ub[pit->srcPart];
    const float vRough = (float)(hull_volume_grid<G>(h, hs, sm) * (double)volScale);
    // bound = ssum + rv_cost(meshVol, vRough) > ub, decided with a float32
    // cube root when it clears the comparison by more than its error (cbrtf
    // and the products are within 1e-6 relative of rv_cost's double form,
    // so a margin of 1e-5 of the operands is safe); the double form, which
    // is slow on this GPU, only runs near the boundary
    const float gapf = fmaxf(vRough - meshVol, 0.0f);
    const float rvf = 0.3f * cbrtf(0.2387324f * gapf);
    const float boundf = ssum + rvf;
    const float margin = 1e-5f * (fabsf(ssum) + rvf + fabsf(meshVol) + fabsf(vRough)) + 1e-30f;
    bool prune;
    if (boundf > ub + margin) prune = true;
    else if (boundf < ub - margin) prune = false;
    else prune = ssum + rv_cost(meshVol, vRough) > ub;
    if (prune) {
      if (lid == 0) {
        pdp->hullVol = vRough;
        pdp->flags = pdp->flags | 4u;
        atomicAdd(D.ctr + CTR_PRUNED, 1u);
      }
      return;
    }
  }
  // every point against the rough hull; candidates = points outside it
  const uint32_t ncand = fail0 == 0 ? hull_assign_all<G>(h, sm, nfPrev) : 0u;
  if (lid == 0) {
    hs.ncand = ncand;
    if (P.exportStride == 0) pdp->pad0 = ncand;
  }
  Grp<G>::sync();
  const uint32_t maxIter = (P.hullStage == 2 || P.hullStage == 3 || fail0 != 0) ? 0 : nv;
  if (tinyUsed && fail0 == 0) {
    if (ncand > 32) {
      tiny = false;
      goto restart;
    }
    uint32_t ci = 0, co = CUACD_NONE;
    float cd = 0.0f;
    if ((uint32_t)lid < ncand) {
      ci = h.cand[lid];
      co = h.owner[ci];
      cd = h.dist[ci];
    }
    const uint32_t n2 = hull_tiny_grow(h, hs, *ts, maxIter, ci, co, cd, 0u);
    if (n2 == CUACD_NONE) {
      tiny = false;
      goto restart;
    }
    nIns += n2;
  } else if (G == 32 && ncand <= 32) {
    uint32_t ci = 0, co = CUACD_NONE;
    float cd = 0.0f;
    if ((uint32_t)lid < ncand) {
      ci = h.cand[lid];
      co = h.owner[ci];
      cd = h.dist[ci];
    }
    nIns += hull_grow_lanes(h, hs, sm, nfPrev, maxIter, ci, co, cd);
  } else {
    if constexpr (G >= 256) nIns += hull_grow_big<G / 32>(h, hs, sm, *bs, maxIter);
    else nIns += hull_grow<G>(h, hs, sm, nfPrev, maxIter);
  }
  if (hs.fail) {
    if (lid == 0) {
      pdp->hullVol = -1.0f;
      pdp->flags = hs.fail;
      atomicAdd(D.ctr + CTR_HULLFAIL, 1u);
    }
    return;
  }
  const float vol = (float)(hull_volume_grid<G>(h, hs, sm) * (double)volScale);
  if (lid == 0) { pdp->hullVol = vol; pdp->pad1 = nIns; }
  if (P.exportStride != 0) {
    const uint32_t nf = hs.nf;
    uint32_t run = 0;
    const size_t base = (size_t)P.exportBase + (size_t)idx * P.exportStride;
    for (uint32_t c = 0; c * G < nf; c++) {
      const uint32_t f = c * G + lid;
      uint32_t al = 0, a = 0, b = 0, cc = 0;
      if (f < nf && h.alive(f)) { al = 1; h.abc(f, a, b, cc); }
      uint32_t tot;
      uint32_t pre = grp_scan_bit<G>(al != 0, &tot, sm);
      if (al && 3 * (run + pre) + 3 <= P.exportStride) {
        uint32_t* w = D.T + base + 3 * (size_t)(run + pre);
        w[0] = a; w[1] = b; w[2] = cc;
      }
      run += tot;
    }
    if (lid == 0) {
      const uint32_t nx = min(run, P.exportStride / 3);
      pdp->pad0 = nx;
      if (P.hdDescBase != 0) {
        PartDesc hd;
        hd.vOff = vOff; hd.nv = nv; hd.tOff = (uint32_t)base; hd.nt = nx;
        hd.eOff = 0; hd.ne = 0; hd.meshVol = 0.0f; hd.hullVol = vol;
        hd.planeIds[0] = hd.planeIds[1] = hd.planeIds[2] = hd.planeIds[3] = CUACD_NONE;
        hd.nPlanes = 0; hd.flags = 2; hd.pad0 = 0; hd.pad1 = 0;
        D.parts[partIdx + P.hdDescBase] = hd;
      }
    }
  }
}

// Persistent groups: group s owns slab s and takes the launch's parts from a
// counter, so parts of uneven size balance across the GPU. Warps take parts
// with nv <= smallNv, blocks of 256, 512 or 1024 threads the others (the
// widest whose resident blocks hold the level's parts in one wave): the
// block inserts up to one point per warp (at most 16) per round, and its
// width serves the passes over all points and candidates, which grow with nv.
template <int G>
__global__ void __launch_bounds__(G >= 512 ? G : 256, G == 1024 ? 1 : (G == 512 ? 2 : 4))
    k_hull(const Level P, const Dev D) {
  __shared__ GrpSmem gsm[Grp<G>::PER_BLOCK];
  __shared__ HullSm hsm[Grp<G>::PER_BLOCK];
  __shared__ float qcs[G == 32 ? 8 * 3 * QC_MAX : 1];
  __shared__ TinySm tsm[G == 32 ? 8 : 1];
  // the block path's shared words (BatSm) in the launch's dynamic shared memory
  extern __shared__ __align__(16) unsigned char hull_dyn[];
  using BS = BatSm<(G >= 256 ? G / 32 : 8)>;
  const int gi = Grp<G>::gid();
  const uint32_t s = blockIdx.x * Grp<G>::PER_BLOCK + gi;
  if (s >= P.nSlabs) return;
  if (G != 32) {
    // leave at once when the level has no part above smallNv (the scan
    // recorded its largest child)
    const uint32_t mx = P.maxNvHint ? P.maxNvHint : D.work[32 + P.workSlot];
    if (mx <= P.smallNv) return;
  }
  uint32_t* slab = D.slab + (size_t)s * P.slabStride;
  if (G != 32) {
    for (;;) {
      uint32_t idx = 0;
      if (threadIdx.x == 0) idx = atomicAdd(D.work + 16 + P.workSlot, 1u);
      idx = grp_bcast_u<G>(idx, gsm[0]);
      if (idx >= P.nChildParts) break;
      if (D.parts[P.partBase + idx].nv <= P.smallNv) continue;
      hull_one<G>(P, D, idx, slab, hsm[gi], gsm[gi], nullptr, nullptr, reinterpret_cast<BS*>(hull_dyn));
      Grp<G>::sync();
    }
    return;
  }
  {
    // warp groups take the next part from the launch's counter, so parts of
    // uneven size balance across the GPU
    const int lane = threadIdx.x & 31;
    for (;;) {
      uint32_t idx = 0;
      if (lane == 0) idx = atomicAdd(D.work + P.workSlot, 1u);
      idx = __shfl_sync(FULLMASK, idx, 0);
      if (idx >= P.nChildParts) break;
      if (D.parts[P.partBase + idx].nv > P.smallNv) continue;
      hull_one<G>(P, D, idx, slab, hsm[gi], gsm[gi], qcs + gi * 3 * QC_MAX, tsm + gi, nullptr);
      Grp<G>::sync();
    }
  }
}

// resident blocks per SM of the hull kernel of group width 32, 256, 512 or
// 1024 (0 when a width cannot run)
// (sets the block kernels' dynamic shared memory limit to their BatSm, for
// the device current at the call)
template <int G>
static int wide_blocks_per_sm() {
  const size_t dyn = sizeof(BatSm<G / 32>);
  cudaFuncSetAttribute(k_hull<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_hull<G>, G, dyn);
  return n;
}
int hull_blocks_per_sm(int width) {
  int n = 0;
  if (width == 32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_hull<32>, 256, 0);
  else if (width == 1024) n = wide_blocks_per_sm<1024>();
  else if (width == 512) n = wide_blocks_per_sm<512>();
  else n = wide_blocks_per_sm<256>();
  return n;
}

// hull launch of one group width (32 or 256) over P.nSlabs groups
void launch_hull(const Level& P, const Dev& D, int width, cudaStream_t s) {
  if (P.nChildParts == 0 || P.nSlabs == 0) return;
  if (width == 32) k_hull<32><<<(P.nSlabs + 7) / 8, 256, 0, s>>>(P, D);
  else if (width == 1024) k_hull<1024><<<P.nSlabs, 1024, sizeof(BatSm<32>), s>>>(P, D);
  else if (width == 512) k_hull<512><<<P.nSlabs, 512, sizeof(BatSm<16>), s>>>(P, D);
  else k_hull<256><<<P.nSlabs, 256, sizeof(BatSm<8>), s>>>(P, D);
}

// ---------------------------------------------------------------------------
// Hull of one point set without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a hull:
// a host application that hands every byte of the GPU to its own arena or
// caching allocator, or an interactive loop where cudaMalloc and cudaFree
// would stall work already running on the device. cuacd_tree_create
// allocates pools, so such callers get this entry point instead: they pass
// device buffers they already own for the points and the results, and the
// scratch the hull kernel needs (one slab, one part descriptor and the
// counters) comes from the fixed array below, which every GPU that loads the
// library holds until the process exits.
// ---------------------------------------------------------------------------

int set_error(int code, const char* msg);

// largest point set the fixed scratch holds
#define NOALLOC_MAX_POINTS 4096u
// one slab for NOALLOC_MAX_POINTS points with hullMaxVerts 4096, sized as the
// tree's slabs: ((2 n + n + 7) & ~7) + 16 (2 n + 3 * 2048 + 1024) words
// = 258048, plus the walk's arrays (hull_slab_stride): 436288 words, 1.7 MiB
#define NOALLOC_SLAB_WORDS hull_slab_stride(258048u)
#define NOALLOC_PART_OFF NOALLOC_SLAB_WORDS
#define NOALLOC_CTR_OFF (NOALLOC_PART_OFF + 16u)
#define NOALLOC_WORK_OFF (NOALLOC_CTR_OFF + (uint32_t)CTR_WORDS)
#define NOALLOC_WORDS (NOALLOC_WORK_OFF + 64u)

static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_WORDS];

// the part descriptor of the point set, zeroed counters
__global__ void k_noalloc_setup(uint32_t* scratch, uint32_t nv) {
  const int t = threadIdx.x;
  PartDesc* pd = reinterpret_cast<PartDesc*>(scratch + NOALLOC_PART_OFF);
  if (t == 0) {
    PartDesc p;
    p.vOff = 0; p.nv = nv; p.tOff = 0; p.nt = 0; p.eOff = 0; p.ne = 0;
    p.meshVol = 0.0f; p.hullVol = 0.0f;
    p.planeIds[0] = p.planeIds[1] = p.planeIds[2] = p.planeIds[3] = CUACD_NONE;
    p.nPlanes = 0; p.flags = 2; p.pad0 = 0; p.pad1 = 0;
    *pd = p;
  }
  for (uint32_t i = t; i < (uint32_t)CTR_WORDS; i += blockDim.x) scratch[NOALLOC_CTR_OFF + i] = 0;
  for (uint32_t i = t; i < 64; i += blockDim.x) scratch[NOALLOC_WORK_OFF + i] = 0;
}
// results with the status rule of the hull batches (tree.ts:750-753)
__global__ void k_noalloc_finish(const uint32_t* scratch, float* volume, uint32_t* ntris, int32_t* status) {
  const PartDesc* pd = reinterpret_cast<const PartDesc*>(scratch + NOALLOC_PART_OFF);
  const float vol = pd->hullVol;
  int32_t s = 0;
  if (vol < 0.0f) s = (pd->flags & 3) ? (int32_t)(pd->flags & 3) : 9;
  else if (pd->pad0 < 4) s = 8;
  *volume = vol;
  *ntris = s == 0 ? pd->pad0 : 0;
  *status = s;
}

}  // namespace cuacd

using namespace cuacd;

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

// The scratch array's device address in the calling thread's current
// context. In host code the array's name is only a stand-in, so the address
// is looked up with cudaGetSymbolAddress, once per context: the cache is keyed
// on the context's id (cuCtxGetId, reached through the runtime's driver entry
// points so the library needs no link against libcuda), which changes when a
// device's primary context is re-created (after cudaDeviceReset), when the
// module and with it the array may move.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

static int noalloc_scratch_address(uint32_t** out) {
  static std::mutex mu;
  static CtxGetCurrentFn getCurrent = nullptr;
  static CtxGetIdFn getId = nullptr;
  static bool resolved = false;
  struct Entry { unsigned long long ctx; uint32_t* addr; };
  static Entry cache[64];
  static int nCache = 0;
  std::lock_guard<std::mutex> lock(mu);
  if (!resolved) {
    cudaDriverEntryPointQueryResult q1, q2;
    void* f1 = nullptr;
    void* f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return set_error(-4, "cuacd_hull_points_noalloc: driver entry points cuCtxGetCurrent / cuCtxGetId unavailable");
    getCurrent = (CtxGetCurrentFn)f1;
    getId = (CtxGetIdFn)f2;
    resolved = true;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  void* p = nullptr;
  if (getCurrent(&ctx) != 0) return set_error(-4, "cuacd_hull_points_noalloc: no usable CUDA device");
  if (ctx != nullptr) {
    if (getId(ctx, &id) != 0) return set_error(-4, "cuacd_hull_points_noalloc: cannot read the context id");
    for (int i = 0; i < nCache; i++)
      if (cache[i].ctx == id) {
        *out = cache[i].addr;
        return 0;
      }
  }
  // not seen yet (or no context is current: the runtime makes the current
  // device's primary context current on this call)
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return set_error(-4, cudaGetErrorString(e));
  if (ctx == nullptr) {
    if (getCurrent(&ctx) != 0 || ctx == nullptr || getId(ctx, &id) != 0)
      return set_error(-4, "cuacd_hull_points_noalloc: no current CUDA context");
  }
  Entry ent{id, (uint32_t*)p};
  if (nCache < 64) cache[nCache++] = ent;
  else {  // more contexts than slots over the process's life: reuse the oldest
    std::memmove(cache, cache + 1, sizeof(Entry) * 63);
    cache[63] = ent;
  }
  *out = (uint32_t*)p;
  return 0;
}

extern "C" int cuacd_hull_points_noalloc(const float* points, uint32_t nv, uint32_t* tris, uint32_t trisCap,
                                         float* volume, uint32_t* ntris, int32_t* status, void* stream) {
  if (!points || !tris || !volume || !ntris || !status) return set_error(-1, "cuacd_hull_points_noalloc: null buffer");
  if (nv > NOALLOC_MAX_POINTS)
    return set_error(-2, "cuacd_hull_points_noalloc: at most 4096 points (the fixed scratch holds one 4096-point slab)");
  // a hull of nv points is a closed triangulated surface over at most nv
  // vertices, so it has at most 2 nv - 4 triangles; a smaller buffer could
  // not take every face, and the call is refused before any work is queued
  const uint64_t need = 3ull * std::max<uint64_t>(nv >= 4 ? 2ull * nv - 4 : 0, 4);
  if (trisCap < need) {
    char msg[160];
    snprintf(msg, sizeof(msg),
             "cuacd_hull_points_noalloc: trisCap %u u32 is below the %llu a hull of %u points may need (3 * (2 nv - 4), "
             "at least 12)", trisCap, (unsigned long long)need, nv);
    return set_error(-2, msg);
  }
  uint32_t* scratch = nullptr;
  if (int rc = noalloc_scratch_address(&scratch)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t maxNv = std::max(nv, 1u);
  const uint32_t fmax = 2 * std::min(4096u, maxNv) + 3 * HULL_VIS_MAX + 1024;
  Level P;
  memset(&P, 0, sizeof(P));
  P.totalLevels = 1;
  P.nChildParts = 1;
  P.hullSlabWords = ((2 * maxNv + std::max(maxNv, 80u) + 7) & ~7u) + 16 * fmax;
  P.slabStride = NOALLOC_SLAB_WORDS;
  P.nSlabs = 1;
  P.smallNv = 1024;
  P.exportBase = 0;
  P.exportStride = trisCap;
  P.maxNvHint = maxNv;
  Dev D;
  memset(&D, 0, sizeof(D));
  D.V = const_cast<float*>(points);
  D.T = tris;
  D.slab = scratch;
  D.parts = reinterpret_cast<PartDesc*>(scratch + NOALLOC_PART_OFF);
  D.ctr = scratch + NOALLOC_CTR_OFF;
  D.work = scratch + NOALLOC_WORK_OFF;
  k_noalloc_setup<<<1, 64, 0, s>>>(scratch, nv);
  if (nv <= P.smallNv) k_hull<32><<<1, 256, 0, s>>>(P, D);
  else k_hull<256><<<1, 256, sizeof(BatSm<8>), s>>>(P, D);
  k_noalloc_finish<<<1, 1, 0, s>>>(scratch, volume, ntris, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(-4, cudaGetErrorString(e));
  return 0;
}
