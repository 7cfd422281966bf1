// cuacd_dev.cuh — device-side records, launch parameters and group
// primitives shared by the engine's kernels.
//
// A "group" is the set of threads that cooperates on one job or one part:
// either one warp (G = 32, eight groups per 256-thread block) or one whole
// block (G = 256). Small parts use warps, large parts use blocks; the kernels
// are written once for both.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CUACD_NONE 0xffffffffu
#define FULLMASK 0xffffffffu

namespace cuacd {

enum { CTR_V = 0, CTR_T = 1, CTR_E = 2, CTR_S = 3, CTR_OVERFLOW = 4, CTR_HULLFAIL = 5, CTR_NPOVER = 6, CTR_PRUNED = 7 };
// counters after the reference's eight: candidate cuts evaluated (valid jobs
// after plan, 64-bit as two words), then Hausdorff results
// algorithmic bytes of plan, emit and hull as 64-bit counters (a candidate
// reads its parent once, writes its children once and each child's points
// are read once by its hull), then Hausdorff results
// and the Hausdorff screen's statistics: exact point-triangle distances
// (64-bit), screened pairs (64-bit) and a flag for a tensor-core wait that
// timed out
enum { CTR_VALID_LO = 8, CTR_VALID_HI = 9, CTR_BYTES_PLAN = 10, CTR_BYTES_EMIT = 12, CTR_BYTES_HULL = 14, CTR_HD = 16,
       CTR_HD_EXACT = 16 + 1024, CTR_HD_SCREENED = 16 + 1026, CTR_HD_ERR = 16 + 1028, CTR_WORDS = 16 + 1032 };
__device__ __forceinline__ void add_bytes(uint32_t* ctr, int slot, unsigned long long b) {
  atomicAdd(reinterpret_cast<unsigned long long*>(ctr + slot), b);
}

// PartDesc (shaders.ts:41-46), 16 words
struct PartDesc {
  uint32_t vOff, nv, tOff, nt;
  uint32_t eOff, ne;
  float meshVol, hullVol;
  uint32_t planeIds[4];
  uint32_t nPlanes, flags, pad0, pad1;
};
// ItemDesc (shaders.ts:48-53), 20 words
struct ItemDesc {
  uint32_t partIds[8];
  uint32_t np, srcPart, initialCut, nLevels;
  float levelCosts[4];
  uint32_t flags, parentItem, cutIdx, pad0;
};
// Job (shaders.ts:55-60), 24 words
struct Job {
  float4 plane;
  uint32_t parentItem, parentPart, valid, cutIdx;
  uint32_t cnt[8];  // posNv posNt posNe negNv negNt negNe posKept negKept
  uint32_t off[8];  // posV posT posE negV negT negE scratch pad
};
static_assert(sizeof(PartDesc) == 64, "PartDesc layout");
static_assert(sizeof(ItemDesc) == 80, "ItemDesc layout");
static_assert(sizeof(Job) == 96, "Job layout");

// Device pools and tables of one tree handle
struct Dev {
  float* V;           // vertex floats, 3 per vertex
  uint32_t* T;        // triangle indices, 3 per triangle, part-local
  uint32_t* E;        // open edges, 8 words: p.xyz q.xyz planeId pad
  uint32_t* S;        // per-level scratch (side flags, then vertex remap)
  uint32_t* slab;     // hull scratch slabs
  PartDesc* parts;
  ItemDesc* items;
  Job* jobs;
  float4* planes;
  uint32_t* ctr;
  unsigned long long* scanTmp;  // scan bases and per-block sums (3 + 3 * blocks)
  uint32_t* work;               // hull work counters, one per hull launch of a run
  float* ub;                    // per seed: the last level's pruning upper bound
  uint64_t vCap, tCap, eCap, sCap;
};

// Launch parameters of one tree level (the reference's Params, shaders.ts:30-39)
struct Level {
  uint32_t itemsInBase, nItemsIn, itemsOutBase, jobBase;
  uint32_t width, nEdgeCuts, edgeStride, totalWidth;
  float minEdgeDist;
  uint32_t level, totalLevels, partBase;
  uint32_t edgePlaneBase, nChildParts, nJobs;
  uint32_t hullSlabWords;   // logical slab size (sets fmax, as tree.ts:300-312)
  uint32_t slabStride;      // physical words per slab
  uint32_t nSlabs;          // slabs for this launch
  uint32_t smallNv;         // parts with nv <= smallNv go to warp groups
  uint32_t exportBase, exportStride;  // hull face export into T (u32 offsets)
  uint32_t lastLevel, hullStage, nSeeds;
  uint32_t hdDescBase;      // != 0: write a Hausdorff descriptor at part + hdDescBase
  uint32_t workSlot;        // hull work counters of this launch: D.work[slot] (warp
                            // groups) and D.work[16 + slot] (256-thread groups)
  uint32_t maxNvHint;       // largest part the host knows of, or 0: read D.work[32 + workSlot]
};

// Hausdorff batch: mesh m's descriptor at parts[partBase + m]; pair k is
// (A_k, B_k) = (mesh k, mesh nPairs + k)
struct HdArgs {
  uint32_t nPairs;
  uint32_t nMeshes;          // 2 * nPairs
  const uint32_t* capOff;    // per mesh: sample offset (float4 units)
  const uint32_t* capN;      // per mesh: sample capacity
  float4* samples;
  uint32_t* ns;              // per mesh: sample count
  uint32_t partBase;
  uint32_t maxSide;          // largest per-side capacity
  uint32_t screenMin;        // targets with at least this many triangles are screened
  const uint32_t* triOff;    // per mesh: first triangle of its screen data
  uint4* triB;               // per triangle: tensor-core operand row (16 bf16)
  float4* triG;              // per triangle: corners; w = radius, |c|_1, |c|^2
};

// Physical words of one hull slab whose reference size (which fixes the face
// limit fmax) is W words. After the W words a part of nv points needs the
// visible list and walk queue (2 * 2048), adjacency (4 fmax), two bitmap
// arrays (2 ceil(fmax / 32)) and two horizon maps (2 nv). With fmax <= (W -
// 3 nv) / 16 and nv <= (W - 1024) / 3 that is below 3672 + 0.671 W.
__host__ __device__ constexpr uint32_t hull_slab_stride(uint32_t W) {
  return (W + 4096u + (uint32_t)(((uint64_t)W * 2) / 3) + W / 128 + 64u + 63u) & ~63u;
}

// ---------------- group primitives ----------------
template <int G> struct Grp;

template <> struct Grp<32> {
  static __device__ __forceinline__ void sync() { __syncwarp(); }
  static __device__ __forceinline__ int lid() { return threadIdx.x & 31; }
  static __device__ __forceinline__ int gid() { return threadIdx.x >> 5; }
  static constexpr int PER_BLOCK = 8;
};
template <> struct Grp<256> {
  static __device__ __forceinline__ void sync() { __syncthreads(); }
  static __device__ __forceinline__ int lid() { return threadIdx.x; }
  static __device__ __forceinline__ int gid() { return 0; }
  static constexpr int PER_BLOCK = 1;
};
template <> struct Grp<512> {
  static __device__ __forceinline__ void sync() { __syncthreads(); }
  static __device__ __forceinline__ int lid() { return threadIdx.x; }
  static __device__ __forceinline__ int gid() { return 0; }
  static constexpr int PER_BLOCK = 1;
};
template <> struct Grp<1024> {
  static __device__ __forceinline__ void sync() { __syncthreads(); }
  static __device__ __forceinline__ int lid() { return threadIdx.x; }
  static __device__ __forceinline__ int gid() { return 0; }
  static constexpr int PER_BLOCK = 1;
};

// Per-group shared scratch for cross-warp reductions (unused by warp groups)
// (one entry per warp of the widest group, 1024 threads)
struct GrpSmem {
  double d[32];
  uint32_t u[32][4];
  float f[32][4];
  uint32_t bc[8];
};

__device__ __forceinline__ uint32_t warp_sum_u(uint32_t v) { return __reduce_add_sync(FULLMASK, v); }
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
  return v;
}
__device__ __forceinline__ float warp_min_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(FULLMASK, v, o));
  return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULLMASK, v, o));
  return v;
}
// inclusive scan within a warp
__device__ __forceinline__ uint32_t warp_incl_u(uint32_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(FULLMASK, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

template <int G> __device__ __forceinline__ uint32_t grp_sum_u(uint32_t v, GrpSmem& sm) {
  v = warp_sum_u(v);
  if (G == 32) return v;
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sm.u[w][0] = v;
  __syncthreads();
  uint32_t r = 0;
#pragma unroll
  for (int i = 0; i < G / 32; i++) r += sm.u[i][0];
  return r;
}
template <int G> __device__ __forceinline__ double grp_sum_d(double v, GrpSmem& sm) {
  v = warp_sum_d(v);
  if (G == 32) return v;
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sm.d[w] = v;
  __syncthreads();
  double r = 0;
#pragma unroll
  for (int i = 0; i < G / 32; i++) r += sm.d[i];
  return r;
}
template <int G> __device__ __forceinline__ float grp_min_f(float v, GrpSmem& sm) {
  v = warp_min_f(v);
  if (G == 32) return v;
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sm.f[w][0] = v;
  __syncthreads();
  float r = sm.f[0][0];
#pragma unroll
  for (int i = 1; i < G / 32; i++) r = fminf(r, sm.f[i][0]);
  return r;
}
template <int G> __device__ __forceinline__ float grp_max_f(float v, GrpSmem& sm) {
  v = warp_max_f(v);
  if (G == 32) return v;
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sm.f[w][0] = v;
  __syncthreads();
  float r = sm.f[0][0];
#pragma unroll
  for (int i = 1; i < G / 32; i++) r = fmaxf(r, sm.f[i][0]);
  return r;
}
// exclusive scan over the group in lane order; total in *tot
template <int G> __device__ __forceinline__ uint32_t grp_scan_u(uint32_t v, uint32_t* tot, GrpSmem& sm) {
  int lane = threadIdx.x & 31;
  uint32_t inc = warp_incl_u(v, lane);
  if (G == 32) {
    *tot = __shfl_sync(FULLMASK, inc, 31);
    return inc - v;
  }
  int w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 31) sm.u[w][1] = inc;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int i = 0; i < G / 32; i++) {
    uint32_t t = sm.u[i][1];
    if (i < w) before += t;
    all += t;
  }
  *tot = all;
  return before + inc - v;
}
// exclusive scan of 0/1 flags in lane order (ballot and popcount per warp)
template <int G> __device__ __forceinline__ uint32_t grp_scan_bit(bool b, uint32_t* tot, GrpSmem& sm) {
  const unsigned m = __ballot_sync(FULLMASK, b);
  const int lane = threadIdx.x & 31;
  const uint32_t pre = __popc(m & ((1u << lane) - 1u));
  if (G == 32) {
    *tot = __popc(m);
    return pre;
  }
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sm.u[w][1] = __popc(m);
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int i = 0; i < G / 32; i++) {
    uint32_t t = sm.u[i][1];
    if (i < w) before += t;
    all += t;
  }
  *tot = all;
  return before + pre;
}
// argmax of (value, index): largest value, lowest index on ties
__device__ __forceinline__ void am_merge(float& v, uint32_t& i, float v2, uint32_t i2) {
  if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}
template <int G> __device__ __forceinline__ void grp_argmax(float& v, uint32_t& i, GrpSmem& sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float v2 = __shfl_xor_sync(FULLMASK, v, o);
    uint32_t i2 = __shfl_xor_sync(FULLMASK, i, o);
    am_merge(v, i, v2, i2);
  }
  if (G == 32) return;
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) { sm.f[w][1] = v; sm.u[w][2] = i; }
  __syncthreads();
  v = sm.f[0][1];
  i = sm.u[0][2];
#pragma unroll
  for (int k = 1; k < G / 32; k++) am_merge(v, i, sm.f[k][1], sm.u[k][2]);
}
// argmax over lanes whose value is positive: largest value, lowest index on
// ties; lanes with v <= 0 take no part. Positive floats order like their
// bits, so a warp needs two redux instructions. With no positive value the
// result is v = -1, i = NONE.
template <int G> __device__ __forceinline__ void grp_argmax_pos(float& v, uint32_t& i, GrpSmem& sm) {
  if (G == 32) {
    const uint32_t key = v > 0.0f ? __float_as_uint(v) : 0u;
    const uint32_t mk = __reduce_max_sync(FULLMASK, key);
    const uint32_t mi = __reduce_min_sync(FULLMASK, (key == mk && mk != 0u) ? i : 0xffffffffu);
    v = mk != 0u ? __uint_as_float(mk) : -1.0f;
    i = mk != 0u ? mi : 0xffffffffu;
    return;
  }
  if (!(v > 0.0f)) { v = -1.0f; i = 0xffffffffu; }
  grp_argmax<G>(v, i, sm);
}
// broadcast a value from lane 0 of the group
template <int G> __device__ __forceinline__ uint32_t grp_bcast_u(uint32_t v, GrpSmem& sm) {
  if (G == 32) return __shfl_sync(FULLMASK, v, 0);
  __syncthreads();
  if (threadIdx.x == 0) sm.bc[0] = v;
  __syncthreads();
  return sm.bc[0];
}
template <int G> __device__ __forceinline__ bool grp_any(bool p, GrpSmem& sm) {
  bool w = __any_sync(FULLMASK, p);
  if (G == 32) return w;
  return grp_sum_u<G>(w ? 1u : 0u, sm) != 0;
}

// ---------------- float32 geometry in a fixed operation order ----------------
// These files are compiled with --fmad=false, so every multiply and add
// rounds separately, as in the CPU oracle.
struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(f3 a, f3 b) {
  float r = a.x * b.x;
  r = r + a.y * b.y;
  r = r + a.z * b.z;
  return r;
}
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 xyz(float4 p) { return mk3(p.x, p.y, p.z); }
__device__ __forceinline__ float comp(f3 a, uint32_t k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
__device__ __forceinline__ f3 vmin3(f3 a, f3 b) { return mk3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ f3 vmax3(f3 a, f3 b) { return mk3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ float l1(f3 a) { return (fabsf(a.x) + fabsf(a.y)) + fabsf(a.z); }

__device__ __forceinline__ f3 ldv(const float* V, size_t off) { return mk3(V[off], V[off + 1], V[off + 2]); }
__device__ __forceinline__ void stv(float* V, size_t off, f3 p) { V[off] = p.x; V[off + 1] = p.y; V[off + 2] = p.z; }

// Neumaier compensated float32 sum
struct KSum {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.0f; c = 0.0f; }
  __device__ __forceinline__ void add(float x) {
    float t = s + x;
    if (fabsf(s) >= fabsf(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// rv cost (part.ts:24-26, shaders.ts:154-157) with the gap and cube root in double
__device__ __forceinline__ float rv_cost(float meshVol, float hullVol) {
  double gap = (double)hullVol - (double)meshVol;
  if (gap < 0.0) gap = 0.0;
  return (float)(0.3 * cbrt(0.238732414637843 * gap));
}

}  // namespace cuacd
