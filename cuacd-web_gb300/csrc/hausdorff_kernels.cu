// hausdorff_kernels.cu — bidirectional sampled Hausdorff distance of mesh
// pairs on sm_103a (the reference's src/gpu/hausdorff_shader.ts:13-153).
//
// Sampling rule (as the reference): res = max(1000, floor(2000 * area));
// each triangle gets floor(res / area * a_t) samples, or one on every
// step-th (or every even) triangle that gets none; barycentrics from a Wang
// hash of t * 65537 + k.
//
// GB300 design: each mesh is sampled exactly once by one group (the
// reference re-samples both meshes in every 256-sample slice); the total
// area is summed in double so the per-triangle counts do not depend on a
// reduction order. The distance pass gives each thread one sample and
// streams the other mesh's triangles through shared memory in tiles; the
// squared distance maximum goes to one word per pair by an atomic max on
// its (non-negative) float bits.
#include <cuda_bf16.h>

#include "cuacd_dev.cuh"

namespace cuacd {

__device__ __forceinline__ uint32_t wang(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s = s * 9u;
  s = s ^ (s >> 4);
  s = s * 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}
__device__ __forceinline__ float tri_area(f3 a, f3 b, f3 c) {
  f3 n = cross(b - a, c - a);
  return 0.5f * sqrtf(dot(n, n));
}

template <int G>
__global__ void __launch_bounds__(256) k_hd_sample(const HdArgs A, const Dev D) {
  __shared__ GrpSmem gsm[Grp<G>::PER_BLOCK];
  const int gi = Grp<G>::gid(), lid = Grp<G>::lid();
  GrpSmem& sm = gsm[gi];
  const uint32_t m = blockIdx.x * Grp<G>::PER_BLOCK + gi;
  if (m >= A.nMeshes) return;
  const PartDesc pd = D.parts[A.partBase + m];
  const uint32_t nt = pd.nt, cap = A.capN[m];
  float4* out = A.samples + A.capOff[m];
  if (nt == 0) {
    if (lid == 0) A.ns[m] = 0;
    return;
  }
  double a = 0.0;
  for (uint32_t t = lid; t < nt; t += G) {
    const uint32_t* tr = D.T + pd.tOff + 3 * (size_t)t;
    a += (double)tri_area(ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[0]), ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[1]),
                          ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[2]));
  }
  const float total = (float)grp_sum_d<G>(a, sm);
  float res = floorf(2000.0f * total);
  if (res < 1000.0f) res = 1000.0f;
  const uint32_t step = (float)nt > res ? nt / (uint32_t)res : 0;
  uint32_t run = 0;
  for (uint32_t c = 0; c * G < nt; c++) {
    const uint32_t t = c * G + lid;
    uint32_t N = 0;
    f3 pa = mk3(0.f, 0.f, 0.f), pb = pa, pc = pa;
    if (t < nt) {
      const uint32_t* tr = D.T + pd.tOff + 3 * (size_t)t;
      pa = ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[0]);
      pb = ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[1]);
      pc = ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[2]);
      const float ta = tri_area(pa, pb, pc);
      const uint32_t areaCount = total > 1e-20f ? (uint32_t)floorf((res / total) * ta) : 0u;
      if ((float)nt > res) N = areaCount > 0 ? areaCount : ((t % max(step, 1u)) == 0 ? 1u : 0u);
      else N = areaCount > 0 ? areaCount : ((t % 2u) == 0 ? 1u : 0u);
    }
    uint32_t tot;
    const uint32_t pre = grp_scan_u<G>(N, &tot, sm);
    for (uint32_t k = 0; k < N; k++) {
      const uint32_t idx = run + pre + k;
      if (idx >= cap) break;
      const uint32_t ha = wang(t * 65537u + k);
      const uint32_t hb = wang(ha + 0x9e3779b9u);
      const float ra = (float)(ha & 0xFFFFFFu) / (float)0xFFFFFFu;
      const float rb = (float)(hb & 0xFFFFFFu) / (float)0xFFFFFFu;
      const float sqa = sqrtf(ra);
      const f3 s = ((1.0f - sqa) * pa + (sqa * (1.0f - rb)) * pb) + (sqa * rb) * pc;
      out[idx] = make_float4(s.x, s.y, s.z, 0.0f);
    }
    run += tot;
  }
  if (lid == 0) A.ns[m] = min(run, cap);
}

// squared distance from p to triangle (a, b, c) (hausdorff_shader.ts:32-52)
__device__ __forceinline__ float seg_sq(f3 p, f3 a, f3 b) {
  const f3 ab = b - a, ap = p - a;
  const float ab2 = dot(ab, ab);
  float t = ab2 > 1e-20f ? dot(ap, ab) / ab2 : 0.0f;
  t = fminf(fmaxf(t, 0.0f), 1.0f);
  const f3 d = ap - t * ab;
  return dot(d, d);
}
__device__ __forceinline__ float tri_sq(f3 p, f3 a, f3 b, f3 c) {
  const f3 ab = b - a, ac = c - a, ap = p - a;
  const f3 n = cross(ab, ac);
  const float n2 = dot(n, n);
  if (n2 < 1e-20f) {
    const f3 bp = p - b, cp = p - c;
    return fminf(dot(ap, ap), fminf(dot(bp, bp), dot(cp, cp)));
  }
  const float d00 = dot(ab, ab), d01 = dot(ab, ac), d02 = dot(ab, ap);
  const float d11 = dot(ac, ac), d12 = dot(ac, ap);
  const float inv = 1.0f / (d00 * d11 - d01 * d01);
  const float u = (d11 * d02 - d01 * d12) * inv;
  const float v = (d00 * d12 - d01 * d02) * inv;
  if (u >= 0.0f && v >= 0.0f && u + v <= 1.0f) {
    const float dist = dot(n, ap);
    return (dist * dist) / n2;
  }
  return fminf(seg_sq(p, a, b), fminf(seg_sq(p, b, c), seg_sq(p, c, a)));
}

#define HD_TILE 128

// grid: x = sample tile, y = pair, z = direction (0: A samples vs B, 1: B vs A)
__global__ void __launch_bounds__(HD_TILE) k_hd_dist(const HdArgs A, const Dev D) {
  __shared__ float tv[HD_TILE][9];
  __shared__ float red[HD_TILE / 32];
  const uint32_t pair = blockIdx.y, dir = blockIdx.z;
  const uint32_t src = dir == 0 ? pair : A.nPairs + pair;
  const uint32_t dst = dir == 0 ? A.nPairs + pair : pair;
  const PartDesc ps = D.parts[A.partBase + src], pt = D.parts[A.partBase + dst];
  if (ps.nt == 0 || pt.nt == 0 || pt.nt >= A.screenMin) return;
  const uint32_t ns = A.ns[src];
  const uint32_t s0 = blockIdx.x * HD_TILE;
  if (s0 >= ns) return;
  const uint32_t si = s0 + threadIdx.x;
  f3 p = mk3(0.f, 0.f, 0.f);
  if (si < ns) {
    float4 q = A.samples[A.capOff[src] + si];
    p = mk3(q.x, q.y, q.z);
  }
  float best = 1e30f;
  for (uint32_t t0 = 0; t0 < pt.nt; t0 += HD_TILE) {
    const uint32_t t = t0 + threadIdx.x;
    __syncthreads();
    if (t < pt.nt) {
      const uint32_t* tr = D.T + pt.tOff + 3 * (size_t)t;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        f3 v = ldv(D.V, (size_t)pt.vOff + 3 * (size_t)tr[k]);
        tv[threadIdx.x][3 * k] = v.x; tv[threadIdx.x][3 * k + 1] = v.y; tv[threadIdx.x][3 * k + 2] = v.z;
      }
    }
    __syncthreads();
    const uint32_t cnt = min((uint32_t)HD_TILE, pt.nt - t0);
    for (uint32_t k = 0; k < cnt; k++) {
      const float* w = tv[k];
      best = fminf(best, tri_sq(p, mk3(w[0], w[1], w[2]), mk3(w[3], w[4], w[5]), mk3(w[6], w[7], w[8])));
    }
  }
  float worst = si < ns ? best : 0.0f;
  worst = warp_max_f(worst);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = worst;
  __syncthreads();
  if (threadIdx.x == 0) {
    float w = red[0];
    for (int i = 1; i < HD_TILE / 32; i++) w = fmaxf(w, red[i]);
    atomicMax(D.ctr + CTR_HD + pair, __float_as_uint(w));
  }
}

// ---------------------------------------------------------------------------
// Tensor-core screen for target meshes of at least A.screenMin triangles.
//
// For sample p and triangle t with centroid c and bounding radius r,
// dist(p, t) >= |p - c| - r and the smallest distance is at most |p - c|.
// |p - c|^2 = |p|^2 + (|c|^2 - 2 p . c), and the bracket for 128 samples x
// 128 triangles is one tcgen05 MMA (kind::f16, bf16 operands, fp32
// accumulation in TMEM) with K = 16: each coordinate is split into a bf16
// high part and a bf16 low part, and the 16 products of the row
// [p_hi, p_hi, p_lo, p_lo, 1, 1, 0, 0] with [-2c_hi, -2c_lo, -2c_hi, -2c_lo,
// |c|^2_hi, |c|^2_lo, 0, 0] (three lanes per point) give -2 p . c + |c|^2 to
// about 2^-16 of its terms. Each thread owns one sample (one TMEM lane), reads
// its row of distances and computes the exact float32 distance (tri_sq, the
// same function as the exhaustive kernel) only for triangles whose lower
// bound, with the screen's error bound and a 1e-3 relative margin, does not
// exceed the running minimum or the smallest upper bound: the triangle that
// attains the exhaustive minimum is never skipped, so the result is that
// minimum bit for bit.
#define HDS_M 128u          // samples per CTA = TMEM lanes
#define HDS_N 128u          // triangles per MMA = TMEM columns (fp32)

__device__ __forceinline__ uint32_t bf16_bits(float x) { return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_val(uint32_t b) { return __bfloat162float(__ushort_as_bfloat16((unsigned short)b)); }
__device__ __forceinline__ void bf16_split(float x, uint32_t& hi, uint32_t& lo) {
  hi = bf16_bits(x);
  lo = bf16_bits(x - bf16_val(hi));
}
__device__ __forceinline__ uint32_t pack2(uint32_t lo16, uint32_t hi16) { return lo16 | (hi16 << 16); }

// one block per mesh: the screen data of its triangles
__global__ void __launch_bounds__(256) k_hd_prep(const HdArgs A, const Dev D) {
  const uint32_t m = blockIdx.x;
  if (m >= A.nMeshes) return;
  const PartDesc pd = D.parts[A.partBase + m];
  const uint32_t base = A.triOff[m];
  for (uint32_t t = threadIdx.x; t < pd.nt; t += blockDim.x) {
    const uint32_t* tr = D.T + pd.tOff + 3 * (size_t)t;
    const f3 a = ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[0]);
    const f3 b = ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[1]);
    const f3 c = ldv(D.V, (size_t)pd.vOff + 3 * (size_t)tr[2]);
    const f3 g = mk3((a.x + b.x + c.x) / 3.0f, (a.y + b.y + c.y) / 3.0f, (a.z + b.z + c.z) / 3.0f);
    const float ra = sqrtf(dot(a - g, a - g)), rb = sqrtf(dot(b - g, b - g)), rc = sqrtf(dot(c - g, c - g));
    // radius rounded up past its float32 error
    const float r = fmaxf(fmaxf(ra, rb), rc) * 1.00001f + 1e-30f;
    const float c1 = fabsf(g.x) + fabsf(g.y) + fabsf(g.z);
    const float cc = dot(g, g);
    uint32_t h[3], l[3], ch, cl;
    bf16_split(-2.0f * g.x, h[0], l[0]);
    bf16_split(-2.0f * g.y, h[1], l[1]);
    bf16_split(-2.0f * g.z, h[2], l[2]);
    bf16_split(cc, ch, cl);
    // K order: [-2c_hi, -2c_lo, -2c_hi, -2c_lo, |c|^2 hi, |c|^2 lo, 0, 0]
    const uint32_t k16[16] = {h[0], h[1], h[2], l[0], l[1], l[2], h[0], h[1], h[2], l[0], l[1], l[2], ch, cl, 0u, 0u};
    uint4 r0, r1;
    r0.x = pack2(k16[0], k16[1]); r0.y = pack2(k16[2], k16[3]); r0.z = pack2(k16[4], k16[5]); r0.w = pack2(k16[6], k16[7]);
    r1.x = pack2(k16[8], k16[9]); r1.y = pack2(k16[10], k16[11]); r1.z = pack2(k16[12], k16[13]); r1.w = 0u;
    A.triB[2 * (size_t)(base + t)] = r0;
    A.triB[2 * (size_t)(base + t) + 1] = r1;
    A.triG[3 * (size_t)(base + t)] = make_float4(a.x, a.y, a.z, r);
    A.triG[3 * (size_t)(base + t) + 1] = make_float4(b.x, b.y, b.z, c1);
    A.triG[3 * (size_t)(base + t) + 2] = make_float4(c.x, c.y, c.z, cc);
  }
}

// byte offset of element (row, k) of a K-major bf16 operand tile with K = 16
// in the canonical no-swizzle layout: 8-row x 16-byte core matrices, the two
// K halves of an 8-row group 128 bytes apart (leading byte offset), 8-row
// groups 256 bytes apart (stride byte offset)
__device__ __forceinline__ uint32_t tile_off(uint32_t row, uint32_t khalf) {
  return ((row >> 3) * 2 + khalf) * 128 + (row & 7) * 16;
}
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(256u >> 4) << 32) |
         (1ull << 46);
}
// instruction descriptor, kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N = HDS_N, M = HDS_M
constexpr uint32_t HDS_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((HDS_N >> 3) << 17) | ((HDS_M >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// at most 4 CTAs of this kernel per SM (the static shared memory below), so
// their 4 x 128 TMEM columns never exceed the SM's 512 and allocation never
// waits
#define HDS_PAD_BYTES (46u * 1024u)

__global__ void __launch_bounds__(HDS_M) k_hd_screen(const HdArgs A, const Dev D) {
  __shared__ __align__(1024) uint8_t smem[HDS_PAD_BYTES];
  uint8_t* sA = smem;                      // 128 rows x 32 bytes
  uint8_t* sB = smem + HDS_M * 32;         // 128 rows x 32 bytes
  float* sR = reinterpret_cast<float*>(smem + (HDS_M + HDS_N) * 32);  // per tile triangle: radius, |c|_1, |c|^2
  float* sC1 = sR + HDS_N;
  float* sCC = sC1 + HDS_N;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sCC + HDS_N);
  uint32_t* tbase = reinterpret_cast<uint32_t*>(mbar + 1);
  float* red = reinterpret_cast<float*>(tbase + 1);
  const uint32_t pair = blockIdx.y, dir = blockIdx.z;
  const uint32_t src = dir == 0 ? pair : A.nPairs + pair;
  const uint32_t dst = dir == 0 ? A.nPairs + pair : pair;
  const PartDesc ps = D.parts[A.partBase + src], pt = D.parts[A.partBase + dst];
  if (ps.nt == 0 || pt.nt == 0 || pt.nt < A.screenMin) return;
  const uint32_t ns = A.ns[src];
  const uint32_t s0 = blockIdx.x * HDS_M;
  if (s0 >= ns) return;
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase)),
                 "r"(HDS_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  // this thread's sample as operand row A
  const uint32_t si = s0 + tid;
  f3 p = mk3(0.f, 0.f, 0.f);
  if (si < ns) {
    const float4 q = A.samples[A.capOff[src] + si];
    p = mk3(q.x, q.y, q.z);
  }
  {
    uint32_t h[3], l[3];
    bf16_split(p.x, h[0], l[0]);
    bf16_split(p.y, h[1], l[1]);
    bf16_split(p.z, h[2], l[2]);
    const uint32_t one = bf16_bits(1.0f);
    // K order: [p_hi, p_hi, p_lo, p_lo, 1, 1, 0, 0]
    const uint4 r0 = make_uint4(pack2(h[0], h[1]), pack2(h[2], h[0]), pack2(h[1], h[2]), pack2(l[0], l[1]));
    const uint4 r1 = make_uint4(pack2(l[2], l[0]), pack2(l[1], l[2]), pack2(one, one), 0u);
    *reinterpret_cast<uint4*>(sA + tile_off(tid, 0)) = r0;
    *reinterpret_cast<uint4*>(sA + tile_off(tid, 1)) = r1;
  }
  const float p2 = dot(p, p);
  const float p1 = fabsf(p.x) + fabsf(p.y) + fabsf(p.z);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tbase;
  const uint64_t descA = smem_desc(smem_u32(sA)), descB = smem_desc(smem_u32(sB));
  const uint32_t base = A.triOff[dst], nt = pt.nt;
  float best = 3.4e38f, ub = 3.4e38f;
  uint32_t phase = 0, exact = 0;
  bool ok = true;
  for (uint32_t t0 = 0; t0 < nt && ok; t0 += HDS_N) {
    // triangle rows of this tile (zero rows past the end)
    {
      const uint32_t t = t0 + tid;
      uint4 r0 = make_uint4(0, 0, 0, 0), r1 = r0;
      float rr = 0.f, c1 = 0.f, cc = 0.f;
      if (t < nt) {
        r0 = A.triB[2 * (size_t)(base + t)];
        r1 = A.triB[2 * (size_t)(base + t) + 1];
        rr = A.triG[3 * (size_t)(base + t)].w;
        c1 = A.triG[3 * (size_t)(base + t) + 1].w;
        cc = A.triG[3 * (size_t)(base + t) + 2].w;
      }
      *reinterpret_cast<uint4*>(sB + tile_off(tid, 0)) = r0;
      *reinterpret_cast<uint4*>(sB + tile_off(tid, 1)) = r1;
      sR[tid] = rr;
      sC1[tid] = c1;
      sCC[tid] = cc;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      asm volatile(
          "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
          "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
          "l"(descA), "l"(descB), "r"(HDS_IDESC), "r"(0u));
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(mbar))
                   : "memory");
    }
    // the MMA's completion, with a bounded wait
    bool done = false;
    for (uint32_t it = 0; it < (1u << 20) && !done; it++) {
      uint32_t r;
      asm volatile(
          "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}"
          : "=r"(r)
          : "r"(smem_u32(mbar)), "r"(phase)
          : "memory");
      done = r != 0;
    }
    phase ^= 1u;
    ok = __syncthreads_and(done) != 0;
    if (!ok) {
      if (tid == 0) atomicExch(D.ctr + CTR_HD_ERR, 1u);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t cnt = min(HDS_N, nt - t0);
    for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((warp * 32u) << 16) + c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      // the 32 columns' bounds (the bound may only be larger than the
      // final one: best and ub only decrease), then the exact distances of
      // the survivors
      uint32_t keep = 0;
#pragma unroll
      for (uint32_t j = 0; j < 32; j++) {
        const uint32_t k = c0 + j;
        if (k < cnt) {
          // |p - c|^2 as screened, and its error bound e = 2^-13 (|p|^2 +
          // |c|^2 + 2 |p|_1 |c|_1). Derivation (u = 2^-24, bf16 unit
          // roundoff 2^-8): the hi/lo split leaves |x - x_hi - x_lo| <=
          // 2^-16 |x| for every coordinate of p and of -2c and for |c|^2, so
          // the split products miss at most 2^-14 sum|p_i||c_i| + 2^-16
          // |c|^2; the bf16 x bf16 products are exact in fp32 and the 16-term
          // accumulation (at most 15 roundings, each at most 2^-23 relative
          // even if the tensor core truncates) adds at most 1.8e-6 (2
          // sum|p_i||c_i| + |c|^2); |p|^2 and |c|^2 themselves are fp32 dot
          // products (3u) and the final add one more u. In total e_true <=
          // 6.5e-5 sum|p_i||c_i| + 1.8e-5 |c|^2 + 2.4e-7 |p|^2, which e
          // exceeds by 3.8x, 7x and 500x (sum|p_i||c_i| <= |p|_1 |c|_1);
          // the fp32 rounding of e, q2 + e and the square roots below are
          // covered by the 1e-3 relative margin of the comparison. Far from
          // the origin |p|^2 and -2 p.c cancel and e grows with them: the
          // screen then keeps more triangles, never a wrong one.
          const float q2 = p2 + __uint_as_float(v[j]);
          const float e = 1.220703125e-4f * (p2 + sCC[k] + 2.0f * p1 * sC1[k]);
          ub = fminf(ub, q2 + e);
          const float lo = sqrtf(fmaxf(q2 - e, 0.0f)) - sR[k];
          const float lb2 = lo > 0.0f ? lo * lo : 0.0f;
          const float bound = fminf(best, ub);
          if (lb2 <= bound * 1.001f + 1e-10f * (p2 + sCC[k]) + 1e-30f) keep |= 1u << j;
        }
      }
      while (keep) {
        const uint32_t j = __ffs(keep) - 1;
        keep &= keep - 1;
        const float4* g = A.triG + 3 * (size_t)(base + t0 + c0 + j);
        const float4 a = g[0], b = g[1], c = g[2];
        best = fminf(best, tri_sq(p, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z)));
        exact++;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // every thread is done with this tile's radii before the next tile's
    // rows overwrite them
    __syncthreads();
  }
  // the tile's largest smallest distance (squared)
  float worst = (ok && si < ns) ? best : 0.0f;
  worst = warp_max_f(worst);
  unsigned long long ex = warp_sum_u(exact);
  if ((tid & 31) == 0) {
    red[warp] = worst;
    add_bytes(D.ctr, CTR_HD_EXACT, ex);
  }
  __syncthreads();
  if (tid == 0) {
    float w = red[0];
    for (uint32_t i = 1; i < HDS_M / 32; i++) w = fmaxf(w, red[i]);
    if (ok) atomicMax(D.ctr + CTR_HD + pair, __float_as_uint(w));
    const uint32_t nsTile = min(HDS_M, ns - s0);
    add_bytes(D.ctr, CTR_HD_SCREENED, (unsigned long long)nsTile * nt);
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(HDS_N));
}

void launch_hd(const HdArgs& A, const Dev& D, cudaStream_t s) {
  if (A.nPairs == 0) return;
  k_hd_sample<32><<<(A.nMeshes + 7) / 8, 256, 0, s>>>(A, D);
  k_hd_prep<<<A.nMeshes, 256, 0, s>>>(A, D);
  dim3 grid((A.maxSide + HD_TILE - 1) / HD_TILE, A.nPairs, 2);
  k_hd_dist<<<grid, HD_TILE, 0, s>>>(A, D);
  dim3 gs((A.maxSide + HDS_M - 1) / HDS_M, A.nPairs, 2);
  k_hd_screen<<<gs, HDS_M, 0, s>>>(A, D);
}

}  // namespace cuacd
