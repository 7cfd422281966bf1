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
  if (ps.nt == 0 || pt.nt == 0) return;
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

void launch_hd(const HdArgs& A, const Dev& D, cudaStream_t s) {
  if (A.nPairs == 0) return;
  k_hd_sample<32><<<(A.nMeshes + 7) / 8, 256, 0, s>>>(A, D);
  dim3 grid((A.maxSide + HD_TILE - 1) / HD_TILE, A.nPairs, 2);
  k_hd_dist<<<grid, HD_TILE, 0, s>>>(A, D);
}

}  // namespace cuacd
