// tree_kernels.cu — one level of the lookahead tree on sm_103a: plan, scan,
// emit and record, plus evaluate (the reference's src/gpu/shaders.ts kernels
// of the same names, lines 296-750 and 1404-1544).
//
// Design (GB300): every job (an item and one candidate plane) is handled by
// one group, a warp for small parents and a 256-thread block for large
// ones, with warp shuffles instead of workgroup barrier trees. Output order
// is the reference's (kept vertices in index order, then intersection
// vertices, triangles and open edges in source-triangle order), produced
// with group prefix sums. Per-job flux is accumulated with a compensated
// float32 sum per lane and combined in double.
//
// Compiled with --fmad=false: float32 results match the CPU oracle bit for
// bit.
#include "cuacd_dev.cuh"

namespace cuacd {

__device__ __forceinline__ int vsign(float d) { return d > 1e-6f ? 1 : (d < -1e-6f ? -1 : 0); }

struct Poly { uint32_t n; uint32_t src[4]; };

// Sutherland-Hodgman clip of one triangle (shaders.ts:171-181)
__device__ __forceinline__ Poly clip_tri(int s0, int s1, int s2, int side) {
  int sg[3] = {s0, s1, s2};
  Poly p;
  p.n = 0;
#pragma unroll
  for (uint32_t k = 0; k < 3; k++) {
    uint32_t q = k == 2 ? 0 : k + 1;
    int sp = sg[k] * side, sq = sg[q] * side;
    if (sp >= 0) p.src[p.n++] = k;
    if (sg[k] != 0 && sg[q] != 0 && sp * sq < 0) p.src[p.n++] = 4 + k;
  }
  return p;
}
// triangles, intersection vertices and on-plane edges of a polygon (shaders.ts:184-198)
__device__ __forceinline__ void poly_stats(const Poly& p, const int sg[3], uint32_t& ntri, uint32_t& nnew, uint32_t& nedge) {
  ntri = p.n >= 3 ? p.n - 2 : 0;
  nnew = 0;
  nedge = 0;
  if (p.n >= 3) {
    for (uint32_t i = 0; i < p.n; i++) {
      uint32_t u = p.src[i], v = p.src[(i + 1) % p.n];
      if (u >= 4) nnew++;
      bool uOn = u >= 4 || sg[u] == 0;
      bool vOn = v >= 4 || sg[v] == 0;
      if (uOn && vOn) nedge++;
    }
  }
}

__device__ __forceinline__ f3 plane_point(float4 pl) {
  f3 n = xyz(pl);
  float n2 = fmaxf(dot(n, n), 1e-30f);
  return ((-pl.w) * n) / n2;
}
// divergence-theorem anchor (shaders.ts:123-143)
__device__ f3 anchor_for(const float4* pl, uint32_t n) {
  if (n == 0) return mk3(0.f, 0.f, 0.f);
  if (n == 1) return plane_point(pl[0]);
  if (n >= 3) {
    f3 n1 = xyz(pl[n - 3]), n2 = xyz(pl[n - 2]), n3 = xyz(pl[n - 1]);
    float det = dot(n1, cross(n2, n3));
    if (fabsf(det) > 1e-4f) {
      float e1 = -pl[n - 3].w, e2 = -pl[n - 2].w, e3 = -pl[n - 1].w;
      return ((e1 * cross(n2, n3) + e2 * cross(n3, n1)) + e3 * cross(n1, n2)) / det;
    }
  }
  float4 a = pl[n - 2], b = pl[n - 1];
  f3 L = cross(xyz(a), xyz(b));
  float l2 = dot(L, L);
  if (l2 > 1e-8f) {
    float e1 = -a.w, e2 = -b.w;
    return (e1 * cross(xyz(b), L) + e2 * cross(L, xyz(a))) / l2;
  }
  return plane_point(b);
}
__device__ __forceinline__ float tri_flux(f3 a, f3 b, f3 c, f3 o) { return dot(a - o, cross(b - o, c - o)) / 6.0f; }
__device__ __forceinline__ float edge_term(f3 p, f3 q, f3 c, f3 o) { return dot(c - o, cross(q - o, p - o)) / 6.0f; }

__device__ __forceinline__ void put_edge(uint32_t* E, size_t e, f3 p, f3 q, uint32_t pl) {
  uint4* w = reinterpret_cast<uint4*>(E + 8 * e);
  w[0] = make_uint4(__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(p.z), __float_as_uint(q.x));
  w[1] = make_uint4(__float_as_uint(q.y), __float_as_uint(q.z), pl, 0u);
}
__device__ __forceinline__ void get_edge(const uint32_t* E, size_t e, f3& p, f3& q, uint32_t& pl) {
  const uint4* w = reinterpret_cast<const uint4*>(E + 8 * e);
  uint4 a = w[0], b = w[1];
  p = mk3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
  q = mk3(__uint_as_float(a.w), __uint_as_float(b.x), __uint_as_float(b.y));
  pl = b.z;
}

// ======================= plan (shaders.ts:296-444) =======================
template <int G>
__global__ void __launch_bounds__(256) k_plan(const Level P, const Dev D) {
  __shared__ GrpSmem gsm[Grp<G>::PER_BLOCK];
  __shared__ uint32_t hdr[Grp<G>::PER_BLOCK][12];
  const int gi = Grp<G>::gid(), lid = Grp<G>::lid();
  GrpSmem& sm = gsm[gi];
  uint32_t* H = hdr[gi];
  const uint32_t g = blockIdx.x * Grp<G>::PER_BLOCK + gi;
  if (g >= P.nJobs) return;
  const uint32_t itemIdx = g / P.totalWidth, cut = g % P.totalWidth, jobIdx = P.jobBase + g;
  Job* J = D.jobs + jobIdx;
  if (lid == 0) {
    uint4* jw = reinterpret_cast<uint4*>(J);
#pragma unroll
    for (int k = 0; k < 6; k++) jw[k] = make_uint4(0, 0, 0, 0);
    J->parentItem = itemIdx;
    J->cutIdx = cut;
    D.planes[jobIdx] = make_float4(0.f, 0.f, 0.f, 0.f);
    const ItemDesc* it = D.items + P.itemsInBase + itemIdx;
    uint32_t flags = it->flags, np = it->np;
    uint32_t ok = (flags == 1 && np > 0) ? 1u : 0u;
    H[0] = ok;
    if (ok) {
      uint32_t partId = it->partIds[np - 1];
      const PartDesc* pd = D.parts + partId;
      J->parentPart = partId;
      H[1] = pd->vOff; H[2] = pd->nv; H[3] = pd->tOff; H[4] = pd->nt; H[5] = pd->eOff; H[6] = pd->ne;
      H[7] = it->srcPart;
    }
  }
  Grp<G>::sync();
  if (H[0] == 0) return;
  const uint32_t vOff = H[1], nv = H[2], tOff = H[3], nt = H[4], eOff = H[5], ne = H[6], srcPart = H[7];
  // bounding box
  f3 lo = mk3(1e30f, 1e30f, 1e30f), hi = mk3(-1e30f, -1e30f, -1e30f);
  for (uint32_t i = lid; i < nv; i += G) {
    f3 p = ldv(D.V, (size_t)vOff + 3 * (size_t)i);
    lo = vmin3(lo, p);
    hi = vmax3(hi, p);
  }
  lo.x = grp_min_f<G>(lo.x, sm); lo.y = grp_min_f<G>(lo.y, sm); lo.z = grp_min_f<G>(lo.z, sm);
  hi.x = grp_max_f<G>(hi.x, sm); hi.y = grp_max_f<G>(hi.y, sm); hi.z = grp_max_f<G>(hi.z, sm);
  f3 ext = hi - lo;
  float lim = 2.0f * P.minEdgeDist + 1e-6f;
  if (ext.x <= lim && ext.y <= lim && ext.z <= lim) {
    // too small to cut on every axis: the item becomes a leaf with zero cost
    // for the remaining levels
    if (cut == 0 && lid == 0) {
      ItemDesc* it = D.items + P.itemsInBase + itemIdx;
      uint32_t lvl = min(P.totalLevels, 4u);
      for (uint32_t l = it->nLevels; l < lvl; l++) it->levelCosts[l] = 0.0f;
      it->nLevels = lvl;
      it->flags = 2;
    }
    return;
  }
  // the plane (every lane computes the same value)
  float4 pl = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t ok = 1;
  if (cut >= P.width) {
    pl = D.planes[P.edgePlaneBase + srcPart * P.edgeStride + (cut - P.width)];
    ok = dot(xyz(pl), xyz(pl)) > 0.0f ? 1u : 0u;
  } else {
    uint32_t cpa = P.width / 3;
    uint32_t axis = cut / cpa, slice = cut % cpa;
    float loV = comp(lo, axis) + P.minEdgeDist;
    float hiV = comp(hi, axis) - P.minEdgeDist;
    if (loV >= hiV) ok = 0;
    float frac = ((float)slice + 1.0f) / ((float)cpa + 1.0f);
    float pos = loV + frac * (hiV - loV);
    pl = make_float4(axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f, -pos);
  }
  uint32_t sOff = 0;
  if (lid == 0 && ok) {
    sOff = atomicAdd(D.ctr + CTR_S, 2 * nv);
    if ((uint64_t)sOff + 2 * (uint64_t)nv > D.sCap) {
      ok = 0;
      atomicExch(D.ctr + CTR_OVERFLOW, 1u);
    }
  }
  ok = grp_bcast_u<G>(ok, sm);
  sOff = grp_bcast_u<G>(sOff, sm);
  if (!ok) return;
  const f3 n = xyz(pl);
  uint2* flags2 = reinterpret_cast<uint2*>(D.S + sOff);
  for (uint32_t i = lid; i < nv; i += G) flags2[i] = make_uint2(0, 0);
  Grp<G>::sync();
  uint32_t posT = 0, negT = 0, posNew = 0, negNew = 0, posE = 0, negE = 0;
  for (uint32_t t = lid; t < nt; t += G) {
    const uint32_t* tr = D.T + tOff + 3 * (size_t)t;
    uint32_t i0 = tr[0], i1 = tr[1], i2 = tr[2];
    float d0 = dot(n, ldv(D.V, (size_t)vOff + 3 * (size_t)i0)) + pl.w;
    float d1 = dot(n, ldv(D.V, (size_t)vOff + 3 * (size_t)i1)) + pl.w;
    float d2 = dot(n, ldv(D.V, (size_t)vOff + 3 * (size_t)i2)) + pl.w;
    int sg[3] = {vsign(d0), vsign(d1), vsign(d2)};
    if (sg[0] == 0 && sg[1] == 0 && sg[2] == 0) continue;
    Poly pp = clip_tri(sg[0], sg[1], sg[2], 1), pn = clip_tri(sg[0], sg[1], sg[2], -1);
    uint32_t a, b, c;
    poly_stats(pp, sg, a, b, c);
    posT += a; posNew += b; posE += c;
    poly_stats(pn, sg, a, b, c);
    negT += a; negNew += b; negE += c;
    uint32_t tri[3] = {i0, i1, i2};
    if (pp.n >= 3)
      for (uint32_t i = 0; i < pp.n; i++) if (pp.src[i] < 4) D.S[sOff + 2 * tri[pp.src[i]]] = 1;
    if (pn.n >= 3)
      for (uint32_t i = 0; i < pn.n; i++) if (pn.src[i] < 4) D.S[sOff + 2 * tri[pn.src[i]] + 1] = 1;
  }
  Grp<G>::sync();
  uint32_t posKept = 0, negKept = 0;
  for (uint32_t i = lid; i < nv; i += G) {
    uint2 f = flags2[i];
    posKept += f.x;
    negKept += f.y;
  }
  for (uint32_t e = lid; e < ne; e += G) {
    f3 p, q;
    uint32_t pid;
    get_edge(D.E, (size_t)eOff + e, p, q, pid);
    float dp = dot(n, p) + pl.w, dq = dot(n, q) + pl.w;
    bool sp = dp >= 0.0f, sq = dq >= 0.0f;
    if (sp == sq) { if (sp) posE++; else negE++; }
    else { posE++; negE++; }
  }
  posKept = grp_sum_u<G>(posKept, sm); negKept = grp_sum_u<G>(negKept, sm);
  posT = grp_sum_u<G>(posT, sm); negT = grp_sum_u<G>(negT, sm);
  posNew = grp_sum_u<G>(posNew, sm); negNew = grp_sum_u<G>(negNew, sm);
  posE = grp_sum_u<G>(posE, sm); negE = grp_sum_u<G>(negE, sm);
  if (lid == 0) {
    J->plane = pl;
    J->valid = 1;
    J->cnt[0] = posKept + posNew; J->cnt[1] = posT; J->cnt[2] = posE;
    J->cnt[3] = negKept + negNew; J->cnt[4] = negT; J->cnt[5] = negE;
    J->cnt[6] = posKept; J->cnt[7] = negKept;
    J->off[6] = sOff;
    D.planes[jobIdx] = pl;
    unsigned long long* vc = reinterpret_cast<unsigned long long*>(D.ctr + CTR_VALID_LO);
    atomicAdd(vc, 1ull);
    add_bytes(D.ctr, CTR_BYTES_PLAN, 12ull * nv + 12ull * nt + 32ull * ne);
  }
}

// ======================= scan (shaders.ts:446-554) =======================
// The reference runs this as one serial workgroup. Here it is device-wide:
// k_scan_sums writes each 1024-job block's vertex, triangle and edge needs
// (and the pool tops as the bases); k_scan then gives every block its offset
// from the sums of the blocks before it and scans within the block.
__device__ __forceinline__ void job_needs(const Level& P, const Dev& D, uint32_t j, uint32_t need[3]) {
  need[0] = need[1] = need[2] = 0;
  if (j >= P.nJobs) return;
  const Job* J = D.jobs + P.jobBase + j;
  if (J->valid != 1) return;
  const uint4* cw = reinterpret_cast<const uint4*>(J->cnt);
  uint4 a = cw[0], b = cw[1];
  need[0] = 3 * (a.x + a.w);
  if (P.lastLevel == 0) {
    need[1] = 3 * (a.y + b.x);
    need[2] = a.z + b.y;
  }
}
__global__ void __launch_bounds__(1024) k_scan_sums(const Level P, const Dev D) {
  __shared__ unsigned long long ws[3][32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  uint32_t need[3];
  job_needs(P, D, blockIdx.x * 1024 + tid, need);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    uint32_t s = warp_sum_u(need[k]);
    if (lane == 0) ws[k][w] = s;
  }
  __syncthreads();
  if (tid < 3) {
    unsigned long long s = 0;
    for (int i = 0; i < 32; i++) s += ws[tid][i];
    D.scanTmp[3 + 3 * blockIdx.x + tid] = s;
    if (blockIdx.x == 0) D.scanTmp[tid] = D.ctr[CTR_V + tid];
  }
}
__global__ void __launch_bounds__(1024) k_scan(const Level P, const Dev D) {
  __shared__ uint32_t wsum[3][32];
  __shared__ unsigned long long run[3];
  __shared__ unsigned long long bsum[3][32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  {
    // base = pool tops + needs of all earlier blocks
    unsigned long long s[3] = {0, 0, 0};
    for (uint32_t b = tid; b < blockIdx.x; b += 1024)
      for (int k = 0; k < 3; k++) s[k] += D.scanTmp[3 + 3 * b + k];
    for (int k = 0; k < 3; k++) {
      unsigned long long v = s[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
      if (lane == 0) bsum[k][w] = v;
    }
    __syncthreads();
    if (tid < 3) {
      unsigned long long v = D.scanTmp[tid];
      for (int i = 0; i < 32; i++) v += bsum[tid][i];
      run[tid] = v;
    }
    __syncthreads();
  }
  const bool keepTopo = P.lastLevel == 0;
  uint32_t childMax = 0;
  {
    const uint32_t c = blockIdx.x;
    const uint32_t j = c * 1024 + tid;
    const bool inRange = j < P.nJobs;
    Job* J = D.jobs + P.jobBase + (inRange ? j : 0);
    uint32_t cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t jv = 0;
    if (inRange) {
      jv = J->valid == 1 ? 1u : 0u;
      const uint4* cw = reinterpret_cast<const uint4*>(J->cnt);
      uint4 a = cw[0], b = cw[1];
      cnt[0] = a.x; cnt[1] = a.y; cnt[2] = a.z; cnt[3] = a.w; cnt[4] = b.x; cnt[5] = b.y; cnt[6] = b.z; cnt[7] = b.w;
    }
    uint32_t need[3];
    need[0] = jv ? 3 * (cnt[0] + cnt[3]) : 0;
    need[1] = (jv && keepTopo) ? 3 * (cnt[1] + cnt[4]) : 0;
    need[2] = (jv && keepTopo) ? cnt[2] + cnt[5] : 0;
    uint32_t incl[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      incl[k] = warp_incl_u(need[k], lane);
      if (lane == 31) wsum[k][w] = incl[k];
    }
    __syncthreads();
    unsigned long long off[3], tot[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      unsigned long long before = 0, all = 0;
      for (int i = 0; i < 32; i++) {
        uint32_t t = wsum[k][i];
        if (i < w) before += t;
        all += t;
      }
      off[k] = run[k] + before + incl[k] - need[k];
      tot[k] = all;
    }
    __syncthreads();
    if (tid == 0) { run[0] += tot[0]; run[1] += tot[1]; run[2] += tot[2]; }
    if (inRange) {
      bool valid = jv != 0;
      if (valid && (off[0] + need[0] > D.vCap || off[1] + need[1] > D.tCap || off[2] + need[2] > D.eCap)) {
        valid = false;
        atomicExch(D.ctr + CTR_OVERFLOW, 1u);
      }
      const uint32_t posP = P.partBase + 2 * j, negP = posP + 1, outIdx = P.itemsOutBase + j;
      ItemDesc it;
      {
        uint32_t* iw = reinterpret_cast<uint32_t*>(&it);
        for (int k = 0; k < 20; k++) iw[k] = 0;
      }
      if (valid) {
        const uint32_t vOff = (uint32_t)off[0], tOff = (uint32_t)off[1], eOff = (uint32_t)off[2];
        const uint32_t parentItem = J->parentItem, parentPart = J->parentPart, cutIdx = J->cutIdx;
        const ItemDesc parent = D.items[P.itemsInBase + parentItem];
        const PartDesc pp = D.parts[parentPart];
        J->off[0] = vOff; J->off[1] = tOff; J->off[2] = eOff;
        J->off[3] = vOff + 3 * cnt[0];
        J->off[4] = keepTopo ? tOff + 3 * cnt[1] : tOff;
        J->off[5] = keepTopo ? eOff + cnt[2] : eOff;
        PartDesc pd;
        pd.planeIds[0] = pp.planeIds[0]; pd.planeIds[1] = pp.planeIds[1];
        pd.planeIds[2] = pp.planeIds[2]; pd.planeIds[3] = pp.planeIds[3];
        pd.nPlanes = pp.nPlanes;
        if (pd.nPlanes < 4) { pd.planeIds[pd.nPlanes] = P.jobBase + j; pd.nPlanes++; }
        else { pd.planeIds[0] = pp.planeIds[1]; pd.planeIds[1] = pp.planeIds[2]; pd.planeIds[2] = pp.planeIds[3]; pd.planeIds[3] = P.jobBase + j; }
        pd.meshVol = 0.0f; pd.hullVol = 0.0f; pd.flags = keepTopo ? 0u : 2u; pd.pad0 = 0; pd.pad1 = 0;
        PartDesc pos = pd, neg = pd;
        pos.vOff = vOff; pos.nv = cnt[0]; pos.tOff = tOff; pos.nt = keepTopo ? cnt[1] : 0;
        pos.eOff = eOff; pos.ne = keepTopo ? cnt[2] : 0;
        neg.vOff = vOff + 3 * cnt[0]; neg.nv = cnt[3]; neg.tOff = keepTopo ? tOff + 3 * cnt[1] : tOff;
        neg.nt = keepTopo ? cnt[4] : 0; neg.eOff = keepTopo ? eOff + cnt[2] : eOff; neg.ne = keepTopo ? cnt[5] : 0;
        D.parts[posP] = pos;
        D.parts[negP] = neg;
        childMax = max(cnt[0], cnt[3]);
        const bool bothNonEmpty = cnt[0] > 0 && cnt[1] > 0 && cnt[3] > 0 && cnt[4] > 0;
        it = parent;
        if (parent.np >= 8) {
          atomicExch(D.ctr + CTR_NPOVER, 1u);
          it.flags = 0;
        } else if (bothNonEmpty) {
          it.partIds[parent.np - 1] = posP;
          it.partIds[parent.np] = negP;
          it.np = parent.np + 1;
          it.flags = 1;
          it.parentItem = parentItem;
          it.cutIdx = cutIdx;
          if (parent.nLevels == 0) it.initialCut = cutIdx;
        } else {
          it.flags = 0;
          J->valid = 2;  // empty half: cut discarded
        }
      } else {
        if (inRange) J->valid = 0;
        PartDesc z;
        uint32_t* zw = reinterpret_cast<uint32_t*>(&z);
        for (int k = 0; k < 16; k++) zw[k] = 0;
        D.parts[posP] = z;
        D.parts[negP] = z;
      }
      D.items[outIdx] = it;
    }
    __syncthreads();
  }
  // the level's largest child: hull launches for large parts skip levels
  // without any
  childMax = __reduce_max_sync(FULLMASK, childMax);
  if (lane == 0 && childMax != 0) atomicMax(D.work + 32 + P.workSlot, childMax);
  if (tid == 0 && blockIdx.x == gridDim.x - 1) {
    // the last block holds the level's totals; the bases were read from the
    // copy k_scan_sums made, so the counters can move now
    D.ctr[CTR_V] = (uint32_t)min(run[0], (unsigned long long)D.vCap);
    D.ctr[CTR_T] = (uint32_t)min(run[1], (unsigned long long)D.tCap);
    D.ctr[CTR_E] = (uint32_t)min(run[2], (unsigned long long)D.eCap);
    D.ctr[CTR_S] = 0;
  }
}

// ======================= emit (shaders.ts:556-750) =======================
template <int G>
__global__ void __launch_bounds__(256) k_emit(const Level P, const Dev D) {
  __shared__ GrpSmem gsm[Grp<G>::PER_BLOCK];
  const int gi = Grp<G>::gid(), lid = Grp<G>::lid();
  GrpSmem& sm = gsm[gi];
  const uint32_t g = blockIdx.x * Grp<G>::PER_BLOCK + gi;
  if (g >= P.nJobs) return;
  const uint32_t jobIdx = P.jobBase + g;
  const Job* J = D.jobs + jobIdx;
  if (J->valid != 1) return;  // written by scan, uniform for the group
  const PartDesc part = D.parts[J->parentPart];
  const float4 pl = J->plane;
  const f3 n = xyz(pl);
  const f3 cP = plane_point(pl);
  float4 pls[4];
  uint32_t npl = 0;
  for (uint32_t k = 0; k < part.nPlanes; k++) pls[npl++] = D.planes[part.planeIds[k]];
  if (npl < 4) pls[npl++] = pl;
  else { pls[0] = pls[1]; pls[1] = pls[2]; pls[2] = pls[3]; pls[3] = pl; }
  const f3 o = anchor_for(pls, npl);
  const uint32_t posV = J->off[0], posTo = J->off[1], posEo = J->off[2];
  const uint32_t negV = J->off[3], negTo = J->off[4], negEo = J->off[5];
  const uint32_t sOff = J->off[6];
  const uint32_t posKept = J->cnt[6], negKept = J->cnt[7];
  const bool keepTopo = P.lastLevel == 0;
  uint2* flags2 = reinterpret_cast<uint2*>(D.S + sOff);

  // 1. vertex remap (side flags -> compact indices) and copy of kept vertices
  uint32_t runP = 0, runN = 0;
  for (uint32_t c = 0; c * G < part.nv; c++) {
    const uint32_t i = c * G + lid;
    uint32_t fp = 0, fn = 0;
    f3 p = mk3(0.f, 0.f, 0.f);
    if (i < part.nv) {
      uint2 f = flags2[i];
      fp = f.x;
      fn = f.y;
      p = ldv(D.V, (size_t)part.vOff + 3 * (size_t)i);
    }
    uint32_t totP, totN;
    uint32_t preP = grp_scan_u<G>(fp, &totP, sm);
    uint32_t preN = grp_scan_u<G>(fn, &totN, sm);
    if (i < part.nv) {
      uint32_t ip = CUACD_NONE, in = CUACD_NONE;
      if (fp == 1) { ip = runP + preP; stv(D.V, (size_t)posV + 3 * (size_t)ip, p); }
      if (fn == 1) { in = runN + preN; stv(D.V, (size_t)negV + 3 * (size_t)in, p); }
      flags2[i] = make_uint2(ip, in);
    }
    runP += totP;
    runN += totN;
  }
  Grp<G>::sync();

  // 2. triangles
  KSum fluxP, fluxN;
  fluxP.init();
  fluxN.init();
  uint32_t rT[2] = {0, 0}, rV[2] = {0, 0}, rE[2] = {0, 0};
  for (uint32_t c = 0; c * G < part.nt; c++) {
    const uint32_t t = c * G + lid;
    uint32_t tri[3] = {0, 0, 0};
    f3 pos3[3];
    float d[3] = {0.f, 0.f, 0.f};
    int sg[3] = {0, 0, 0};
    Poly polys[2];
    polys[0].n = 0;
    polys[1].n = 0;
    uint32_t st[2][3] = {{0, 0, 0}, {0, 0, 0}};
    bool live = false;
    if (t < part.nt) {
      const uint32_t* tr = D.T + part.tOff + 3 * (size_t)t;
      tri[0] = tr[0]; tri[1] = tr[1]; tri[2] = tr[2];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        pos3[k] = ldv(D.V, (size_t)part.vOff + 3 * (size_t)tri[k]);
        d[k] = dot(n, pos3[k]) + pl.w;
        sg[k] = vsign(d[k]);
      }
      live = !(sg[0] == 0 && sg[1] == 0 && sg[2] == 0);
      if (live) {
        polys[0] = clip_tri(sg[0], sg[1], sg[2], 1);
        polys[1] = clip_tri(sg[0], sg[1], sg[2], -1);
        poly_stats(polys[0], sg, st[0][0], st[0][1], st[0][2]);
        poly_stats(polys[1], sg, st[1][0], st[1][1], st[1][2]);
      }
    }
    uint32_t tot[2];
    uint32_t pre[2];
    pre[0] = grp_scan_u<G>(st[0][0] | (st[0][1] << 10) | (st[0][2] << 20), &tot[0], sm);
    pre[1] = grp_scan_u<G>(st[1][0] | (st[1][1] << 10) | (st[1][2] << 20), &tot[1], sm);
    if (live) {
      for (int side = 0; side < 2; side++) {
        const Poly& poly = polys[side];
        if (poly.n < 3) continue;
        const bool isPos = side == 0;
        const uint32_t vOff = isPos ? posV : negV, tOff = isPos ? posTo : negTo, eOff = isPos ? posEo : negEo;
        uint32_t tB = rT[side] + (pre[side] & 1023u);
        uint32_t vB = (isPos ? posKept : negKept) + rV[side] + ((pre[side] >> 10) & 1023u);
        uint32_t eB = rE[side] + (pre[side] >> 20);
        uint32_t idx[4];
        f3 pts[4];
        bool onp[4];
        for (uint32_t i = 0; i < poly.n; i++) {
          uint32_t u = poly.src[i];
          if (u < 4) {
            idx[i] = D.S[sOff + 2 * tri[u] + (isPos ? 0 : 1)];
            pts[i] = pos3[u];
            onp[i] = sg[u] == 0;
          } else {
            uint32_t k = u - 4, q = k == 2 ? 0 : k + 1;
            float tt = d[k] / (d[k] - d[q]);
            f3 x = pos3[k] + tt * (pos3[q] - pos3[k]);
            stv(D.V, (size_t)vOff + 3 * (size_t)vB, x);
            idx[i] = vB++;
            pts[i] = x;
            onp[i] = true;
          }
        }
        float flux = 0.0f;
        for (uint32_t i = 1; i + 1 < poly.n; i++) {
          if (keepTopo) {
            uint32_t* w = D.T + tOff + 3 * (size_t)tB;
            w[0] = idx[0]; w[1] = idx[i]; w[2] = idx[i + 1];
          }
          tB++;
          flux += tri_flux(pts[0], pts[i], pts[i + 1], o);
        }
        for (uint32_t i = 0; i < poly.n; i++) {
          uint32_t j2 = (i + 1) % poly.n;
          if (onp[i] && onp[j2]) {
            if (keepTopo) put_edge(D.E, (size_t)eOff + eB, pts[i], pts[j2], jobIdx);
            eB++;
            flux += edge_term(pts[i], pts[j2], cP, o);
          }
        }
        if (isPos) fluxP.add(flux); else fluxN.add(flux);
      }
    }
#pragma unroll
    for (int side = 0; side < 2; side++) {
      rT[side] += tot[side] & 1023u;
      rV[side] += (tot[side] >> 10) & 1023u;
      rE[side] += tot[side] >> 20;
    }
  }

  // 3. inherited open edges, clipped by the new plane
  for (uint32_t c = 0; c * G < part.ne; c++) {
    const uint32_t e = c * G + lid;
    uint32_t cp = 0, cn = 0;
    f3 p = mk3(0.f, 0.f, 0.f), q = p;
    uint32_t pid = 0;
    float dp = 0.f, dq = 0.f;
    if (e < part.ne) {
      get_edge(D.E, (size_t)part.eOff + e, p, q, pid);
      dp = dot(n, p) + pl.w;
      dq = dot(n, q) + pl.w;
      bool sp = dp >= 0.0f, sq = dq >= 0.0f;
      if (sp == sq) { cp = sp ? 1 : 0; cn = 1 - cp; } else { cp = 1; cn = 1; }
    }
    uint32_t totP, totN;
    uint32_t preP = grp_scan_u<G>(cp, &totP, sm);
    uint32_t preN = grp_scan_u<G>(cn, &totN, sm);
    if (e < part.ne) {
      f3 cE = plane_point(D.planes[pid]);
      bool sp = dp >= 0.0f, sq = dq >= 0.0f;
      size_t ep = (size_t)posEo + rE[0] + preP, en = (size_t)negEo + rE[1] + preN;
      if (sp == sq) {
        if (sp) { if (keepTopo) put_edge(D.E, ep, p, q, pid); fluxP.add(edge_term(p, q, cE, o)); }
        else { if (keepTopo) put_edge(D.E, en, p, q, pid); fluxN.add(edge_term(p, q, cE, o)); }
      } else {
        float tt = dp / (dp - dq);
        f3 x = p + tt * (q - p);
        if (sp) {
          if (keepTopo) { put_edge(D.E, ep, p, x, pid); put_edge(D.E, en, x, q, pid); }
          fluxP.add(edge_term(p, x, cE, o));
          fluxN.add(edge_term(x, q, cE, o));
        } else {
          if (keepTopo) { put_edge(D.E, en, p, x, pid); put_edge(D.E, ep, x, q, pid); }
          fluxN.add(edge_term(p, x, cE, o));
          fluxP.add(edge_term(x, q, cE, o));
        }
      }
    }
    rE[0] += totP;
    rE[1] += totN;
  }
  double vp = grp_sum_d<G>(fluxP.value(), sm);
  double vn = grp_sum_d<G>(fluxN.value(), sm);
  if (lid == 0) {
    unsigned long long b = 12ull * part.nv + 12ull * part.nt + 32ull * part.ne + 12ull * (J->cnt[0] + J->cnt[3]);
    if (keepTopo) b += 12ull * (J->cnt[1] + J->cnt[4]) + 32ull * (J->cnt[2] + J->cnt[5]);
    add_bytes(D.ctr, CTR_BYTES_EMIT, b);
    D.parts[P.partBase + 2 * g].meshVol = (float)fabs(vp);
    D.parts[P.partBase + 2 * g + 1].meshVol = (float)fabs(vn);
  }
}

// ============ last-level pruning bound per seed (shaders.ts:1300-1315) ============
// The reference's hull kernel computes, for every part of the last level, the
// best completed-path upper bound over its seed's parent-level items; the
// bound is the same for every part of a seed, so one warp per seed computes
// it once (same operations, same float32 rounding) and the hulls read it.
__global__ void __launch_bounds__(256) k_seed_bound(const Level P, const Dev D) {
  const uint32_t s = blockIdx.x * 8 + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31;
  if (s >= P.nSeeds) return;
  const uint32_t perSeed = P.nItemsIn / P.nSeeds;
  float ubMin = 1e30f;
  for (uint32_t i = lane; i < perSeed; i += 32) {
    const ItemDesc* it = D.items + P.itemsInBase + s * perSeed + i;
    if (it->flags == 1 && it->nLevels > 0) {
      float ps = 0.0f;
      for (uint32_t l = 0; l < it->nLevels; l++) ps += it->levelCosts[l];
      const float u = ps + it->levelCosts[it->nLevels - 1] * (float)(P.totalLevels - it->nLevels);
      ubMin = fminf(ubMin, u);
    }
  }
  ubMin = warp_min_f(ubMin);
  if (lane == 0) D.ub[s] = ubMin;
}
void launch_seed_bound(const Level& P, const Dev& D, cudaStream_t s) {
  k_seed_bound<<<(P.nSeeds + 7) / 8, 256, 0, s>>>(P, D);
}

// ======================= record (shaders.ts:1519-1544) =======================
__global__ void __launch_bounds__(256) k_record(const Level P, const Dev D) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= P.nJobs) return;
  ItemDesc* itp = D.items + P.itemsOutBase + g;
  ItemDesc it = *itp;
  if (it.flags != 1) return;
  float costs[8];
  bool bad = false;
  for (uint32_t i = 0; i < it.np; i++) {
    const PartDesc* pd = D.parts + it.partIds[i];
    float hv = pd->hullVol;
    if (hv < 0.0f || (pd->flags & 4) != 0) bad = true;
    costs[i] = rv_cost(pd->meshVol, hv);
  }
  if (bad) { itp->flags = 0; return; }
  for (uint32_t i = 1; i < it.np; i++) {
    float kc = costs[i];
    uint32_t kp = it.partIds[i];
    uint32_t j = i;
    while (j > 0 && costs[j - 1] > kc) { costs[j] = costs[j - 1]; it.partIds[j] = it.partIds[j - 1]; j--; }
    costs[j] = kc;
    it.partIds[j] = kp;
  }
  if (it.nLevels < 4) { it.levelCosts[it.nLevels] = costs[it.np - 1]; it.nLevels++; }
  *itp = it;
}

// ======================= evaluate (shaders.ts:1404-1517) =======================
// One warp per seed. State layout in the planes table at stateBase:
//   [0..4] tree header, [5..9] probe-round header, [16 + 4 s ..] per seed
struct EvalArgs {
  uint32_t stateBase, headerOff, mode, nSeeds, jobBase, edgePlaneBase, edgeStride;
};
__device__ __forceinline__ uint4 ev_u4(const Dev& D, uint32_t i) {
  float4 f = D.planes[i];
  return make_uint4(__float_as_uint(f.x), __float_as_uint(f.y), __float_as_uint(f.z), __float_as_uint(f.w));
}
__device__ __forceinline__ void ev_merge(float& c, uint32_t& cut, float c2, uint32_t cut2) {
  if (c2 < c || (c2 == c && cut2 < cut)) { c = c2; cut = cut2; }
}
__device__ __forceinline__ void ev_warp_argmin(float& c, uint32_t& cut) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float c2 = __shfl_xor_sync(FULLMASK, c, o);
    uint32_t k2 = __shfl_xor_sync(FULLMASK, cut, o);
    ev_merge(c, cut, c2, k2);
  }
}
__global__ void __launch_bounds__(256) k_evaluate(const EvalArgs A, const Dev D) {
  const uint32_t s = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= A.nSeeds) return;
  const uint32_t sb = A.stateBase, hb = sb + A.headerOff;
  const uint4 hdr = ev_u4(D, hb);
  const uint32_t depth = hdr.x, w0t = hdr.z, nProbes = hdr.w;
  float bestC = 1e30f;
  uint32_t bestCut = CUACD_NONE;
  for (uint32_t l = 0; l < depth; l++) {
    const uint4 lh = ev_u4(D, hb + 1 + l);
    const uint32_t perSeed = lh.y / A.nSeeds;
    const uint32_t want = l == depth - 1 ? 1u : 2u;
    for (uint32_t i = lane; i < perSeed; i += 32) {
      const ItemDesc* it = D.items + lh.x + s * perSeed + i;
      if (it->flags != want || it->nLevels == 0 || it->initialCut == CUACD_NONE) continue;
      float sum = 0.0f;
      for (uint32_t k = 0; k < it->nLevels; k++) sum += it->levelCosts[k];
      float c = sum / (float)it->nLevels;
      ev_merge(bestC, bestCut, c, it->initialCut);
    }
  }
  ev_warp_argmin(bestC, bestCut);
  if (bestCut == CUACD_NONE) {
    const uint4 lh = ev_u4(D, hb + 1);
    const uint32_t perSeed = lh.y / A.nSeeds;
    bestC = 1e30f;
    for (uint32_t i = lane; i < perSeed; i += 32) {
      const ItemDesc* it = D.items + lh.x + s * perSeed + i;
      if (it->flags == 1 && it->nLevels >= 1 && it->initialCut != CUACD_NONE) ev_merge(bestC, bestCut, it->levelCosts[0], it->initialCut);
    }
    ev_warp_argmin(bestC, bestCut);
  }
  if (lane != 0) return;
  const uint32_t cut = bestCut;
  const float cost = bestC;
  const uint32_t st = sb + 16 + 4 * s;
  float4 plane = D.planes[st];
  float4 s1 = D.planes[st + 1];
  float half = s1.y;
  bool valid = (__float_as_uint(s1.w) & 1u) != 0;
  if (A.mode == 0) {
    valid = cut != CUACD_NONE;
    if (valid) plane = D.planes[A.jobBase + s * w0t + cut];
    s1 = make_float4(valid ? cost : 1e30f, half, __uint_as_float(cut), __uint_as_float(valid ? 1u : 0u));
    half = D.planes[st + 2].x;
  } else {
    if (cut != CUACD_NONE && cost < s1.x - 1e-7f) {
      plane = D.planes[A.jobBase + s * w0t + cut];
      s1 = make_float4(cost, s1.y, __uint_as_float(cut), s1.w);
    }
    half = nProbes > 1 ? 2.0f * half / (float)(nProbes - 1) : 0.0f;
  }
  s1.y = half;
  D.planes[st] = plane;
  D.planes[st + 1] = s1;
  for (uint32_t i = 0; i < nProbes; i++) {
    float4 pp = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid && half > 0.0f && nProbes > 1) {
      float off = half * ((2.0f * (float)i) / (float)(nProbes - 1) - 1.0f);
      pp = make_float4(plane.x, plane.y, plane.z, plane.w - off);
    }
    D.planes[A.edgePlaneBase + s * A.edgeStride + i] = pp;
  }
}

// ======================= launchers =======================
void launch_plan(const Level& P, const Dev& D, bool big, cudaStream_t s) {
  if (P.nJobs == 0) return;
  if (big) k_plan<256><<<P.nJobs, 256, 0, s>>>(P, D);
  else k_plan<32><<<(P.nJobs + 7) / 8, 256, 0, s>>>(P, D);
}
void launch_scan(const Level& P, const Dev& D, cudaStream_t s) {
  if (P.nJobs == 0) return;
  const uint32_t blocks = (P.nJobs + 1023) / 1024;
  k_scan_sums<<<blocks, 1024, 0, s>>>(P, D);
  k_scan<<<blocks, 1024, 0, s>>>(P, D);
}
void launch_emit(const Level& P, const Dev& D, bool big, cudaStream_t s) {
  if (P.nJobs == 0) return;
  if (big) k_emit<256><<<P.nJobs, 256, 0, s>>>(P, D);
  else k_emit<32><<<(P.nJobs + 7) / 8, 256, 0, s>>>(P, D);
}
void launch_record(const Level& P, const Dev& D, cudaStream_t s) {
  if (P.nJobs == 0) return;
  k_record<<<(P.nJobs + 255) / 256, 256, 0, s>>>(P, D);
}
void launch_evaluate(uint32_t stateBase, uint32_t headerOff, uint32_t mode, uint32_t nSeeds, uint32_t jobBase,
                     uint32_t edgePlaneBase, uint32_t edgeStride, const Dev& D, cudaStream_t s) {
  EvalArgs A{stateBase, headerOff, mode, nSeeds, jobBase, edgePlaneBase, edgeStride};
  k_evaluate<<<(nSeeds + 7) / 8, 256, 0, s>>>(A, D);
}

}  // namespace cuacd
