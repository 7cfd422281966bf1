// concave_kernels.cu — candidate cutting planes from concave mesh edges
// (src/cpu/concave.ts:25-92) on the GPU, for a batch of meshes.
//
// The planes are the host restatement's (csrc/host_mesh.cpp) bit for bit:
//   degree     one thread per directed edge: out-degree of every vertex; a
//              scan gives each vertex's edge list (the directed-edge CSR of
//              mesh.ts:79-98, each list in arbitrary order);
//   edges      one thread per vertex v0: its distinct partners v1 > v0 in
//              ascending order, the lowest face holding v0 -> v1 and the
//              lowest holding v1 -> v0 (the CSR's first entries, which are
//              in face order), the dihedral angle, and the concave edges
//              stored in (v0, v1) order; a scan of the per-vertex counts
//              lists every mesh's concave edges in that order;
//   reservoir  one thread per mesh: the reference's seeded LCG reservoir
//              (concave.ts:37-74) over the ordered concave edges, then two
//              face-offset planes and, unless the normals are nearly
//              opposite, two bisector planes per kept edge.
// Everything is double arithmetic on float32 inputs compiled with
// --fmad=false (the host restatement compiles without contraction); the
// dihedral angle uses CUDA's acos where the host uses the C library's: both
// are within an ulp, so only an edge whose dihedral lies within an ulp of
// the threshold could be classified differently.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cuacd.h"
#include "concave_engine.h"
#include "dev_ptr.h"
#include "dev_scan.cuh"

#define CONC_NONE 0xffffffffu

namespace cuacd {
int set_error(int code, const char* msg);

namespace conc {

struct MeshDesc {
  uint32_t vOff, nv, tOff, nt;  // the mesh in the input pools
  uint32_t vBase, eBase;        // its ranges in the per-vertex and per-directed-edge scratch
  uint32_t seed, pad;
};

struct EdgeRec {
  uint32_t v0, v1, f0, f1;
};

__device__ __forceinline__ uint32_t find_seg(const uint32_t* __restrict__ pre, uint32_t n, uint32_t g) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (pre[mid] <= g) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void k_degree(const MeshDesc* __restrict__ M, const uint32_t* __restrict__ ePre, uint32_t nm, uint32_t total,
                         const uint32_t* __restrict__ T, uint32_t* __restrict__ deg) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const MeshDesc& m = M[find_seg(ePre, nm, g)];
  const uint32_t e = g - m.eBase;
  atomicAdd(deg + m.vBase + T[3 * (size_t)m.tOff + e], 1u);
}

// list entry: (destination vertex, face) of a directed edge
__global__ void k_fill(const MeshDesc* __restrict__ M, const uint32_t* __restrict__ ePre, uint32_t nm, uint32_t total,
                       const uint32_t* __restrict__ T, const uint32_t* __restrict__ off, uint32_t* __restrict__ fill,
                       uint2* __restrict__ list) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const MeshDesc& m = M[find_seg(ePre, nm, g)];
  const uint32_t e = g - m.eBase, t = e / 3, k = e % 3;
  const uint32_t* tri = T + 3 * ((size_t)m.tOff + t);
  const uint32_t a = tri[k], b = tri[(k + 1) % 3];
  const uint32_t at = atomicAdd(fill + m.vBase + a, 1u);
  list[off[m.vBase + a] + at] = make_uint2(b, t);
}

__device__ __forceinline__ bool face_normal(const float* V, const uint32_t* T, uint32_t f, double n[3]) {
  const uint32_t* tri = T + 3 * (size_t)f;
  const float* A = V + 3 * (size_t)tri[0];
  const float* B = V + 3 * (size_t)tri[1];
  const float* C = V + 3 * (size_t)tri[2];
  const double e1x = (double)B[0] - A[0], e1y = (double)B[1] - A[1], e1z = (double)B[2] - A[2];
  const double e2x = (double)C[0] - A[0], e2y = (double)C[1] - A[1], e2z = (double)C[2] - A[2];
  const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  const double l = sqrt(nx * nx + ny * ny + nz * nz);
  if (l < 1e-12) return false;
  n[0] = nx / l;
  n[1] = ny / l;
  n[2] = nz / l;
  return true;
}

// the lowest face of directed edge a -> b, CONC_NONE when absent
__device__ __forceinline__ uint32_t first_face(const uint2* list, const uint32_t* off, uint32_t base, uint32_t a,
                                               uint32_t b) {
  uint32_t f = CONC_NONE;
  for (uint32_t k = off[base + a]; k < off[base + a + 1]; k++)
    if (list[k].x == b) f = min(f, list[k].y);
  return f;
}

__global__ void k_edges(const MeshDesc* __restrict__ M, const uint32_t* __restrict__ vPre, uint32_t nm, uint32_t total,
                        const float* __restrict__ Vpool, const uint32_t* __restrict__ Tpool,
                        const uint32_t* __restrict__ off, const uint2* __restrict__ list, double thr,
                        EdgeRec* __restrict__ slots, uint32_t* __restrict__ cnt) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const MeshDesc& m = M[find_seg(vPre, nm, g)];
  const uint32_t v0 = g - m.vBase;
  const float* V = Vpool + 3 * (size_t)m.vOff;
  const uint32_t* T = Tpool + 3 * (size_t)m.tOff;
  const uint32_t s0 = off[g], s1 = off[g + 1];
  uint32_t n = 0, last = v0;
  for (;;) {
    // the next partner above `last`, in ascending order
    uint32_t v1 = CONC_NONE;
    for (uint32_t k = s0; k < s1; k++) {
      const uint32_t b = list[k].x;
      if (b > last && b < v1) v1 = b;
    }
    if (v1 == CONC_NONE) break;
    last = v1;
    const uint32_t fa = first_face(list, off, m.vBase, v0, v1), fb = first_face(list, off, m.vBase, v1, v0);
    if (fa == CONC_NONE || fb == CONC_NONE) continue;
    const uint32_t f0 = min(fa, fb), f1 = max(fa, fb);
    double n0[3], n1[3];
    if (!face_normal(V, T, f0, n0) || !face_normal(V, T, f1, n1)) continue;
    double cosA = n0[0] * n1[0] + n0[1] * n1[1] + n0[2] * n1[2];
    cosA = fmax(-1.0, fmin(1.0, cosA));
    const double alpha = acos(cosA);
    uint32_t vOther = CONC_NONE;
    for (int i = 0; i < 3; i++) {
      const uint32_t vv = T[3 * (size_t)f0 + i];
      if (vv != v0 && vv != v1) {
        vOther = vv;
        break;
      }
    }
    if (vOther == CONC_NONE) continue;
    const double dx = (double)V[3 * (size_t)vOther] - V[3 * (size_t)v0];
    const double dy = (double)V[3 * (size_t)vOther + 1] - V[3 * (size_t)v0 + 1];
    const double dz = (double)V[3 * (size_t)vOther + 2] - V[3 * (size_t)v0 + 2];
    const double d = dx * n1[0] + dy * n1[1] + dz * n1[2];
    const double dihedral = d > 0 ? M_PI + alpha : M_PI - alpha;
    if (!(dihedral > thr)) continue;
    EdgeRec r;
    r.v0 = v0;
    r.v1 = v1;
    r.f0 = f0;
    r.f1 = f1;
    slots[s0 + n++] = r;  // at most one per list entry
  }
  cnt[g] = n;
}

__global__ void k_compact(const MeshDesc* __restrict__ M, const uint32_t* __restrict__ vPre, uint32_t nm,
                          uint32_t total, const uint32_t* __restrict__ off, const EdgeRec* __restrict__ slots,
                          const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ cpre,
                          EdgeRec* __restrict__ ordered) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  for (uint32_t j = 0; j < cnt[g]; j++) ordered[cpre[g] + j] = slots[off[g] + j];
}

__global__ void k_reservoir(const MeshDesc* __restrict__ M, uint32_t nm, const float* __restrict__ Vpool,
                            const uint32_t* __restrict__ Tpool, const uint32_t* __restrict__ cpre,
                            const EdgeRec* __restrict__ ordered, int nEdges, double eps, EdgeRec* __restrict__ res,
                            float* __restrict__ out, int32_t* __restrict__ counts) {
  const uint32_t mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= nm) return;
  const MeshDesc& m = M[mi];
  EdgeRec* rs = res + (size_t)mi * nEdges;
  float* o = out + (size_t)mi * 16 * nEdges;
  if (m.nt == 0 || nEdges <= 0) {
    counts[mi] = 0;
    return;
  }
  const uint32_t e0 = cpre[m.vBase], e1 = cpre[m.vBase + m.nv];
  uint32_t rng = m.seed;
  uint32_t nRes = 0;
  double seen = 0;
  for (uint32_t k = e0; k < e1; k++) {
    seen += 1;
    if ((int)nRes < nEdges) {
      rs[nRes++] = ordered[k];
    } else {
      rng = rng * 1664525u + 1013904223u;
      const double thresh = floor((double)nEdges / seen * 4294967295.0);
      if ((double)rng < thresh) {
        rng = rng * 1664525u + 1013904223u;
        rs[rng % (uint32_t)nEdges] = ordered[k];
      }
    }
  }
  const float* V = Vpool + 3 * (size_t)m.vOff;
  const uint32_t* T = Tpool + 3 * (size_t)m.tOff;
  int np = 0;
  for (uint32_t k = 0; k < nRes; k++) {
    const EdgeRec r = rs[k];
    double n0[3], n1[3];
    if (!face_normal(V, T, r.f0, n0) || !face_normal(V, T, r.f1, n1)) continue;
    const double mx = ((double)V[3 * (size_t)r.v0] + V[3 * (size_t)r.v1]) / 2;
    const double my = ((double)V[3 * (size_t)r.v0 + 1] + V[3 * (size_t)r.v1 + 1]) / 2;
    const double mz = ((double)V[3 * (size_t)r.v0 + 2] + V[3 * (size_t)r.v1 + 2]) / 2;
    auto push = [&](double a, double b, double c, double d) {
      o[4 * np] = (float)a;
      o[4 * np + 1] = (float)b;
      o[4 * np + 2] = (float)c;
      o[4 * np + 3] = (float)d;
      np++;
    };
    push(n1[0], n1[1], n1[2], -(n1[0] * mx + n1[1] * my + n1[2] * mz + eps));
    push(n0[0], n0[1], n0[2], -(n0[0] * mx + n0[1] * my + n0[2] * mz + eps));
    double bx = n0[0] + n1[0], by = n0[1] + n1[1], bz = n0[2] + n1[2];
    const double bl = sqrt(bx * bx + by * by + bz * bz);
    if (bl >= 1e-4) {
      bx /= bl;
      by /= bl;
      bz /= bl;
      push(bx, by, bz, -(bx * mx + by * my + bz * mz + eps));
      push(bx, by, bz, -(bx * mx + by * my + bz * mz - eps));
    }
  }
  counts[mi] = np;
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
    if (cudaMalloc(&p, need) != cudaSuccess) return set_error(CUACD_E_CUDA, "concave: device allocation failed");
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
  Buf inV, inT, desc, vPre, ePre, deg, off, fill, list, slots, cnt, cpre, ordered, res, out, counts, tiles;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
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
  for (const Buf* b : {&e->inV, &e->inT, &e->desc, &e->vPre, &e->ePre, &e->deg, &e->off, &e->fill, &e->list, &e->slots,
                       &e->cnt, &e->cpre, &e->ordered, &e->res, &e->out, &e->counts, &e->tiles})
    n += b->bytes;
  return n;
}

#define CONCK(x)                                                                                 \
  do {                                                                                           \
    cudaError_t err_ = (x);                                                                      \
    if (err_ != cudaSuccess)                                                                     \
      return set_error(CUACD_E_CUDA, (std::string("concave: ") + #x + ": " + cudaGetErrorString(err_)).c_str()); \
  } while (0)

static inline uint32_t blocks(uint64_t n, uint32_t t) { return (uint32_t)std::max<uint64_t>(1, (n + t - 1) / t); }

int engine_run(Engine* e, cudaStream_t s, const cuacd_mesh* meshes, int nMeshes, int nConcaveEdges, double eps,
               double thr, const uint32_t* seeds, float* out, int32_t* counts, float* gpuMs) {
  if (!e || nMeshes < 0 || (nMeshes > 0 && (!meshes || !seeds || !out || !counts)))
    return set_error(CUACD_E_INVALID, "concave: invalid argument");
  if (gpuMs) *gpuMs = 0;
  if (nMeshes == 0) return CUACD_OK;
  const int nE = std::max(nConcaveEdges, 0);
  const uint32_t nm = (uint32_t)nMeshes;
  std::vector<MeshDesc> desc(nm);
  std::vector<uint32_t> vPre(nm + 1, 0), ePre(nm + 1, 0);
  uint64_t totV = 0, totT = 0;
  for (uint32_t i = 0; i < nm; i++) {
    const cuacd_mesh& m = meshes[i];
    if ((m.nv && !m.verts) || (m.nt && !m.tris)) return set_error(CUACD_E_INVALID, "concave: null mesh buffer");
    // a device mesh is copied on the device and its indices are the
    // caller's to vouch for; a host mesh is checked
    const bool dv = is_device_ptr(m.verts), dt = is_device_ptr(m.tris);
    if ((m.nv && m.nt && dv != dt) || (!m.nv && dt) || (!m.nt && dv))
      return set_error(CUACD_E_INVALID, "concave: a mesh's buffers must both be host or both be device memory");
    if (!dt)
      for (uint64_t k = 0; k < 3ull * m.nt; k++)
        if (m.tris[k] >= m.nv) return set_error(CUACD_E_INVALID, "concave: triangle index out of range");
    MeshDesc& d = desc[i];
    d.vOff = (uint32_t)totV;
    d.nv = m.nv;
    d.tOff = (uint32_t)totT;
    d.nt = nE > 0 ? m.nt : 0;  // no edges are looked at when no plane is asked for
    d.vBase = (uint32_t)totV;
    d.eBase = 3 * (uint32_t)totT;
    d.seed = seeds[i];
    d.pad = 0;
    totV += m.nv;
    totT += d.nt;
    vPre[i + 1] = (uint32_t)totV;
    ePre[i + 1] = 3 * (uint32_t)totT;
  }
  if (totV >= (1ull << 31) || 3 * totT >= (1ull << 31)) return set_error(CUACD_E_CAPACITY, "concave: batch too large");
  const uint64_t totE = 3 * totT;
  int rc;
  if ((rc = e->inV.ensure(12 * totV)) || (rc = e->inT.ensure(12 * totT)) || (rc = e->desc.ensure(sizeof(MeshDesc) * nm)) ||
      (rc = e->vPre.ensure(4 * (nm + 1))) || (rc = e->ePre.ensure(4 * (nm + 1))) || (rc = e->deg.ensure(4 * totV)) ||
      (rc = e->off.ensure(4 * (totV + 1))) || (rc = e->fill.ensure(4 * totV)) || (rc = e->list.ensure(8 * totE)) ||
      (rc = e->slots.ensure(sizeof(EdgeRec) * totE)) || (rc = e->cnt.ensure(4 * totV)) ||
      (rc = e->cpre.ensure(4 * (totV + 1))) || (rc = e->ordered.ensure(sizeof(EdgeRec) * totE)) ||
      (rc = e->res.ensure(sizeof(EdgeRec) * (size_t)nm * std::max(nE, 1))) ||
      (rc = e->out.ensure(64 * (size_t)nm * std::max(nE, 1))) || (rc = e->counts.ensure(4 * nm)) ||
      (rc = e->tiles.ensure(4 * (scan::tiles_for((uint32_t)totV) + 1))))
    return rc;
  CONCK(cudaEventRecord(e->ev0, s));
  for (uint32_t i = 0; i < nm; i++) {
    const cuacd_mesh& m = meshes[i];
    if (m.nv) CONCK(cudaMemcpyAsync(e->inV.as<float>() + 3 * (size_t)desc[i].vOff, m.verts, 12ull * m.nv, cudaMemcpyDefault, s));
    if (desc[i].nt)
      CONCK(cudaMemcpyAsync(e->inT.as<uint32_t>() + 3 * (size_t)desc[i].tOff, m.tris, 12ull * m.nt, cudaMemcpyDefault, s));
  }
  CONCK(cudaMemcpyAsync(e->desc.p, desc.data(), sizeof(MeshDesc) * nm, cudaMemcpyHostToDevice, s));
  CONCK(cudaMemcpyAsync(e->vPre.p, vPre.data(), 4 * (nm + 1), cudaMemcpyHostToDevice, s));
  CONCK(cudaMemcpyAsync(e->ePre.p, ePre.data(), 4 * (nm + 1), cudaMemcpyHostToDevice, s));
  if (totV) {
    CONCK(cudaMemsetAsync(e->deg.p, 0, 4 * totV, s));
    CONCK(cudaMemsetAsync(e->fill.p, 0, 4 * totV, s));
  }
  const MeshDesc* dM = e->desc.as<MeshDesc>();
  if (totE) k_degree<<<blocks(totE, 256), 256, 0, s>>>(dM, e->ePre.as<uint32_t>(), nm, (uint32_t)totE, e->inT.as<uint32_t>(),
                                                        e->deg.as<uint32_t>());
  scan::exclusive<uint32_t>(e->deg.as<uint32_t>(), (uint32_t)totV, e->off.as<uint32_t>(), e->tiles.as<uint32_t>(), s);
  if (totE) k_fill<<<blocks(totE, 256), 256, 0, s>>>(dM, e->ePre.as<uint32_t>(), nm, (uint32_t)totE, e->inT.as<uint32_t>(),
                                                      e->off.as<uint32_t>(), e->fill.as<uint32_t>(), e->list.as<uint2>());
  if (totV) k_edges<<<blocks(totV, 128), 128, 0, s>>>(dM, e->vPre.as<uint32_t>(), nm, (uint32_t)totV, e->inV.as<float>(),
                                                       e->inT.as<uint32_t>(), e->off.as<uint32_t>(), e->list.as<uint2>(),
                                                       thr, e->slots.as<EdgeRec>(), e->cnt.as<uint32_t>());
  scan::exclusive<uint32_t>(e->cnt.as<uint32_t>(), (uint32_t)totV, e->cpre.as<uint32_t>(), e->tiles.as<uint32_t>(), s);
  if (totV) k_compact<<<blocks(totV, 256), 256, 0, s>>>(dM, e->vPre.as<uint32_t>(), nm, (uint32_t)totV,
                                                         e->off.as<uint32_t>(), e->slots.as<EdgeRec>(),
                                                         e->cnt.as<uint32_t>(), e->cpre.as<uint32_t>(),
                                                         e->ordered.as<EdgeRec>());
  k_reservoir<<<blocks(nm, 64), 64, 0, s>>>(dM, nm, e->inV.as<float>(), e->inT.as<uint32_t>(), e->cpre.as<uint32_t>(),
                                            e->ordered.as<EdgeRec>(), nE, eps, e->res.as<EdgeRec>(), e->out.as<float>(),
                                            e->counts.as<int32_t>());
  CONCK(cudaGetLastError());
  CONCK(cudaMemcpyAsync(counts, e->counts.p, 4 * nm, cudaMemcpyDeviceToHost, s));
  if (nE > 0) CONCK(cudaMemcpyAsync(out, e->out.p, 64 * (size_t)nm * nE, cudaMemcpyDeviceToHost, s));
  CONCK(cudaEventRecord(e->ev1, s));
  CONCK(cudaStreamSynchronize(s));
  if (gpuMs) cudaEventElapsedTime(gpuMs, e->ev0, e->ev1);
  return CUACD_OK;
}

}  // namespace conc
}  // namespace cuacd
