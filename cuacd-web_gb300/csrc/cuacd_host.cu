// cuacd_host.cu — host driver and C ABI of the engine (include/cuacd.h).
//
// Mirrors the reference's GpuTree (src/gpu/tree.ts): device pools sized by
// TreeConfig, per-run tables for up to nSeeds seeds, level layouts of the
// tree and of the refinement rounds, and one submission per run. The whole
// run (seed-table reset, every level's plan / scan / emit / hull / record,
// evaluate, each refinement round) is captured once into a CUDA graph and
// replayed; a graph is reused while the run's layout is unchanged.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/cuacd.h"
#include "cuacd_dev.cuh"
#include "concave_engine.h"
#include "cut_engine.h"
#include "dev_ptr.h"
#include "host_mesh.h"

namespace cuacd {
void launch_plan(const Level& P, const Dev& D, bool big, cudaStream_t s);
void launch_scan(const Level& P, const Dev& D, cudaStream_t s);
void launch_emit(const Level& P, const Dev& D, bool big, cudaStream_t s);
void launch_record(const Level& P, const Dev& D, cudaStream_t s);
void launch_seed_bound(const Level& P, const Dev& D, cudaStream_t s);
void launch_evaluate(uint32_t stateBase, uint32_t headerOff, uint32_t mode, uint32_t nSeeds, uint32_t jobBase,
                     uint32_t edgePlaneBase, uint32_t edgeStride, const Dev& D, cudaStream_t s);
void launch_hull(const Level& P, const Dev& D, int width, cudaStream_t s);
void launch_hd(const HdArgs& A, const Dev& D, cudaStream_t s);
int hull_blocks_per_sm(int width);
}  // namespace cuacd

using namespace cuacd;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
namespace cuacd {
// records the message of a failed call for cuacd_last_error (used by entry
// points defined next to their kernels)
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace cuacd

#define CK(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) return fail(CUACD_E_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

static const uint32_t VIS_MAX = CUACD_VIS_MAX;
// parts with at most SMALL_NV points get a warp per hull, larger ones a
// 256-thread block (narrower blocks for mid-sized parts measured slower: the
// passes over all points and candidates need the width)
static const uint32_t SMALL_NV = 1024;
// parents with more points than this get a block per plan / emit job
static const uint32_t BIG_JOB_NV = 2048;

// Schedules the autotuner chooses between: the largest part a warp hulls
// (larger ones go to blocks) and the largest parent a warp plans and emits.
// The kernels' outputs do not depend on which group shape handles a part,
// so every schedule gives the same results; they differ in speed with the
// distribution of part sizes. The first is the fixed default.
struct Schedule {
  uint32_t smallNv, bigJobNv;
};
static const Schedule kSchedules[] = {{SMALL_NV, BIG_JOB_NV}, {512, BIG_JOB_NV}, {256, BIG_JOB_NV}, {SMALL_NV, 4096}};
static const int kNumSchedules = (int)(sizeof(kSchedules) / sizeof(kSchedules[0]));
// per key: device time of one run or batch under each schedule tried so far
struct TuneEntry {
  float ms[kNumSchedules];
  int tried = 0;
  int best = 0;
};
static uint32_t log2_bucket(uint64_t x) {
  uint32_t b = 0;
  while (b < 63 && (1ull << b) < x) b++;
  return b;
}
// the key of a batch's part-size distribution: log2 buckets of its largest,
// median and total point counts and of its part count, with the kind of
// work (tree run layout or hull batch) in the low bits
static uint64_t size_key(uint64_t kind, const cuacd_mesh* m, int n) {
  std::vector<uint32_t> nv((size_t)std::max(n, 0));
  uint64_t sum = 0;
  uint32_t mx = 0;
  for (int k = 0; k < n; k++) {
    nv[(size_t)k] = m[k].nv;
    sum += m[k].nv;
    mx = std::max(mx, m[k].nv);
  }
  uint32_t med = 0;
  if (n > 0) {
    std::nth_element(nv.begin(), nv.begin() + n / 2, nv.end());
    med = nv[(size_t)n / 2];
  }
  return (kind & 0xffffull) | ((uint64_t)log2_bucket(mx) << 16) | ((uint64_t)log2_bucket(med) << 24) |
         ((uint64_t)log2_bucket(sum) << 32) | ((uint64_t)log2_bucket((uint64_t)std::max(n, 0)) << 40);
}

struct LevelLayout {
  uint32_t itemsInBase, nItemsIn, itemsOutBase, jobBase, partBase, nJobs, width, nEdgeCuts, totalWidth;
};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t need) {
    if (need <= bytes) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (cudaMalloc(&p, need) != cudaSuccess) return fail(CUACD_E_CUDA, "device allocation failed");
    bytes = need;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};
struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t need) {
    if (need <= bytes) return 0;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    if (cudaMallocHost(&p, need) != cudaSuccess) return fail(CUACD_E_CUDA, "pinned allocation failed");
    bytes = need;
    return 0;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
};

struct Tree {
  cuacd_tree_config cfg;
  uint32_t edgeStride = 0;
  int device = 0, nSM = 0, bpsSmall = 1, bpsBig = 1, bpsWide = 0, bpsXL = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool profile = false;
  // profile mode: eager launches with an event after each kernel; kernel
  // classes are reset, plan, scan, emit, hull, record, evaluate
  std::vector<cudaEvent_t> pev;
  std::vector<int> pcls;
  float kernelMs[7] = {0, 0, 0, 0, 0, 0, 0};
  uint64_t bytes[3] = {0, 0, 0};  // algorithmic bytes of plan, emit, hull in the last run
  void mark(int cls) {
    if (!profile) return;
    size_t i = pcls.size();
    if (i >= pev.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pev.push_back(e);
    }
    // inside a stream capture only an external record becomes an event node
    cudaEventRecordWithFlags(pev[i], stream, cudaEventRecordExternal);
    pcls.push_back(cls);
  }
  Dev D{};
  DevBuf bV, bT, bE, bS, bCtr, bSlab, bParts, bItems, bJobs, bPlanes, bSnap, bHd, bScan, bWork, bUb;
  uint32_t workSlots = 0;  // hull launches of the prepared run
  HostBuf hStage, hRead, hSnap, hMeta;
  uint32_t capSeeds = 0, capJobs = 0, capItems = 0, capParts = 0, capPlanes = 0;
  // prepared run
  bool prepared = false;
  uint32_t nSeeds = 0, depth = 0, nProbes = 0, rounds = 0;
  uint32_t vTop = 0, tTop = 0;
  uint32_t slabWords = 0, slabStride = 0, nSlabsSmall = 0, nSlabsBig = 0;
  uint32_t maxSeedNv = 0;
  uint32_t edgePlaneBase = 0, stateBase = 0, lastItems = 0;
  std::vector<LevelLayout> tree, probe;
  size_t snapParts = 0, snapItems = 0, snapCtr = 0, snapEdge = 0, snapState = 0, snapBytes = 0;
  // graph of the prepared run
  cudaGraphExec_t gexec = nullptr;
  std::vector<uint64_t> gsig;
  bool gvalid = false;

  // autotuner (cfg.autotune and no fixed warpMaxNv): each new key tries the
  // schedules in turn on real work, one run or batch each, then keeps the
  // fastest
  std::map<uint64_t, TuneEntry> tuneTable;
  uint64_t tuneKey = 0;
  int sched = 0;
  bool tuneOpen = false;  // the prepared run or batch times a schedule under trial
  bool lastTrial = false;  // the last prepared run or batch tried a schedule
  bool autotuned() const { return cfg.autotune != 0 && cfg.warpMaxNv <= 0; }
  void choose(uint64_t key) {
    tuneKey = key;
    tuneOpen = false;
    lastTrial = false;
    sched = 0;
    if (!autotuned()) return;
    TuneEntry& e = tuneTable[key];
    if (e.tried < kNumSchedules) {
      sched = e.tried;
      tuneOpen = true;
      lastTrial = true;
    } else {
      sched = e.best;
    }
  }
  void record(float ms) {
    if (!tuneOpen) return;
    tuneOpen = false;
    TuneEntry& e = tuneTable[tuneKey];
    if (e.tried != sched) return;
    e.ms[sched] = ms;
    e.tried++;
    if (e.tried == kNumSchedules) {
      e.best = 0;
      for (int k = 1; k < kNumSchedules; k++)
        if (e.ms[k] < e.ms[e.best]) e.best = k;
    }
  }
  uint32_t smallNv() const { return cfg.warpMaxNv > 0 ? (uint32_t)cfg.warpMaxNv : kSchedules[sched].smallNv; }
  uint32_t bigJobNv() const { return kSchedules[sched].bigJobNv; }

  cut::Engine* cutter = nullptr;  // the GPU capped cut, created on first use
  conc::Engine* concave = nullptr;  // the GPU concave-edge planes, created on first use
  float lastConcaveMs = 0.0f;
  float lastEvalMs = 0.0f;        // device time of the last cuacd_tree_eval_cuts

  ~Tree() {
    if (cutter) cut::engine_destroy(cutter);
    if (concave) conc::engine_destroy(concave);
    if (gexec) cudaGraphExecDestroy(gexec);
    for (DevBuf* b : {&bV, &bT, &bE, &bS, &bCtr, &bSlab, &bParts, &bItems, &bJobs, &bPlanes, &bSnap, &bHd, &bScan, &bWork, &bUb}) b->release();
    for (HostBuf* b : {&hStage, &hRead, &hSnap, &hMeta}) b->release();
    for (cudaEvent_t e : pev) cudaEventDestroy(e);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
  void bind() {
    D.V = (float*)bV.p; D.T = (uint32_t*)bT.p; D.E = (uint32_t*)bE.p; D.S = (uint32_t*)bS.p;
    D.slab = (uint32_t*)bSlab.p; D.parts = (PartDesc*)bParts.p; D.items = (ItemDesc*)bItems.p;
    D.jobs = (Job*)bJobs.p; D.planes = (float4*)bPlanes.p; D.ctr = (uint32_t*)bCtr.p;
    D.scanTmp = (unsigned long long*)bScan.p; D.work = (uint32_t*)bWork.p; D.ub = (float*)bUb.p;
    D.vCap = cfg.vertexCap; D.tCap = cfg.triCap; D.eCap = cfg.edgeCap; D.sCap = cfg.scratchWords;
  }
  // tree.ts:191-213
  int ensureTables(uint32_t n) {
    if (n <= capSeeds) return 0;
    uint64_t w0 = (uint64_t)cfg.width + edgeStride, nIn = n, totalJobs = 0;
    for (int l = 0; l < cfg.depth; l++) {
      uint64_t w = l == 0 ? w0 : (uint64_t)cfg.width2;
      totalJobs += nIn * w;
      nIn *= w;
    }
    uint64_t nItems = n + totalJobs;
    uint64_t nParts = std::max<uint64_t>(n + 2 * totalJobs, capParts);
    uint64_t nPlanes = totalJobs + (uint64_t)n * edgeStride + 16 + 4 * (uint64_t)n;
    if (nItems > 0xffffffffull / 2 || nParts > 0xffffffffull / 2) return fail(CUACD_E_CAPACITY, "tree tables exceed 32-bit indexing");
    int rc;
    if ((rc = bParts.ensure(nParts * sizeof(PartDesc)))) return rc;
    if ((rc = bItems.ensure(nItems * sizeof(ItemDesc)))) return rc;
    if ((rc = bJobs.ensure(std::max<uint64_t>(totalJobs, 1) * sizeof(Job)))) return rc;
    if ((rc = bPlanes.ensure(std::max<uint64_t>(nPlanes, 1) * 16))) return rc;
    if ((rc = bUb.ensure((size_t)n * 4))) return rc;
    capSeeds = n; capJobs = (uint32_t)totalJobs; capItems = (uint32_t)nItems; capParts = (uint32_t)nParts;
    capPlanes = (uint32_t)nPlanes;
    gvalid = false;
    bind();
    return 0;
  }
  int ensurePartSlots(uint32_t n) {
    if (n <= capParts) return 0;
    int rc = bParts.ensure((size_t)n * sizeof(PartDesc));
    if (rc) return rc;
    capParts = n;
    gvalid = false;
    bind();
    return 0;
  }
  // hull slab of the run (tree.ts:300-312) and the number of slabs in flight
  int planSlabs(uint32_t maxNv, uint32_t nParts) {
    uint32_t fmax = 2 * std::min<uint32_t>((uint32_t)cfg.hullMaxVerts, maxNv) + 3 * VIS_MAX + 1024;
    slabWords = ((2 * maxNv + std::max(maxNv, 80u) + 7) & ~7u) + 16 * fmax;
    slabStride = hull_slab_stride(slabWords);
    uint64_t byBudget = std::max<uint64_t>(1, cfg.hullBudgetBytes / ((uint64_t)slabStride * 4));
    nSlabsSmall = (uint32_t)std::min<uint64_t>({byBudget, (uint64_t)nSM * bpsSmall * 8, (uint64_t)std::max(nParts, 1u)});
    nSlabsBig = (uint32_t)std::min<uint64_t>({byBudget, (uint64_t)nSM * bpsBig, (uint64_t)std::max(nParts, 1u)});
    size_t need = (size_t)std::max(nSlabsSmall, nSlabsBig) * slabStride * 4;
    if (bSlab.bytes < need) {
      gvalid = false;
      int rc = bSlab.ensure(need);
      if (rc) return rc;
      bind();
    }
    return 0;
  }
  Level baseLevel() const {
    Level P;
    std::memset(&P, 0, sizeof(P));
    P.edgeStride = edgeStride;
    P.minEdgeDist = cfg.minEdgeDist;
    P.hullSlabWords = slabWords;
    P.slabStride = slabStride;
    P.smallNv = smallNv();
    return P;
  }
  // hull launches of one level, warp groups then block groups; work
  // counters `slot` and 16 + slot must be zero beforehand. Parts above
  // warpMaxNv points take the widest blocks (1024, then 512 threads) whose
  // resident slots hold all the level's parts in one wave (the more threads
  // per part, the shorter each insertion round), else 256-thread blocks
  // (the most parts at once).
  void hullLaunch(Level P, uint32_t slot) {
    P.workSlot = slot;
    P.nSlabs = nSlabsSmall;
    launch_hull(P, D, 32, stream);
    int width = 256;
    uint32_t slabs = nSlabsBig;
    for (const auto& [w, bps] : {std::pair<int, int>{1024, bpsXL}, {512, bpsWide}}) {
      const uint32_t cap = (uint32_t)(nSM * bps);
      if (bps > 0 && P.nChildParts <= cap) {
        width = w;
        slabs = std::min(nSlabsBig, cap);
        break;
      }
    }
    P.nSlabs = slabs;
    launch_hull(P, D, width, stream);
  }
  // upload meshes at the start of the pools and write their part descriptors
  // (tree.ts:233-278); returns the host-side descriptors in parts
  // Host meshes are staged in pinned memory and uploaded in two copies;
  // device meshes (both buffers in device memory, e.g. the halves of the
  // last GPU cut batch) are copied on the device after the upload, into the
  // places the staging left for them.
  int uploadMeshes(const cuacd_mesh* m, uint32_t n, std::vector<PartDesc>& parts) {
    uint64_t totV = 0, totT = 0;
    std::vector<char> dev(n, 0);
    bool anyHost = false;
    for (uint32_t k = 0; k < n; k++) {
      if (m[k].nv && !m[k].verts) return fail(CUACD_E_INVALID, "mesh has vertices but no vertex pointer");
      if (m[k].nt && !m[k].tris) return fail(CUACD_E_INVALID, "mesh has triangles but no index pointer");
      const bool dv = is_device_ptr(m[k].verts), dt = is_device_ptr(m[k].tris);
      if ((m[k].nv && m[k].nt && dv != dt) || (!m[k].nv && dt) || (!m[k].nt && dv))
        return fail(CUACD_E_INVALID, "a mesh's buffers must both be host or both be device memory");
      dev[k] = dv || dt;
      anyHost |= !dev[k];
      totV += 3ull * m[k].nv;
      totT += 3ull * m[k].nt;
    }
    if (totV > cfg.vertexCap || totT > cfg.triCap) return fail(CUACD_E_CAPACITY, "seed meshes exceed pool capacity");
    float* hv = nullptr;
    uint32_t* ht = nullptr;
    if (anyHost) {
      int rc = hStage.ensure(std::max<size_t>((totV + totT) * 4, 64));
      if (rc) return rc;
      hv = (float*)hStage.p;
      ht = (uint32_t*)(hv + totV);
    }
    parts.assign(n, PartDesc{});
    uint32_t vt = 0, tt = 0;
    for (uint32_t k = 0; k < n; k++) {
      if (!dev[k]) {
        std::memcpy(hv + vt, m[k].verts, 12ull * m[k].nv);
        if (m[k].nt) std::memcpy(ht + tt, m[k].tris, 12ull * m[k].nt);
      }
      PartDesc& p = parts[k];
      std::memset(&p, 0, sizeof(p));
      p.vOff = vt; p.nv = m[k].nv; p.tOff = tt; p.nt = m[k].nt;
      p.planeIds[0] = p.planeIds[1] = p.planeIds[2] = p.planeIds[3] = CUACD_NONE;
      p.flags = m[k].nt == 0 ? 2u : 0u;
      vt += 3 * m[k].nv;
      tt += 3 * m[k].nt;
    }
    if (anyHost && totV) CK(cudaMemcpyAsync(D.V, hv, totV * 4, cudaMemcpyHostToDevice, stream));
    if (anyHost && totT) CK(cudaMemcpyAsync(D.T, ht, totT * 4, cudaMemcpyHostToDevice, stream));
    for (uint32_t k = 0; k < n; k++) {
      if (!dev[k]) continue;
      if (m[k].nv)
        CK(cudaMemcpyAsync(D.V + parts[k].vOff, m[k].verts, 12ull * m[k].nv, cudaMemcpyDeviceToDevice, stream));
      if (m[k].nt)
        CK(cudaMemcpyAsync(D.T + parts[k].tOff, m[k].tris, 12ull * m[k].nt, cudaMemcpyDeviceToDevice, stream));
    }
    vTop = vt;
    tTop = tt;
    return 0;
  }
  // host copies of the meshes of the next hull-with-Hausdorff or Hausdorff
  // call, whose sample counts follow each mesh's area (computed on the
  // host); needed when those meshes are in device memory
  std::vector<cuacd_mesh> twins;
  const cuacd_mesh& host_side(const cuacd_mesh* m, size_t k) const {
    return k < twins.size() ? twins[k] : m[k];
  }

  std::vector<LevelLayout> layout(uint32_t n, uint32_t dep, uint32_t w0, uint32_t ne0) const {
    std::vector<LevelLayout> lv;
    uint32_t itemsInBase = 0, nItemsIn = n, itemsOutBase = n, jobBase = 0;
    for (uint32_t l = 0; l < dep; l++) {
      uint32_t width = l == 0 ? w0 : (uint32_t)cfg.width2;
      uint32_t nEdge = l == 0 ? ne0 : 0;
      uint32_t tw = width + nEdge;
      uint32_t nJobs = nItemsIn * tw;
      lv.push_back(LevelLayout{itemsInBase, nItemsIn, itemsOutBase, jobBase, n + 2 * jobBase, nJobs, width, nEdge, tw});
      itemsInBase = itemsOutBase;
      nItemsIn = nJobs;
      itemsOutBase += nJobs;
      jobBase += nJobs;
    }
    return lv;
  }

  int prepare(const cuacd_mesh* seeds, int n, const float* edgePlanes, int planesPerSeed, const cuacd_run_opts* o) {
    CK(cudaStreamSynchronize(stream));
    prepared = false;
    cuacd_run_opts def;
    std::memset(&def, 0, sizeof(def));
    def.width = -1;
    def.nEdgeCuts = -1;
    if (!o) o = &def;
    if (n < 0) return fail(CUACD_E_INVALID, "negative seed count");
    uint32_t dep = o->depth > 0 ? (uint32_t)o->depth : (uint32_t)cfg.depth;
    uint32_t width0 = o->width >= 0 ? (uint32_t)o->width : (uint32_t)cfg.width;
    uint32_t nEdge0 = std::min<uint32_t>(o->nEdgeCuts >= 0 ? (uint32_t)o->nEdgeCuts : edgeStride, edgeStride);
    if (width0 % 3 != 0 || width0 > (uint32_t)cfg.width) return fail(CUACD_E_INVALID, "width override must be a multiple of 3 and <= configured width");
    if (dep < 1 || dep > (uint32_t)cfg.depth) return fail(CUACD_E_INVALID, "depth out of range for this tree");
    nSeeds = (uint32_t)n;
    depth = dep;
    if (n == 0) { prepared = true; return 0; }
    bool refine = o->refineRounds > 0 && o->refineProbes >= 3;
    nProbes = refine ? std::min<uint32_t>((uint32_t)o->refineProbes, edgeStride) : 0;
    rounds = refine ? (uint32_t)o->refineRounds : 0;
    int rc = ensureTables(nSeeds);
    if (rc) return rc;
    maxSeedNv = 0;
    for (int k = 0; k < n; k++) maxSeedNv = std::max(maxSeedNv, seeds[k].nv);
    choose(size_key(1u | (dep << 1) | ((refine ? 1u : 0u) << 4) | ((width0 / 3) << 5) | ((nEdge0 > 0 ? 1u : 0u) << 12),
                    seeds, n));
    tree = layout(nSeeds, depth, width0, nEdge0);
    probe = refine ? layout(nSeeds, depth, 0, nProbes) : std::vector<LevelLayout>();
    uint32_t maxChild = 0;
    for (auto& L : tree) maxChild = std::max(maxChild, 2 * L.nJobs);
    for (auto& L : probe) maxChild = std::max(maxChild, 2 * L.nJobs);
    if ((rc = planSlabs(maxSeedNv, maxChild))) return rc;
    // scan bases and per-block sums of the largest level
    uint32_t maxJobs = 0;
    for (auto& L : tree) maxJobs = std::max(maxJobs, L.nJobs);
    for (auto& L : probe) maxJobs = std::max(maxJobs, L.nJobs);
    size_t scanBytes = (3 + 3 * (size_t)((maxJobs + 1023) / 1024)) * 8;
    if (scanBytes > bScan.bytes) {
      if ((rc = bScan.ensure(scanBytes))) return rc;
      gvalid = false;
      bind();
    }
    std::vector<PartDesc> parts;
    if ((rc = uploadMeshes(seeds, nSeeds, parts))) return rc;
    edgePlaneBase = capJobs;
    stateBase = edgePlaneBase + capSeeds * edgeStride;
    // snapshot: seed parts | seed items | counters | edge planes | evaluate state
    snapParts = 0;
    snapItems = snapParts + (size_t)nSeeds * sizeof(PartDesc);
    snapCtr = snapItems + (size_t)nSeeds * sizeof(ItemDesc);
    snapEdge = snapCtr + CTR_WORDS * 4;
    snapState = snapEdge + (size_t)nSeeds * edgeStride * 16;
    snapBytes = snapState + (16 + 4 * (size_t)nSeeds) * 16;
    if ((rc = hSnap.ensure(snapBytes))) return rc;
    uint8_t* h = (uint8_t*)hSnap.p;
    std::memset(h, 0, snapBytes);
    std::memcpy(h + snapParts, parts.data(), (size_t)nSeeds * sizeof(PartDesc));
    ItemDesc* items = (ItemDesc*)(h + snapItems);
    for (uint32_t k = 0; k < nSeeds; k++) {
      items[k].partIds[0] = k;
      items[k].np = 1;
      items[k].srcPart = k;
      items[k].initialCut = CUACD_NONE;
      items[k].nLevels = 0;
      items[k].flags = 1;
      items[k].parentItem = CUACD_NONE;
    }
    uint32_t* ctr = (uint32_t*)(h + snapCtr);
    ctr[CTR_V] = vTop;
    ctr[CTR_T] = tTop;
    float* ep = (float*)(h + snapEdge);
    if (edgePlanes && planesPerSeed > 0) {
      uint32_t k0 = std::min<uint32_t>((uint32_t)planesPerSeed, edgeStride);
      for (uint32_t k = 0; k < nSeeds; k++)
        std::memcpy(ep + (size_t)4 * k * edgeStride, edgePlanes + (size_t)4 * k * planesPerSeed, 16ull * k0);
    }
    uint32_t* su = (uint32_t*)(h + snapState);
    float* sf = (float*)su;
    auto header = [&](uint32_t at, const std::vector<LevelLayout>& L) {
      su[at] = depth; su[at + 1] = nSeeds; su[at + 2] = L[0].totalWidth; su[at + 3] = nProbes;
      for (size_t l = 0; l < L.size(); l++) { su[at + 4 + 4 * l] = L[l].itemsOutBase; su[at + 5 + 4 * l] = L[l].nJobs; }
    };
    header(0, tree);
    if (refine) header(20, probe);
    for (uint32_t k = 0; k < nSeeds; k++) sf[(16 + 4 * k + 2) * 4] = (refine && o->refineSpacing) ? o->refineSpacing[k] : 0.0f;
    if ((rc = bSnap.ensure(snapBytes))) return rc;
    CK(cudaMemcpyAsync(bSnap.p, h, snapBytes, cudaMemcpyHostToDevice, stream));
    const std::vector<LevelLayout>& last = refine ? probe : tree;
    lastItems = last.back().itemsOutBase + last.back().nJobs;
    prepared = true;
    return 0;
  }

  // the whole run on the stream (tree.ts:559-594)
  void enqueue() {
    mark(-1);
    uint8_t* snap = (uint8_t*)bSnap.p;
    cudaMemcpyAsync(D.parts, snap + snapParts, (size_t)nSeeds * sizeof(PartDesc), cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(D.items, snap + snapItems, (size_t)nSeeds * sizeof(ItemDesc), cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(D.ctr, snap + snapCtr, CTR_WORDS * 4, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(D.planes + edgePlaneBase, snap + snapEdge, (size_t)nSeeds * edgeStride * 16, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(D.planes + stateBase, snap + snapState, (16 + 4 * (size_t)nSeeds) * 16, cudaMemcpyDeviceToDevice, stream);
    mark(0);
    auto stage = [&](const std::vector<LevelLayout>& L, uint32_t mode, uint32_t headerOff) {
      // one hull work counter per level of the stage
      // (work[l]: the level's hull counter; work[32 + l]: its largest child)
      cudaMemsetAsync(D.work, 0, 64 * 4, stream);
      for (uint32_t l = 0; l < L.size(); l++) {
        const LevelLayout& v = L[l];
        Level P = baseLevel();
        P.itemsInBase = v.itemsInBase; P.nItemsIn = v.nItemsIn; P.itemsOutBase = v.itemsOutBase; P.jobBase = v.jobBase;
        P.width = v.width; P.nEdgeCuts = v.nEdgeCuts; P.totalWidth = v.totalWidth;
        P.level = l; P.totalLevels = depth; P.partBase = v.partBase;
        P.edgePlaneBase = edgePlaneBase; P.nChildParts = 2 * v.nJobs; P.nJobs = v.nJobs;
        P.lastLevel = l == depth - 1 ? 1u : 0u;
        P.nSeeds = cfg.pruneLastLevel ? nSeeds : 0;
        P.workSlot = l;
        // parents shrink roughly by half per level
        bool big = (maxSeedNv >> l) > bigJobNv();
        launch_plan(P, D, big, stream);
        mark(1);
        launch_scan(P, D, stream);
        mark(2);
        launch_emit(P, D, big, stream);
        mark(3);
        // the last level's pruning bound, once per seed (the parent level's
        // items are final once its record ran)
        if (P.lastLevel && P.level > 0 && P.nSeeds > 0 && P.nItemsIn > 0) launch_seed_bound(P, D, stream);
        hullLaunch(P, l);
        mark(4);
        launch_record(P, D, stream);
        mark(5);
      }
      launch_evaluate(stateBase, headerOff, mode, nSeeds, L[0].jobBase, edgePlaneBase, edgeStride, D, stream);
      mark(6);
    };
    stage(tree, 0, 0);
    for (uint32_t r = 0; r < rounds; r++) {
      cudaMemcpyAsync(D.ctr, snap + snapCtr, 4 * 4, cudaMemcpyDeviceToDevice, stream);
      mark(0);
      stage(probe, 1, 5);
    }
  }
  std::vector<uint64_t> signature() const {
    std::vector<uint64_t> s = {nSeeds, depth, nProbes, rounds, slabWords, slabStride, nSlabsSmall, nSlabsBig,
                               maxSeedNv > bigJobNv() ? maxSeedNv : 0, edgePlaneBase, stateBase, (uint64_t)bSnap.p,
                               (uint64_t)bSlab.p, (uint64_t)bParts.p, (uint64_t)bItems.p, (uint64_t)bJobs.p,
                               (uint64_t)bPlanes.p, (uint64_t)bCtr.p, snapBytes, (uint64_t)bScan.p,
                               (uint64_t)bWork.p};
    for (auto& L : tree) { s.push_back(L.nJobs); s.push_back(L.totalWidth); s.push_back(L.width); }
    for (uint32_t l = 0; l < depth; l++) s.push_back((maxSeedNv >> l) > bigJobNv());
    s.push_back(smallNv());
    return s;
  }
  int launch() {
    if (!prepared) return fail(CUACD_E_INVALID, "launch before prepare");
    if (nSeeds == 0) return 0;
    std::vector<uint64_t> sig = signature();
    sig.push_back(profile ? 1 : 0);
    if (!gvalid || sig != gsig) {
      pcls.clear();
      if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      enqueue();
      CK(cudaStreamEndCapture(stream, &g));
      cudaError_t e = cudaGraphInstantiate(&gexec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return fail(CUACD_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
      gsig = sig;
      gvalid = true;
    }
    CK(cudaEventRecord(ev0, stream));
    CK(cudaGraphLaunch(gexec, stream));
    CK(cudaEventRecord(ev1, stream));
    return 0;
  }
  int collect(cuacd_seed_result* out, cuacd_run_stats* st) {
    if (!prepared) return fail(CUACD_E_INVALID, "collect before prepare");
    if (st) std::memset(st, 0, sizeof(*st));
    if (nSeeds == 0) return 0;
    size_t stateBytes = (16 + 4 * (size_t)nSeeds) * 16;
    int rc = hRead.ensure(stateBytes + 64 * 4);
    if (rc) return rc;
    uint8_t* h = (uint8_t*)hRead.p;
    CK(cudaMemcpyAsync(h, D.planes + stateBase, stateBytes, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h + stateBytes, D.ctr, 16 * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    CK(cudaGetLastError());
    const float* sf = (const float*)h;
    const uint32_t* sw = (const uint32_t*)h;
    const uint32_t* ctr = (const uint32_t*)(h + stateBytes);
    for (uint32_t k = 0; k < nSeeds && out; k++) {
      size_t o = (16 + 4 * (size_t)k) * 4;
      bool valid = (sw[o + 7] & 1) != 0;
      out[k].valid = valid ? 1 : 0;
      out[k].bestCut = valid ? (int32_t)sw[o + 6] : -1;
      out[k].bestCost = valid ? sf[o + 4] : INFINITY;
      for (int a = 0; a < 4; a++) out[k].plane[a] = valid ? sf[o + a] : 0.0f;
      out[k].reserved = 0;
    }
    if (st) {
      st->overflow = ctr[CTR_OVERFLOW] != 0;
      st->hullFail = ctr[CTR_HULLFAIL] != 0;
      st->hullFailCount = ctr[CTR_HULLFAIL];
      st->npOverflow = ctr[CTR_NPOVER] != 0;
      st->pruned = ctr[CTR_PRUNED];
      st->nLevels = (uint32_t)tree.size();
      for (size_t l = 0; l < tree.size() && l < 4; l++) st->jobsPerLevel[l] = tree[l].nJobs;
      st->validJobs = (uint64_t)ctr[CTR_VALID_LO] | ((uint64_t)ctr[CTR_VALID_HI] << 32);
      st->hullSlabWords = slabWords;
      st->hullChunkSize = nSlabsSmall;
    }
    {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess) cudaGetLastError();
      if (st) st->gpuMs = ms;
      record(ms);
    }
    for (int c = 0; c < 7; c++) kernelMs[c] = 0;
    std::memcpy(bytes, ctr + CTR_BYTES_PLAN, sizeof(bytes));
    if (profile) {
      for (size_t i = 1; i < pcls.size(); i++) {
        float d = 0;
        if (cudaEventElapsedTime(&d, pev[i - 1], pev[i]) != cudaSuccess) {
          cudaGetLastError();  // a timing failure must not poison later calls
          d = 0;
        }
        if (pcls[i] >= 0) kernelMs[pcls[i]] += d;
      }
    }
    return 0;
  }

  // ---- hull batches (tree.ts:382-443, 671-756) ----
  int hulls(const cuacd_mesh* m, int n, int hullStage, uint32_t* trisOut, uint32_t exportStrideOut, float* volOut,
            uint32_t* ntOut, int32_t* status, float* hdOut) {
    // the host twins serve this call only
    struct ClearTwins {
      std::vector<cuacd_mesh>& t;
      ~ClearTwins() { t.clear(); }
    } clearTwins{twins};
    if (n < 0) return fail(CUACD_E_INVALID, "negative mesh count");
    if (n == 0) return 0;
    if (hdOut)
      for (int k = 0; k < n; k++)
        if ((size_t)k >= twins.size() && is_device_ptr(m[k].verts))
          return fail(CUACD_E_INVALID, "hull with Hausdorff of a device mesh needs its host copy");
    CK(cudaStreamSynchronize(stream));
    bool withHd = hdOut != nullptr;
    if (withHd && n > CUACD_HD_MAX_PAIRS) return fail(CUACD_E_INVALID, "hullsWithHausdorff: at most 1024 meshes per call");
    int rc = ensureTables(1);
    if (rc) return rc;
    if ((rc = ensurePartSlots(withHd ? 2 * n : n))) return rc;
    uint32_t maxNv = 0;
    for (int k = 0; k < n; k++) maxNv = std::max(maxNv, m[k].nv);
    choose(size_key(2u | ((withHd ? 1u : 0u) << 2), m, n));
    if ((rc = planSlabs(maxNv, (uint32_t)n))) return rc;
    std::vector<PartDesc> parts;
    if ((rc = uploadMeshes(m, (uint32_t)n, parts))) return rc;
    const bool doExport = trisOut != nullptr || withHd;
    uint32_t stride = doExport ? 3 * 2 * std::min<uint32_t>((uint32_t)cfg.hullMaxVerts, maxNv) : 0;
    if ((uint64_t)tTop + (uint64_t)n * stride > cfg.triCap) return fail(CUACD_E_CAPACITY, "hull export exceeds triangle pool");
    // sample scratch of the fused Hausdorff (tree.ts:686-698)
    std::vector<uint32_t> capOff, capN;
    uint64_t totalCap = 0;
    uint32_t maxSide = 0;
    if (withHd) {
      capOff.resize(2 * n);
      capN.resize(2 * n);
      uint64_t off = 0;
      for (int k = 0; k < n; k++) {
        double area = mesh_area(host_side(m, (size_t)k));
        uint64_t res = std::max<uint64_t>(1000, (uint64_t)std::floor(2000.0 * area));
        uint64_t cap = 2 * (2 * res + std::max<uint64_t>(m[k].nt, 2ull * m[k].nv) + 16);
        if (3 * (off + cap) > cfg.scratchWords) return fail(CUACD_E_SCRATCH, "hausdorff sample scratch exceeds capacity");
        uint32_t ca = (uint32_t)(cap / 2), cb = (uint32_t)(cap - cap / 2);
        capOff[k] = (uint32_t)off; capN[k] = ca;
        capOff[n + k] = (uint32_t)(off + ca); capN[n + k] = cb;
        off += cap;
        maxSide = std::max(maxSide, std::max(ca, cb));
      }
      totalCap = off;
    }
    CK(cudaMemcpyAsync(D.parts, parts.data(), (size_t)n * sizeof(PartDesc), cudaMemcpyHostToDevice, stream));
    if (withHd) CK(cudaMemsetAsync(D.parts + n, 0, (size_t)n * sizeof(PartDesc), stream));
    CK(cudaMemsetAsync(D.ctr, 0, CTR_WORDS * 4, stream));
    Level P = baseLevel();
    P.nItemsIn = n; P.itemsOutBase = n; P.totalLevels = 1;
    P.edgePlaneBase = capJobs; P.nChildParts = n; P.nJobs = 0;
    P.exportBase = tTop; P.exportStride = stride; P.hullStage = (uint32_t)hullStage;
    P.hdDescBase = withHd ? (uint32_t)n : 0;
    P.maxNvHint = std::max(maxNv, 1u);
    CK(cudaMemsetAsync(D.work, 0, 64 * 4, stream));
    CK(cudaEventRecord(ev0, stream));
    hullLaunch(P, 0);
    if (withHd) {
      std::vector<uint32_t> triCap(2 * n);
      for (int k = 0; k < n; k++) {
        triCap[k] = m[k].nt;
        triCap[n + k] = stride / 3;
      }
      if ((rc = runHd((uint32_t)n, 0, capOff, capN, totalCap, maxSide, triCap))) return rc;
    }
    CK(cudaEventRecord(ev1, stream));
    CK(cudaGetLastError());
    // the faces come back either as the whole export range (small strides)
    // or, when that range is large and mostly unused (a chunk's stride
    // follows its largest mesh), as each hull's own faces after the face
    // counts are known
    const size_t pb = (size_t)n * sizeof(PartDesc), hb = withHd ? 4 * (size_t)n : 0;
    const bool wantTris = trisOut != nullptr && exportStrideOut > 0 && stride > 0;
    const bool compact = wantTris && (size_t)n * stride * 4 > (16u << 20);
    const size_t tb = wantTris && !compact ? (size_t)n * stride * 4 : 0;
    if ((rc = hRead.ensure(pb + hb + tb + 64))) return rc;
    uint8_t* h = (uint8_t*)hRead.p;
    CK(cudaMemcpyAsync(h, D.parts, pb, cudaMemcpyDeviceToHost, stream));
    if (withHd) CK(cudaMemcpyAsync(h + pb, D.ctr + CTR_HD, hb, cudaMemcpyDeviceToHost, stream));
    if (tb) CK(cudaMemcpyAsync(h + pb + hb, D.T + tTop, tb, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess) cudaGetLastError();
      record(ms);
    }
    std::vector<size_t> faceOff;  // compact readback: word offset of hull k's faces
    if (compact) {
      const PartDesc* pd0 = (const PartDesc*)h;
      faceOff.assign((size_t)n, 0);
      size_t words = 0;
      for (int k = 0; k < n; k++) {
        faceOff[k] = words;
        if (pd0[k].hullVol >= 0.0f && pd0[k].pad0 >= 4) words += std::min<size_t>(3 * (size_t)pd0[k].pad0, stride);
      }
      std::vector<PartDesc> keep(pd0, pd0 + n);  // hRead may move when it grows
      std::vector<uint32_t> hdKeep;
      if (withHd) hdKeep.assign((const uint32_t*)(h + pb), (const uint32_t*)(h + pb) + n);
      if ((rc = hRead.ensure(pb + hb + 4 * words + 64))) return rc;
      h = (uint8_t*)hRead.p;
      std::memcpy(h, keep.data(), pb);
      if (withHd) std::memcpy(h + pb, hdKeep.data(), hb);
      for (int k = 0; k < n; k++) {
        const size_t w = (k + 1 < n ? faceOff[k + 1] : words) - faceOff[k];
        if (w)
          CK(cudaMemcpyAsync(h + pb + hb + 4 * faceOff[k], D.T + tTop + (size_t)k * stride, 4 * w,
                             cudaMemcpyDeviceToHost, stream));
      }
      CK(cudaStreamSynchronize(stream));
    }
    const PartDesc* pd = (const PartDesc*)h;
    const uint32_t* tw = (const uint32_t*)(h + pb + hb);
    const uint32_t* hdw = (const uint32_t*)(h + pb);
    for (int k = 0; k < n; k++) {
      float vol = pd[k].hullVol;
      uint32_t nf = doExport ? pd[k].pad0 : 4;
      int32_t s = 0;
      if (vol < 0.0f) s = (pd[k].flags & 3) ? (int32_t)(pd[k].flags & 3) : 9;
      else if (nf < 4) s = 8;
      if (status) status[k] = s;
      if (volOut) volOut[k] = vol;
      if (ntOut) ntOut[k] = s == 0 && doExport ? nf : 0;
      if (wantTris && s == 0) {
        const uint32_t cpy = std::min({3 * nf, exportStrideOut, stride});
        const uint32_t* src = compact ? tw + faceOff[k] : tw + (size_t)k * stride;
        std::memcpy(trisOut + (size_t)k * exportStrideOut, src, 4ull * cpy);
      }
      if (withHd) {
        float w;
        std::memcpy(&w, &hdw[k], 4);
        hdOut[k] = std::sqrt(w);
      }
    }
    return 0;
  }
  static double mesh_area(const cuacd_mesh& m) {
    double area = 0;
    for (uint32_t t = 0; t < m.nt; t++) {
      const float* a = m.verts + 3 * m.tris[3 * t];
      const float* b = m.verts + 3 * m.tris[3 * t + 1];
      const float* c = m.verts + 3 * m.tris[3 * t + 2];
      double abx = (double)b[0] - a[0], aby = (double)b[1] - a[1], abz = (double)b[2] - a[2];
      double acx = (double)c[0] - a[0], acy = (double)c[1] - a[1], acz = (double)c[2] - a[2];
      double nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
      area += 0.5 * std::sqrt(nx * nx + ny * ny + nz * nz);
    }
    return area;
  }
  // triCap: per mesh, an upper bound on its triangles (the screen's data)
  int runHd(uint32_t nPairs, uint32_t partBase, const std::vector<uint32_t>& capOff, const std::vector<uint32_t>& capN,
            uint64_t totalCap, uint32_t maxSide, const std::vector<uint32_t>& triCap) {
    const size_t metaBytes = (size_t)(4 * 2 * nPairs) * 4;
    std::vector<uint32_t> hm(8 * nPairs, 0u);
    std::memcpy(hm.data(), capOff.data(), 4ull * 2 * nPairs);
    std::memcpy(hm.data() + 2 * nPairs, capN.data(), 4ull * 2 * nPairs);
    uint64_t nTri = 0;
    for (uint32_t m = 0; m < 2 * nPairs; m++) {
      hm[6 * nPairs + m] = (uint32_t)nTri;
      nTri += triCap[m];
    }
    if (nTri > 0xffffffffull) return fail(CUACD_E_CAPACITY, "hausdorff batch: too many triangles");
    const size_t sampOff = (metaBytes + 255) & ~(size_t)255;
    const size_t triBOff = (sampOff + (size_t)totalCap * 16 + 255) & ~(size_t)255;
    const size_t triGOff = triBOff + (size_t)nTri * 32;
    int rc = bHd.ensure(triGOff + (size_t)nTri * 48 + 16);
    if (rc) return rc;
    uint32_t* meta = (uint32_t*)bHd.p;
    if ((rc = hMeta.ensure(hm.size() * 4))) return rc;
    std::memcpy(hMeta.p, hm.data(), hm.size() * 4);
    CK(cudaMemcpyAsync(meta, hMeta.p, hm.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(D.ctr + CTR_HD_EXACT, 0, 8 * 4, stream));
    HdArgs A;
    A.nPairs = nPairs;
    A.nMeshes = 2 * nPairs;
    A.capOff = meta;
    A.capN = meta + 2 * nPairs;
    A.ns = meta + 4 * nPairs;
    A.triOff = meta + 6 * nPairs;
    A.samples = (float4*)((uint8_t*)bHd.p + sampOff);
    A.triB = (uint4*)((uint8_t*)bHd.p + triBOff);
    A.triG = (float4*)((uint8_t*)bHd.p + triGOff);
    A.partBase = partBase;
    A.maxSide = maxSide;
    A.screenMin = cfg.hdScreenMinTris == 0 ? 256u : (cfg.hdScreenMinTris < 0 ? 0xffffffffu : (uint32_t)cfg.hdScreenMinTris);
    launch_hd(A, D, stream);
    hdStatsPending = true;
    return 0;
  }
  // statistics of the last Hausdorff batch's screen: exact distances,
  // screened sample-triangle pairs, timeout flag
  bool hdStatsPending = false;
  uint64_t hdStats[3] = {0, 0, 0};
  int readHdStats() {
    if (!hdStatsPending) return 0;
    uint32_t w[6];
    CK(cudaStreamSynchronize(stream));
    CK(cudaMemcpy(w, D.ctr + CTR_HD_EXACT, sizeof w, cudaMemcpyDeviceToHost));
    hdStats[0] = (uint64_t)w[0] | ((uint64_t)w[1] << 32);
    hdStats[1] = (uint64_t)w[2] | ((uint64_t)w[3] << 32);
    hdStats[2] = w[4];
    hdStatsPending = false;
    return 0;
  }
  // GpuTree.hausdorff (tree.ts:318-372)
  int hausdorff(const cuacd_mesh* a, const cuacd_mesh* b, int n, float* out) {
    if (n < 0) return fail(CUACD_E_INVALID, "negative pair count");
    if (n == 0) return 0;
    for (int k = 0; k < n; k++)
      if (is_device_ptr(a[k].verts) || is_device_ptr(b[k].verts))
        return fail(CUACD_E_INVALID, "hausdorff: the sample counts follow host meshes' areas; pass host meshes");
    if (n > CUACD_HD_MAX_PAIRS) return fail(CUACD_E_INVALID, "hausdorff: at most 1024 pairs per call");
    CK(cudaStreamSynchronize(stream));
    int rc = ensureTables(1);
    if (rc) return rc;
    if ((rc = ensurePartSlots(2 * n))) return rc;
    std::vector<cuacd_mesh> all(2 * n);
    for (int k = 0; k < n; k++) { all[k] = a[k]; all[n + k] = b[k]; }
    std::vector<PartDesc> parts;
    if ((rc = uploadMeshes(all.data(), 2 * n, parts))) return rc;
    auto bound = [](const cuacd_mesh& m) {
      uint64_t res = std::max<uint64_t>(1000, (uint64_t)std::floor(2000.0 * mesh_area(m)));
      return 2 * res + m.nt + 16;
    };
    std::vector<uint32_t> capOff(2 * n), capN(2 * n);
    uint64_t off = 0;
    uint32_t maxSide = 0;
    for (int k = 0; k < n; k++) {
      uint64_t cap = 2 * std::max(bound(a[k]), bound(b[k]));
      if (3 * (off + cap) > cfg.scratchWords) return fail(CUACD_E_SCRATCH, "hausdorff sample scratch exceeds capacity");
      uint32_t ca = (uint32_t)(cap / 2), cb = (uint32_t)(cap - cap / 2);
      capOff[k] = (uint32_t)off; capN[k] = ca;
      capOff[n + k] = (uint32_t)(off + ca); capN[n + k] = cb;
      off += cap;
      maxSide = std::max(maxSide, std::max(ca, cb));
    }
    CK(cudaMemcpyAsync(D.parts, parts.data(), 2ull * n * sizeof(PartDesc), cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(D.ctr + CTR_HD, 0, 4ull * n, stream));
    CK(cudaEventRecord(ev0, stream));
    std::vector<uint32_t> triCap(2 * n);
    for (int k = 0; k < 2 * n; k++) triCap[k] = all[k].nt;
    if ((rc = runHd((uint32_t)n, 0, capOff, capN, off, maxSide, triCap))) return rc;
    CK(cudaEventRecord(ev1, stream));
    CK(cudaGetLastError());
    if ((rc = hRead.ensure(4ull * n))) return rc;
    CK(cudaMemcpyAsync(hRead.p, D.ctr + CTR_HD, 4ull * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    const uint32_t* w = (const uint32_t*)hRead.p;
    for (int k = 0; k < n; k++) {
      float f;
      std::memcpy(&f, &w[k], 4);
      out[k] = std::sqrt(f);
    }
    return 0;
  }
  int readBack(void* dst, const void* src, size_t bytes) {
    CK(cudaStreamSynchronize(stream));
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return 0;
  }
};

// the host copies of the meshes of the handle's next hull-with-Hausdorff
// call (internal: the decomposer passes device meshes with their host
// copies, tree_internal.h)
namespace cuacd {
int tree_set_host_twins(void* tree, const cuacd_mesh* twins, int n) {
  Tree* t = (Tree*)tree;
  if (!t || n < 0 || (n > 0 && !twins)) return fail(CUACD_E_INVALID, "host twins: invalid argument");
  t->twins.assign(twins, twins + n);
  return CUACD_OK;
}
}  // namespace cuacd

extern "C" {

const char* cuacd_last_error(void) { return g_err.c_str(); }

void cuacd_tree_config_default(cuacd_tree_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->width = 60;
  c->width2 = 3;
  c->depth = 2;
  c->nConcaveEdges = 32;
  c->minEdgeDist = 0.0125f;
  c->hullMaxVerts = 4096;
  c->vertexCap = 64ull << 20;
  c->triCap = 64ull << 20;
  c->edgeCap = 1ull << 20;
  c->scratchWords = 48ull << 20;
  c->hullBudgetBytes = 256ull << 20;
  c->pruneLastLevel = 1;
  c->autotune = 1;
}

void* cuacd_tree_create(const cuacd_tree_config* c, int* err) {
  auto bad = [&](int code, const char* msg) -> void* {
    g_err = msg;
    if (err) *err = code;
    return nullptr;
  };
  if (!c) return bad(CUACD_E_INVALID, "null config");
  if (c->width % 3 != 0 || c->width2 % 3 != 0 || c->width < 0 || c->width2 < 0)
    return bad(CUACD_E_INVALID, "width and width2 must be multiples of 3");
  if (c->depth < 1 || c->depth > 4) return bad(CUACD_E_INVALID, "depth must be in 1..4");
  if (c->vertexCap >= (1ull << 32) || c->triCap >= (1ull << 32) || c->edgeCap >= (1ull << 28) || c->scratchWords >= (1ull << 32))
    return bad(CUACD_E_INVALID, "pool capacities must fit 32-bit offsets");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return bad(CUACD_E_NODEVICE, "no CUDA device");
  Tree* t = new Tree();
  t->cfg = *c;
  t->edgeStride = (uint32_t)std::max(4 * c->nConcaveEdges, 32);
  cudaGetDevice(&t->device);
  cudaDeviceGetAttribute(&t->nSM, cudaDevAttrMultiProcessorCount, t->device);
  t->bpsSmall = std::max(1, hull_blocks_per_sm(32));
  t->bpsBig = std::max(1, hull_blocks_per_sm(256));
  t->bpsWide = hull_blocks_per_sm(512);
  t->bpsXL = hull_blocks_per_sm(1024);
  int rc = 0;
  if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&t->ev0) != cudaSuccess || cudaEventCreate(&t->ev1) != cudaSuccess) {
    delete t;
    return bad(CUACD_E_CUDA, "stream or event creation failed");
  }
  if ((rc = t->bV.ensure(std::max<uint64_t>(c->vertexCap, 4) * 4)) || (rc = t->bT.ensure(std::max<uint64_t>(c->triCap, 4) * 4)) ||
      (rc = t->bE.ensure(std::max<uint64_t>(c->edgeCap, 1) * 32)) || (rc = t->bS.ensure(std::max<uint64_t>(c->scratchWords, 4) * 4)) ||
      (rc = t->bCtr.ensure(CTR_WORDS * 4)) || (rc = t->bWork.ensure(256 * 4)) || (rc = t->bScan.ensure(64 * 8))) {
    std::string m = g_err;
    delete t;
    return bad(rc, m.c_str());
  }
  t->bind();
  if ((rc = t->ensureTables(16))) {
    std::string m = g_err;
    delete t;
    return bad(rc, m.c_str());
  }
  if (err) *err = 0;
  return t;
}

void cuacd_tree_destroy(void* t) { delete (Tree*)t; }

int cuacd_device_memory(uint64_t* total, uint64_t* freeBytes) {
  size_t f = 0, t = 0;
  const cudaError_t e = cudaMemGetInfo(&f, &t);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(e == cudaErrorNoDevice ? CUACD_E_NODEVICE : CUACD_E_CUDA,
                std::string("cuacd_device_memory: ") + cudaGetErrorString(e));
  }
  if (total) *total = t;
  if (freeBytes) *freeBytes = f;
  return CUACD_OK;
}

int cuacd_tree_memory(const void* tree, uint64_t* deviceBytes, uint64_t* caps4) {
  const Tree* t = (const Tree*)tree;
  if (!t) return fail(CUACD_E_INVALID, "cuacd_tree_memory: null tree");
  uint64_t n = cut::engine_device_bytes(t->cutter) + conc::engine_device_bytes(t->concave);
  for (const DevBuf* b : {&t->bV, &t->bT, &t->bE, &t->bS, &t->bCtr, &t->bSlab, &t->bParts, &t->bItems, &t->bJobs,
                          &t->bPlanes, &t->bSnap, &t->bHd, &t->bScan, &t->bWork, &t->bUb})
    n += b->bytes;
  if (deviceBytes) *deviceBytes = n;
  if (caps4) {
    caps4[0] = t->cfg.vertexCap;
    caps4[1] = t->cfg.triCap;
    caps4[2] = t->cfg.edgeCap;
    caps4[3] = t->cfg.scratchWords;
  }
  return CUACD_OK;
}

int cuacd_tree_schedule(const void* tree, int32_t* out4) {
  const Tree* t = (const Tree*)tree;
  if (!t || !out4) return fail(CUACD_E_INVALID, "cuacd_tree_schedule: invalid argument");
  out4[0] = (int32_t)t->smallNv();
  out4[1] = (int32_t)t->bigJobNv();
  out4[2] = t->lastTrial ? 1 : 0;
  int32_t done = 0;
  for (const auto& kv : t->tuneTable) done += kv.second.tried == kNumSchedules ? 1 : 0;
  out4[3] = done;
  return CUACD_OK;
}

int cuacd_tree_reserve_pools(void* tree, const uint64_t* caps4) {
  Tree* t = (Tree*)tree;
  if (!t || !caps4) return fail(CUACD_E_INVALID, "cuacd_tree_reserve_pools: invalid argument");
  uint64_t* cur[4] = {&t->cfg.vertexCap, &t->cfg.triCap, &t->cfg.edgeCap, &t->cfg.scratchWords};
  DevBuf* buf[4] = {&t->bV, &t->bT, &t->bE, &t->bS};
  const uint64_t unit[4] = {4, 4, 32, 4};
  bool grow = false;
  for (int k = 0; k < 4; k++) {
    if (caps4[k] > 0xffffffffull) return fail(CUACD_E_CAPACITY, "cuacd_tree_reserve_pools: pools exceed 32-bit offsets");
    grow |= caps4[k] > *cur[k];
  }
  if (!grow) return CUACD_OK;
  cudaStreamSynchronize(t->stream);
  // a pool that cannot grow is allocated again at its old size, so the
  // handle stays usable after a refusal
  int rc = 0;
  for (int k = 0; k < 4 && rc == 0; k++) {
    if (caps4[k] <= *cur[k]) continue;
    if (buf[k]->ensure(caps4[k] * unit[k])) {
      const std::string m = g_err;
      buf[k]->ensure(std::max<uint64_t>(*cur[k], 4) * unit[k]);
      rc = fail(CUACD_E_CUDA, "cuacd_tree_reserve_pools: " + m);
      break;
    }
    *cur[k] = caps4[k];
  }
  t->prepared = false;
  t->gvalid = false;
  t->bind();
  return rc;
}

int cuacd_tree_plane_cuts(void* tree, const cuacd_mesh* meshes, int nMeshes, const int32_t* meshOfCut,
                          const double* planes, int nCuts, int flags, void** halves) {
  Tree* t = (Tree*)tree;
  if (!t || !halves || nCuts < 0 || (nCuts > 0 && (!meshOfCut || !planes || !meshes)))
    return fail(CUACD_E_INVALID, "cuacd_tree_plane_cuts: invalid argument");
  *halves = nullptr;
  if (!t->cutter && !(t->cutter = cut::engine_create())) return fail(CUACD_E_CUDA, "cut engine creation failed");
  std::vector<cut::CutSpec> cs((size_t)nCuts);
  for (int k = 0; k < nCuts; k++) {
    const double* p = planes + 4 * (size_t)k;
    const host::PlaneFrame f = host::plane_frame(host::Plane{p[0], p[1], p[2], p[3]});
    cs[k].mesh = meshOfCut[k];
    for (int a = 0; a < 3; a++) {
      cs[k].n[a] = f.n[a];
      cs[k].u[a] = f.u[a];
      cs[k].v[a] = f.v[a];
    }
    cs[k].d = f.d;
  }
  cut::Halves* h = new cut::Halves();
  const int rc = cut::engine_run(t->cutter, t->stream, meshes, nMeshes, cs.data(), nCuts,
                                 (flags & CUACD_CUT_CLOSED) != 0, h);
  if (rc != CUACD_OK) {
    delete h;
    return rc;
  }
  *halves = h;
  return CUACD_OK;
}

int cuacd_cuts_half(const void* halves, int cut, int side, const float** verts, uint32_t* nv, const uint32_t** tris,
                    uint32_t* nt) {
  const cut::Halves* h = (const cut::Halves*)halves;
  if (!h || cut < 0 || (size_t)cut >= h->status.size() || side < 0 || side > 1)
    return fail(CUACD_E_INVALID, "cuacd_cuts_half: invalid argument");
  const size_t k = 2 * (size_t)cut + side;
  const int st = h->status[cut];
  if (verts) *verts = st == 0 ? h->V + 3 * h->vOff[k] : nullptr;
  if (tris) *tris = st == 0 ? h->T + 3 * h->tOff[k] : nullptr;
  if (nv) *nv = st == 0 ? h->nv[k] : 0;
  if (nt) *nt = st == 0 ? h->nt[k] : 0;
  return st;
}

int cuacd_cuts_half_device(const void* halves, int cut, int side, const float** verts, const uint32_t** tris) {
  const cut::Halves* h = (const cut::Halves*)halves;
  if (!h || cut < 0 || (size_t)cut >= h->status.size() || side < 0 || side > 1)
    return fail(CUACD_E_INVALID, "cuacd_cuts_half_device: invalid argument");
  const size_t k = 2 * (size_t)cut + side;
  const int st = h->status[cut];
  if (verts) *verts = st == 0 && h->dV ? h->dV + 3 * h->vOff[k] : nullptr;
  if (tris) *tris = st == 0 && h->dT ? h->dT + 3 * h->tOff[k] : nullptr;
  return st;
}

int cuacd_tree_eval_cuts(void* tree, const cuacd_mesh* mesh, const double* planes, int n, double* out8) {
  Tree* t = (Tree*)tree;
  if (!t || !mesh || n < 0 || (n > 0 && (!planes || !out8))) return fail(CUACD_E_INVALID, "cuacd_tree_eval_cuts: invalid argument");
  if (n == 0) return CUACD_OK;
  std::memset(out8, 0, 8 * sizeof(double) * (size_t)n);
  std::vector<int32_t> which((size_t)n, 0);
  void* hv = nullptr;
  int rc = cuacd_tree_plane_cuts(tree, mesh, 1, which.data(), planes, n, 0, &hv);
  if (rc != CUACD_OK) return rc;
  cut::Halves* h = (cut::Halves*)hv;
  float ms = h->gpuMs;
  // every half of every cut that split, hulled with its Hausdorff distance
  std::vector<cuacd_mesh> halves;
  std::vector<int> owner;
  for (int k = 0; k < n; k++) {
    if (h->status[k] != 0) continue;
    for (int sd = 0; sd < 2; sd++) {
      const size_t i = 2 * (size_t)k + sd;
      halves.push_back(cuacd_mesh{h->V + 3 * h->vOff[i], h->T + 3 * h->tOff[i], h->nv[i], h->nt[i]});
      owner.push_back(2 * k + sd);
    }
  }
  const size_t nh = halves.size();
  std::vector<float> vol(nh), hd(nh);
  std::vector<uint32_t> nt(nh);
  std::vector<int32_t> st(nh);
  size_t batch = std::min<size_t>(nh, CUACD_HD_MAX_PAIRS);
  for (size_t s0 = 0; s0 < nh;) {
    const size_t m = std::min(batch, nh - s0);
    rc = t->hulls(halves.data() + s0, (int)m, 0, nullptr, 0, vol.data() + s0, nt.data() + s0, st.data() + s0,
                  hd.data() + s0);
    if (rc == CUACD_E_SCRATCH && m > 1) {  // halve the batch, as merge.ts:405 does
      batch = std::max<size_t>(1, m / 2);
      continue;
    }
    if (rc != CUACD_OK) {
      cuacd_cuts_free(hv);
      return rc;
    }
    ms += cuacd_tree_last_gpu_ms(tree);
    s0 += m;
  }
  for (size_t i = 0; i < nh; i++) {
    const int k = owner[i] / 2, sd = owner[i] % 2;
    double* o = out8 + 8 * (size_t)k;
    const double mv = std::fabs(h->vol[(size_t)owner[i]]);
    const double hvol = st[i] == 0 ? (double)vol[i] : 0.0;
    o[0] = 1;
    o[1 + sd] = mv;
    o[3 + sd] = hvol;
    o[5 + sd] = 0.3 * std::cbrt((3.0 / (4.0 * M_PI)) * std::max(hvol - mv, 0.0));
    if (st[i] == 0) o[7] = std::max(o[7], (double)hd[i]);
  }
  t->lastEvalMs = ms;
  cuacd_cuts_free(hv);
  return CUACD_OK;
}

float cuacd_tree_eval_cuts_ms(void* tree) { return tree ? ((Tree*)tree)->lastEvalMs : 0.0f; }

int cuacd_tree_concave_planes(void* tree, const cuacd_mesh* meshes, int n, int nConcaveEdges, double concaveEps,
                              double concaveThreshold, const uint32_t* seeds, float* out, int32_t* counts) {
  Tree* t = (Tree*)tree;
  if (!t || n < 0) return fail(CUACD_E_INVALID, "cuacd_tree_concave_planes: invalid argument");
  if (!t->concave && !(t->concave = conc::engine_create())) return fail(CUACD_E_CUDA, "concave engine creation failed");
  return conc::engine_run(t->concave, t->stream, meshes, n, nConcaveEdges, concaveEps, concaveThreshold, seeds, out,
                          counts, &t->lastConcaveMs);
}

float cuacd_tree_concave_ms(void* tree) { return tree ? ((Tree*)tree)->lastConcaveMs : 0.0f; }

float cuacd_cuts_gpu_ms(const void* halves) { return halves ? ((const cut::Halves*)halves)->gpuMs : 0.0f; }

void cuacd_cuts_free(void* halves) { delete (cut::Halves*)halves; }
int cuacd_plane_slots(const void* t) { return (int)((const Tree*)t)->edgeStride; }
int cuacd_vis_max(void) { return CUACD_VIS_MAX; }
void cuacd_set_profile(void* t, int on) {
  Tree* tr = (Tree*)t;
  tr->profile = on != 0;
  // events are created before any capture: a profiled run records up to
  // 2 + (1 + rounds) * (5 * depth + 2) of them as graph nodes
  while (tr->profile && tr->pev.size() < 256) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) break;
    tr->pev.push_back(e);
  }
}
float cuacd_tree_last_gpu_ms(void* t) {
  // device time between the last call's two events (a run, a hull batch or
  // a Hausdorff batch); 0 when the call has not completed
  Tree* tr = (Tree*)t;
  float ms = 0;
  if (!tr || cudaEventElapsedTime(&ms, tr->ev0, tr->ev1) != cudaSuccess) {
    cudaGetLastError();
    return 0.0f;
  }
  return ms;
}
int cuacd_tree_hd_stats(void* t, uint64_t* out3) {
  if (!t || !out3) return fail(CUACD_E_INVALID, "cuacd_tree_hd_stats: invalid argument");
  Tree* tr = (Tree*)t;
  int rc = tr->readHdStats();
  if (rc) return rc;
  std::memcpy(out3, tr->hdStats, sizeof(uint64_t) * 3);
  return 0;
}
int cuacd_tree_kernel_bytes(void* t, uint64_t* bytes3) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  std::memcpy(bytes3, ((Tree*)t)->bytes, sizeof(uint64_t) * 3);
  return 0;
}
int cuacd_tree_kernel_ms(void* t, float* ms7) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  std::memcpy(ms7, ((Tree*)t)->kernelMs, sizeof(float) * 7);
  return 0;
}

int cuacd_tree_prepare(void* t, const cuacd_mesh* seeds, int n, const float* edgePlanes, int planesPerSeed,
                       const cuacd_run_opts* opts) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  return ((Tree*)t)->prepare(seeds, n, edgePlanes, planesPerSeed, opts);
}
int cuacd_tree_launch(void* t) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  return ((Tree*)t)->launch();
}
int cuacd_tree_collect(void* t, cuacd_seed_result* out, cuacd_run_stats* st) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  return ((Tree*)t)->collect(out, st);
}
int cuacd_tree_run(void* t, const cuacd_mesh* seeds, int n, const float* edgePlanes, int planesPerSeed,
                   const cuacd_run_opts* opts, cuacd_seed_result* out, cuacd_run_stats* st) {
  int rc = cuacd_tree_prepare(t, seeds, n, edgePlanes, planesPerSeed, opts);
  if (rc) return rc;
  if ((rc = cuacd_tree_launch(t))) return rc;
  return cuacd_tree_collect(t, out, st);
}
int cuacd_tree_hausdorff(void* t, const cuacd_mesh* a, const cuacd_mesh* b, int n, float* out) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  return ((Tree*)t)->hausdorff(a, b, n, out);
}
int cuacd_tree_hull_meshes(void* t, const cuacd_mesh* m, int n, int hullStage, uint32_t* trisOut, uint32_t exportStride,
                           float* volOut, uint32_t* ntOut, int32_t* status) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  return ((Tree*)t)->hulls(m, n, hullStage, trisOut, exportStride, volOut, ntOut, status, nullptr);
}
int cuacd_tree_hulls_with_hausdorff(void* t, const cuacd_mesh* m, int n, uint32_t* trisOut, uint32_t exportStride,
                                    float* volOut, uint32_t* ntOut, float* hdOut, int32_t* status) {
  if (!t) return fail(CUACD_E_INVALID, "null tree");
  if (!hdOut) {
    ((Tree*)t)->twins.clear();  // the host twins serve one call, even a refused one
    return fail(CUACD_E_INVALID, "null Hausdorff output");
  }
  return ((Tree*)t)->hulls(m, n, 0, trisOut, exportStride, volOut, ntOut, status, hdOut);
}
int cuacd_tree_read_items(void* tp, uint32_t first, uint32_t n, uint32_t* out) {
  Tree* t = (Tree*)tp;
  if ((uint64_t)first + n > t->capItems) return fail(CUACD_E_INVALID, "item range out of bounds");
  return t->readBack(out, t->D.items + first, (size_t)n * sizeof(ItemDesc));
}
int cuacd_tree_read_parts(void* tp, uint32_t first, uint32_t n, uint32_t* out) {
  Tree* t = (Tree*)tp;
  if ((uint64_t)first + n > t->capParts) return fail(CUACD_E_INVALID, "part range out of bounds");
  return t->readBack(out, t->D.parts + first, (size_t)n * sizeof(PartDesc));
}
int cuacd_tree_read_jobs(void* tp, uint32_t first, uint32_t n, uint32_t* out) {
  Tree* t = (Tree*)tp;
  if ((uint64_t)first + n > std::max<uint32_t>(t->capJobs, 1)) return fail(CUACD_E_INVALID, "job range out of bounds");
  return t->readBack(out, t->D.jobs + first, (size_t)n * sizeof(Job));
}
int cuacd_tree_read_part_geometry(void* tp, uint32_t part, float* verts, uint32_t* tris, uint32_t* edges) {
  Tree* t = (Tree*)tp;
  if (part >= t->capParts) return fail(CUACD_E_INVALID, "part out of bounds");
  PartDesc pd;
  int rc = t->readBack(&pd, t->D.parts + part, sizeof(pd));
  if (rc) return rc;
  if ((uint64_t)pd.vOff + 3ull * pd.nv > t->cfg.vertexCap || (uint64_t)pd.tOff + 3ull * pd.nt > t->cfg.triCap ||
      (uint64_t)pd.eOff + pd.ne > t->cfg.edgeCap)
    return fail(CUACD_E_INVALID, "part geometry out of pool bounds");
  if (verts && pd.nv && (rc = t->readBack(verts, t->D.V + pd.vOff, 12ull * pd.nv))) return rc;
  if (tris && pd.nt && (rc = t->readBack(tris, t->D.T + pd.tOff, 12ull * pd.nt))) return rc;
  if (edges && pd.ne && (rc = t->readBack(edges, t->D.E + 8ull * pd.eOff, 32ull * pd.ne))) return rc;
  return 0;
}
int cuacd_tree_read_plane(void* tp, uint32_t idx, float* out4) {
  Tree* t = (Tree*)tp;
  if (idx >= t->capPlanes) return fail(CUACD_E_INVALID, "plane out of bounds");
  return t->readBack(out4, t->D.planes + idx, 16);
}

}  // extern "C"
