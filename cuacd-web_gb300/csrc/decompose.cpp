// decompose.cpp — the decomposition loop (src/decompose.ts) and the hull
// merging pass (src/merge.ts) on the host, driving the GPU tree, hull and
// Hausdorff entry points of this library.
//
// One Engine owns one GPU tree. A call decomposes n meshes: one after
// another, or all together, when every iteration gathers the cutting parts
// of all meshes into one concave-plane batch and one tree run, the winning
// cuts of all meshes into one GPU cut batch, the new halves into one hull +
// Hausdorff submission, and every merge round's pairs into shared hull and
// Hausdorff batches. The GPU work per seed and per part does not depend on
// its batch, so both ways give the same parts. Host geometry (seam planes,
// filtered unions, the output hulls' cleanup) runs on a thread pool.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cuacd.h"
#include "host_mesh.h"
#include "tree_internal.h"

namespace cuacd {
int set_error(int code, const char* msg);
}

namespace cuacd {
namespace dec {

using host::Mesh;
using host::Plane;

constexpr double K_RV = 0.3;  // part.ts:7

// rvCost (part.ts:24-26)
inline double rv_cost(double meshVol, double hullVol) {
  return K_RV * std::cbrt((3.0 / (4.0 * M_PI)) * std::max(hullVol - meshVol, 0.0));
}

struct Part {
  Mesh mesh, hull;
  // the output hull while its cleanup still runs on the engine's workers
  // (hull is set from it before anything reads the hull)
  std::shared_future<Mesh> hullTask;
  double meshVol = 0, hullVol = 0;
  double hd = 0;
  bool hasHd = false;
  bool stuck = false;
  int stuckReason = 0;
  std::vector<Plane> seams;
  int merged = 1;
  uint64_t id = 0;  // identity for the merge pass's pair cache
  // the part's geometry on the device: made by GPU cut batch `gen` of its
  // engine, in that engine's cut output until the next batch
  const float* dV = nullptr;
  const uint32_t* dT = nullptr;
  uint64_t gen = 0;
};

// partCost (part.ts:27-29)
inline double part_cost(const Part& p) { return std::max(rv_cost(p.meshVol, p.hullVol), p.hasHd ? p.hd : 0.0); }

struct Failure {
  int code;
  std::string msg;
};

using Clock = std::chrono::steady_clock;
inline double ms_since(Clock::time_point t) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t).count();
}

// ---------------------------------------------------------------------------
// thread pool for host geometry

template <class F>
void parallel_for(size_t n, int threads, F&& fn) {
  if (n == 0) return;
  const size_t nt = std::min<size_t>(n, (size_t)std::max(threads, 1));
  if (nt <= 1) {
    for (size_t i = 0; i < n; i++) fn(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (size_t t = 0; t < nt; t++)
    pool.emplace_back([&]() {
      for (size_t i; (i = next.fetch_add(1)) < n;) fn(i);
    });
  for (auto& th : pool) th.join();
}

// workers for host tasks that the decomposition loop does not wait for (the
// output hulls' cleanup, needed only by the merge pass and the output)
class TaskPool {
 public:
  explicit TaskPool(int n) : n_(std::max(n, 1)) {}
  ~TaskPool() {
    {
      std::lock_guard<std::mutex> l(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (std::thread& t : th_) t.join();
  }
  std::shared_future<Mesh> submit(std::function<Mesh()> fn) {
    auto task = std::make_shared<std::packaged_task<Mesh()>>(std::move(fn));
    std::shared_future<Mesh> f = task->get_future().share();
    {
      std::lock_guard<std::mutex> l(m_);
      q_.push_back([task]() { (*task)(); });
      if (th_.size() < (size_t)n_ && idle_ == 0) th_.emplace_back([this]() { work(); });
    }
    cv_.notify_one();
    return f;
  }

 private:
  void work() {
    for (;;) {
      std::function<void()> job;
      {
        std::unique_lock<std::mutex> l(m_);
        idle_++;
        cv_.wait(l, [&] { return stop_ || !q_.empty(); });
        idle_--;
        // the queue drains before the workers stop
        if (q_.empty()) return;
        job = std::move(q_.front());
        q_.pop_front();
      }
      job();
    }
  }
  int n_;
  int idle_ = 0;
  bool stop_ = false;
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> q_;
  std::vector<std::thread> th_;
};

// ---------------------------------------------------------------------------
// one decomposition in flight

struct Job {
  Mesh input;
  Mesh mesh;  // normalised
  host::Normalization norm{1.0, {0, 0, 0}};
  bool normalized = false;
  std::vector<Part> parts;
  bool cutting_done = false;
  int iter = 0;  // iterations started
  // output-hull cleanup epsilon (decompose.ts:231-236): above a few float32
  // ulps of the input's largest coordinate relative to its extent
  double hullEps = 2e-5;
  bool merging = false;
  int mergeHullFails = 0;  // merged hulls the GPU could not build (the pair stays apart)
  cuacd_decompose_stats st{};
  // merge state
  std::map<std::pair<uint64_t, uint64_t>, size_t> cache;  // pair -> eval index
};

struct PairEval {
  double cost = 0;
  bool hasHull = false;
  Mesh hull;
  double hullVol = 0;
  double hd = 0;
  bool hasSeam = false;
  Plane seam{0, 0, 0, 0};
};

struct Result {
  std::vector<std::vector<Part>> parts;
  std::vector<cuacd_decompose_stats> stats;
};

class Engine {
 public:
  cuacd_decompose_opts o;
  void* tree = nullptr;
  int planeSlots = 0;
  int threads = 1;
  uint64_t nextId = 1;
  std::vector<PairEval> evals;  // merge pair evaluations of the current call
  // whole-call timings
  double treeMs = 0, cutMs = 0, concaveMs = 0, hullMs = 0, hdMs = 0, mergeMs = 0, gpuMs = 0;
  double cutGpuMs = 0;  // of cutMs: the GPU cut batch and its readback

  ~Engine() {
    if (tree) cuacd_tree_destroy(tree);
    if (bigTree) cuacd_tree_destroy(bigTree);
  }

  // output-hull cleanups run here while the loop goes on
  std::unique_ptr<TaskPool> pool;
  TaskPool& clean_pool() { return *pool; }
  // the part's output hull, once its cleanup is done
  static void resolve(Part& p) {
    if (!p.hullTask.valid()) return;
    p.hull = p.hullTask.get();
    p.hullTask = std::shared_future<Mesh>();
  }

  // GPU cut batches run so far: a part made by the latest one is still in
  // the cut engine's output buffers, and the next concave-plane batch, tree
  // run and cut batch read it there instead of uploading it again
  uint64_t cutGen = 0;
  cuacd_mesh resident(const Part& p) const {
    if (p.gen != 0 && p.gen == cutGen && p.dV && p.dT)
      return cuacd_mesh{p.dV, p.dT, (uint32_t)p.mesh.nv(), (uint32_t)p.mesh.nt()};
    return cuacd_mesh{p.mesh.v.data(), p.mesh.t.data(), (uint32_t)p.mesh.nv(), (uint32_t)p.mesh.nt()};
  }

  [[noreturn]] void cuda_fail(int rc, const char* what) {
    throw Failure{rc, std::string(what) + ": " + cuacd_last_error()};
  }

  // ---- GPU services ------------------------------------------------------

  // hulls (and, when withHd, Hausdorff distances to them) of meshes, in
  // chunks of at most 1024 (the reference hulls new parts in chunks of 256,
  // decompose.ts:178, and merge pairs in chunks of 1024, merge.ts:209; a hull
  // does not depend on its chunk, and larger chunks fill the GPU: 1,535
  // merge-pair hulls took 67 ms of device time in chunks of 256 and 53 ms in
  // chunks of 1024), halved when a chunk's hull export does not fit the
  // triangle pool. A failed hull is an error unless
  // allowFail, when the part gets a NaN hull volume.
  // defer: the output hulls' cleanup goes to the workers (the part's
  // hullTask) instead of finishing before the call returns
  // keep: when given, a hull whose (mesh index, GPU hull volume) it rejects
  // gets its volume only, without the host cleanup of its faces (the merge
  // pass needs the cleaned hull only for pairs under the threshold: merge.ts
  // cleans every pair's hull, merge.ts:213, but keeps it only for those,
  // merge.ts:221)
  // dev: the same meshes in device memory (the GPU then copies them on the
  // device; ms stays the host copy for the sample counts and the cleanup)
  void hulls(const std::vector<const Mesh*>& ms, const std::vector<double>& eps, bool withHd, std::vector<Part>& out,
             bool allowFail = false, bool defer = false,
             const std::function<bool(size_t, double)>* keep = nullptr,
             const std::vector<cuacd_mesh>* dev = nullptr) {
    out.resize(ms.size());
    if (defer && !pool) pool = std::make_unique<TaskPool>(threads);
    // chunks hold meshes of similar size (ascending point count): a chunk's
    // export stride and readback follow its largest mesh, so one large
    // merged hull no longer sizes a thousand small ones (a hull and its
    // Hausdorff samples do not depend on their chunk)
    std::vector<size_t> order(ms.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return ms[a]->nv() < ms[b]->nv(); });
    size_t chunk = CUACD_HD_MAX_PAIRS;
    for (size_t s = 0; s < ms.size();) {
      const size_t n = std::min(chunk, ms.size() - s);
      std::vector<cuacd_mesh> cm(n), twins;
      uint32_t maxNv = 0;
      for (size_t k = 0; k < n; k++) {
        const Mesh& m = *ms[order[s + k]];
        cm[k] = cuacd_mesh{m.v.data(), m.t.data(), (uint32_t)m.nv(), (uint32_t)m.nt()};
        maxNv = std::max(maxNv, (uint32_t)m.nv());
      }
      if (dev) {
        twins = cm;
        for (size_t k = 0; k < n; k++) cm[k] = (*dev)[order[s + k]];
        const int trc = tree_set_host_twins(tree, twins.data(), (int)n);
        if (trc != CUACD_OK) cuda_fail(trc, "hull batch");
      }
      const uint32_t stride = 3 * 2 * std::min<uint32_t>((uint32_t)o.tree.hullMaxVerts, maxNv);
      // not zeroed: only each hull's own faces are written and read
      std::unique_ptr<uint32_t[]> tris(new uint32_t[(size_t)n * stride + 1]);
      std::vector<float> vol(n), hd(n);
      std::vector<uint32_t> ntri(n);
      std::vector<int32_t> status(n);
      const auto t0 = Clock::now();
      const int rc = withHd ? cuacd_tree_hulls_with_hausdorff(tree, cm.data(), (int)n, tris.get(), stride, vol.data(),
                                                              ntri.data(), hd.data(), status.data())
                            : cuacd_tree_hull_meshes(tree, cm.data(), (int)n, 0, tris.get(), stride, vol.data(),
                                                     ntri.data(), status.data());
      gpuMs += ms_since(t0);
      if (rc == CUACD_E_CAPACITY && n > 1) {
        chunk = std::max<size_t>(1, n / 2);
        continue;
      }
      if (rc != CUACD_OK) cuda_fail(rc, "hull batch");
      parallel_for(n, threads, [&](size_t k) {
        const size_t i = order[s + k];
        Part& p = out[i];
        const Mesh& m = *ms[i];
        p.mesh = m;
        p.meshVol = host::volume(m);
        if (status[k] == 8) {
          // fewer than 4 hull faces: the points are flat (or fewer than 4),
          // the hull is the set itself with no volume, and a flat part is its
          // own hull (distance 0)
          p.hull = m;
          p.hullVol = 0.0;
          p.hd = 0.0;
          p.hasHd = true;
          return;
        }
        if (status[k] != 0) {
          p.hullVol = NAN;
          return;
        }
        if (keep && !(*keep)(i, (double)vol[k])) {
          p.hullVol = vol[k];
          return;
        }
        // output faces cleaned (decompose.ts:189, merge.ts:213); the kernel's
        // volume stays the part's hull volume
        const uint32_t* raw = tris.get() + (size_t)k * stride;
        if (defer) {
          std::vector<uint32_t> rt(raw, raw + 3 * (size_t)ntri[k]);
          std::vector<float> pv(m.v);
          const double e = eps[i];
          p.hullTask = clean_pool().submit([pv = std::move(pv), rt = std::move(rt), e]() {
            const std::vector<uint32_t> ct = host::clean_hull_faces(pv.data(), pv.size() / 3, rt.data(), rt.size(), e);
            return host::compact_hull(pv.data(), ct.data(), ct.size() / 3, nullptr);
          });
        } else {
          const std::vector<uint32_t> ct = host::clean_hull_faces(m.v.data(), m.nv(), raw, 3 * (size_t)ntri[k], eps[i]);
          p.hull = host::compact_hull(m.v.data(), ct.data(), ct.size() / 3, nullptr);
        }
        p.hullVol = vol[k];
        if (withHd && std::isfinite(hd[k])) {
          p.hd = hd[k];
          p.hasHd = true;
        }
      });
      // a hull that failed on the tree's slabs (more faces than its hull
      // bound allows) is built again on a second tree with room for every
      // point, where the reference falls back to its CPU hull (decompose.ts:
      // 183-188, merge.ts:371)
      for (size_t k = 0; k < n; k++) {
        const size_t i = order[s + k];
        if (!std::isnan(out[i].hullVol)) continue;
        if (!retry_hull(*ms[i], eps[i], withHd, out[i]) && !allowFail) {
          char msg[160];
          snprintf(msg, sizeof msg, "GPU hull failed (code %d) for a part with %u vertices", status[k], cm[k].nv);
          throw Failure{CUACD_E_CAPACITY, msg};
        }
      }
      s += n;
    }
  }

  // the hull (and Hausdorff distance) of one mesh on a tree whose hull bound
  // covers all of its points; false when that hull fails too
  void* bigTree = nullptr;
  uint32_t bigTreeVerts = 0;
  bool retry_hull(const Mesh& m, double eps, bool withHd, Part& p) {
    const uint32_t need = (uint32_t)m.nv();
    if (need <= (uint32_t)o.tree.hullMaxVerts) {
      // the bound already covered the points: a larger one does not help
      if (bigTree == nullptr || need > bigTreeVerts) return false;
    }
    if (bigTree == nullptr || bigTreeVerts < need) {
      if (bigTree) cuacd_tree_destroy(bigTree);
      cuacd_tree_config cfg = o.tree;
      cfg.hullMaxVerts = (int32_t)std::max<uint32_t>(need, 2 * (uint32_t)o.tree.hullMaxVerts);
      cfg.hullBudgetBytes = std::max<uint64_t>(cfg.hullBudgetBytes, (uint64_t)cfg.hullMaxVerts * 4096);
      int rc = 0;
      bigTree = cuacd_tree_create(&cfg, &rc);
      if (!bigTree) cuda_fail(rc, "hull retry tree");
      bigTreeVerts = (uint32_t)cfg.hullMaxVerts;
    }
    const cuacd_mesh cm{m.v.data(), m.t.data(), need, (uint32_t)m.nt()};
    const uint32_t stride = 6 * need;
    std::vector<uint32_t> tris((size_t)stride + 1);
    float vol = 0, hd = 0;
    uint32_t ntri = 0;
    int32_t status = 0;
    const auto t0 = Clock::now();
    const int rc = withHd ? cuacd_tree_hulls_with_hausdorff(bigTree, &cm, 1, tris.data(), stride, &vol, &ntri, &hd, &status)
                          : cuacd_tree_hull_meshes(bigTree, &cm, 1, 0, tris.data(), stride, &vol, &ntri, &status);
    gpuMs += ms_since(t0);
    if (rc != CUACD_OK) cuda_fail(rc, "hull retry");
    if (status != 0) return false;
    const std::vector<uint32_t> ct = host::clean_hull_faces(m.v.data(), m.nv(), tris.data(), 3 * (size_t)ntri, eps);
    p.hull = host::compact_hull(m.v.data(), ct.data(), ct.size() / 3, nullptr);
    p.hullVol = vol;
    if (withHd && std::isfinite(hd)) {
      p.hd = hd;
      p.hasHd = true;
    }
    return true;
  }

  // Hausdorff distances of pairs (a_k, b_k); batches of up to 1024, halved
  // when the sample scratch overflows (merge.ts:399-409); non-finite
  // results fall back to the CPU (decompose.ts:168)
  void hausdorff(const std::vector<const Mesh*>& a, const std::vector<const Mesh*>& b, std::vector<double>& out) {
    out.assign(a.size(), 0.0);
    size_t batch = CUACD_HD_MAX_PAIRS;
    for (size_t s = 0; s < a.size();) {
      const size_t n = std::min(batch, a.size() - s);
      std::vector<cuacd_mesh> ca(n), cb(n);
      for (size_t k = 0; k < n; k++) {
        ca[k] = cuacd_mesh{a[s + k]->v.data(), a[s + k]->t.data(), (uint32_t)a[s + k]->nv(), (uint32_t)a[s + k]->nt()};
        cb[k] = cuacd_mesh{b[s + k]->v.data(), b[s + k]->t.data(), (uint32_t)b[s + k]->nv(), (uint32_t)b[s + k]->nt()};
      }
      std::vector<float> r(n);
      const auto t0 = Clock::now();
      const int rc = cuacd_tree_hausdorff(tree, ca.data(), cb.data(), (int)n, r.data());
      gpuMs += ms_since(t0);
      if ((rc == CUACD_E_SCRATCH || rc == CUACD_E_CAPACITY) && n > 1) {
        batch = std::max<size_t>(1, n / 2);
        continue;
      }
      if (rc != CUACD_OK) cuda_fail(rc, "hausdorff batch");
      parallel_for(n, threads, [&](size_t k) {
        out[s + k] = std::isfinite(r[k]) ? (double)r[k] : host::hausdorff_cpu(*a[s + k], *b[s + k]);
      });
      s += n;
    }
  }

  // Hausdorff(part, hull) for parts that lack it (decompose.ts:159-170)
  void fill_hausdorff(const std::vector<Part*>& ps) {
    std::vector<const Mesh*> a, b;
    std::vector<Part*> todo;
    for (Part* p : ps)
      if (!p->hasHd) {
        resolve(*p);
        todo.push_back(p);
        a.push_back(&p->mesh);
        b.push_back(&p->hull);
      }
    if (todo.empty()) return;
    const auto t0 = Clock::now();
    std::vector<double> hd;
    hausdorff(a, b, hd);
    for (size_t k = 0; k < todo.size(); k++) {
      todo[k]->hd = hd[k];
      todo[k]->hasHd = true;
    }
    hdMs += ms_since(t0);
  }

  // refineSpacing (decompose.ts:199-211)
  double refine_spacing(const Mesh& m) const {
    const double minEdge = std::min((double)o.threshold / 4, 0.015);
    const int cpa = std::max(1, o.width / 3);
    float lo[3], hi[3];
    host::bbox(m, lo, hi);
    double s = INFINITY;
    for (int a = 0; a < 3; a++) {
      const double valid = (double)hi[a] - (double)lo[a] - 2 * minEdge;
      if (valid > 0) s = std::min(s, valid / (cpa + 1));
    }
    return std::isfinite(s) ? s : 0.0;
  }

  // ---- one decomposition iteration over all active jobs ------------------

  // One iteration (decompose.ts:258-358) of every job whose cutting is not
  // done; each job counts its own iterations, so jobs may join between
  // calls. Returns false when no job had a part to cut.
  bool iterate(std::vector<Job*>& jobs) {
    for (Job* j : jobs)
      if (!j->cutting_done && j->iter >= o.maxIters) j->cutting_done = true;
    // Hausdorff of the parts that lack it
    {
      std::vector<Part*> ps;
      for (Job* j : jobs)
        if (!j->cutting_done)
          for (Part& p : j->parts) ps.push_back(&p);
      fill_hausdorff(ps);
    }
    struct Seed {
      Job* job;
      size_t part;
    };
    std::vector<Seed> seeds;
    int iterShown = 0;
    for (Job* j : jobs) {
      if (j->cutting_done) continue;
      const int iter = j->iter++;
      iterShown = std::max(iterShown, iter);
      j->st.iterations = iter + 1;
      // ascending by cost; the last maxNCutting above the threshold
      std::vector<std::pair<double, size_t>> order;
      for (size_t i = 0; i < j->parts.size(); i++) order.push_back({part_cost(j->parts[i]), i});
      std::stable_sort(order.begin(), order.end(),
                       [](const std::pair<double, size_t>& x, const std::pair<double, size_t>& y) {
                         return x.first < y.first;
                       });
      std::vector<size_t> above;
      for (const auto& e : order)
        if (e.first >= o.threshold && !j->parts[e.second].stuck) above.push_back(e.second);
      const size_t from = above.size() > (size_t)o.maxNCutting ? above.size() - (size_t)o.maxNCutting : 0;
      if (from == above.size()) {
        j->cutting_done = true;
        continue;
      }
      for (size_t k = from; k < above.size(); k++) seeds.push_back(Seed{j, above[k]});
    }
    if (seeds.empty()) return false;
    // concave-edge planes of every cutting part (decompose.ts:276-281), one
    // GPU batch for all of them
    const auto tc = Clock::now();
    std::vector<std::vector<float>> planes(seeds.size());
    if (o.nConcaveEdges > 0) {
      std::vector<cuacd_mesh> cm;
      std::vector<uint32_t> sd;
      std::vector<size_t> which;
      for (size_t k = 0; k < seeds.size(); k++) {
        const int iter = seeds[k].job->iter - 1;
        if (iter >= o.concaveIters) continue;
        cm.push_back(resident(seeds[k].job->parts[seeds[k].part]));
        sd.push_back((uint32_t)(iter * 7919 + (int)seeds[k].part));
        which.push_back(k);
      }
      if (!cm.empty()) {
        const size_t per = 16 * (size_t)o.nConcaveEdges;
        std::vector<float> buf(per * cm.size());
        std::vector<int32_t> cnt(cm.size());
        const int rc = cuacd_tree_concave_planes(tree, cm.data(), (int)cm.size(), o.nConcaveEdges, o.concaveEps,
                                                 o.concaveThreshold, sd.data(), buf.data(), cnt.data());
        if (rc != CUACD_OK) cuda_fail(rc, "concave planes");
        for (size_t q = 0; q < which.size(); q++)
          planes[which[q]].assign(buf.begin() + q * per, buf.begin() + q * per + 4 * (size_t)cnt[q]);
      }
    }
    concaveMs += ms_since(tc);
    // the tree over all cutting parts, halving the batch on pool overflow
    // (decompose.ts:288-320)
    std::vector<cuacd_seed_result> best(seeds.size());
    const int nProbes = std::min(o.refineProbes, planeSlots);
    const bool refine = o.refineRounds > 0 && nProbes >= 3;
    size_t batch = seeds.size();
    for (size_t start = 0; start < seeds.size();) {
      const size_t n = std::min(batch, seeds.size() - start);
      std::vector<cuacd_mesh> cm(n);
      std::vector<float> spacing(n);
      size_t per = 0;
      for (size_t k = 0; k < n; k++) per = std::max(per, planes[start + k].size() / 4);
      std::vector<float> flat(std::max<size_t>(n * per * 4, 1), 0.0f);
      for (size_t k = 0; k < n; k++) {
        const Part& sp = seeds[start + k].job->parts[seeds[start + k].part];
        cm[k] = resident(sp);
        spacing[k] = refine ? (float)refine_spacing(sp.mesh) : 0.0f;
        std::copy(planes[start + k].begin(), planes[start + k].end(), flat.begin() + k * per * 4);
      }
      cuacd_run_opts ro{};
      ro.depth = 0;
      ro.width = -1;
      ro.nEdgeCuts = -1;
      ro.refineRounds = refine ? o.refineRounds : 0;
      ro.refineProbes = refine ? nProbes : 0;
      ro.refineSpacing = refine ? spacing.data() : nullptr;
      cuacd_run_stats rs{};
      const auto t0 = Clock::now();
      const int rc = cuacd_tree_run(tree, cm.data(), (int)n, flat.data(), (int)per, &ro, best.data() + start, &rs);
      const double dt = ms_since(t0);
      treeMs += dt;
      gpuMs += rs.gpuMs;
      if (rc == CUACD_E_CAPACITY && n > 1) {
        batch = std::max<size_t>(1, n / 2);
        continue;
      }
      if (rc != CUACD_OK) cuda_fail(rc, "tree run");
      if (rs.overflow) {
        if (n == 1) throw Failure{CUACD_E_CAPACITY, "GPU pool overflow with a single part; increase tree pool sizes"};
        batch = std::max<size_t>(1, n >> 1);
        continue;
      }
      if (rs.npOverflow) throw Failure{CUACD_E_CAPACITY, "tree depth exceeds LA_MAX_PARTS"};
      // every job whose seeds were in this run counts the run once and the
      // run's candidates in proportion to its seeds
      std::vector<Job*> seen;
      for (size_t k = 0; k < n; k++) {
        Job* j = seeds[start + k].job;
        if (std::find(seen.begin(), seen.end(), j) == seen.end()) {
          seen.push_back(j);
          j->st.treeRuns++;
          if (rs.hullFail) j->st.hullFailRuns++;
        }
        j->st.candidates += rs.validJobs / n;
      }
      start += n;
    }
    // apply the winning cuts (decompose.ts:327-343)
    const auto ta = Clock::now();
    struct Cut {
      bool ok = false;
      Mesh pos, neg;
    };
    std::vector<Cut> cuts(seeds.size());
    // every winning cut in one GPU batch (the host cut's halves bit for bit)
    std::vector<cuacd_mesh> cm;
    std::vector<int32_t> cutOf;
    std::vector<double> cutPlanes;
    std::vector<size_t> cutSeed;
    for (size_t k = 0; k < seeds.size(); k++) {
      Part& p = seeds[k].job->parts[seeds[k].part];
      const cuacd_seed_result& r = best[k];
      if (!(r.valid & 1)) {
        p.stuck = true;
        p.stuckReason = 1;
        continue;
      }
      cutOf.push_back((int32_t)cm.size());
      cm.push_back(resident(p));
      for (int a = 0; a < 4; a++) cutPlanes.push_back((double)r.plane[a]);
      cutSeed.push_back(k);
    }
    void* halvesH = nullptr;
    if (!cm.empty()) {
      // parts are closed when the input was checked closed and every cut's
      // halves are validated; otherwise the GPU cut also looks for open edges
      const int flags = o.requireClosed && o.validateCuts ? CUACD_CUT_CLOSED : 0;
      const int rc = cuacd_tree_plane_cuts(tree, cm.data(), (int)cm.size(), cutOf.data(), cutPlanes.data(),
                                           (int)cm.size(), flags, &halvesH);
      if (rc != CUACD_OK) cuda_fail(rc, "plane cuts");
      cutGen++;  // the batch's halves are the resident generation now
    }
    std::vector<host::CutResult> cutRes(seeds.size());
    // device copies of each cut's halves (positive, negative)
    std::vector<std::array<const void*, 4>> devHalf(seeds.size(), {nullptr, nullptr, nullptr, nullptr});
    for (size_t q = 0; q < cutSeed.size(); q++) {
      host::CutResult& c = cutRes[cutSeed[q]];
      const float* v[2];
      const uint32_t* t[2];
      uint32_t nv[2], nt[2];
      int st = 0;
      for (int sd = 0; sd < 2 && st == 0; sd++) st = cuacd_cuts_half(halvesH, (int)q, sd, &v[sd], &nv[sd], &t[sd], &nt[sd]);
      if (st != 0) continue;
      for (int sd = 0; sd < 2; sd++) {
        const float* dv = nullptr;
        const uint32_t* dt = nullptr;
        cuacd_cuts_half_device(halvesH, (int)q, sd, &dv, &dt);
        devHalf[cutSeed[q]][2 * sd] = dv;
        devHalf[cutSeed[q]][2 * sd + 1] = dt;
      }
      c.ok = true;
      c.pos.v.assign(v[0], v[0] + 3 * (size_t)nv[0]);
      c.pos.t.assign(t[0], t[0] + 3 * (size_t)nt[0]);
      c.neg.v.assign(v[1], v[1] + 3 * (size_t)nv[1]);
      c.neg.t.assign(t[1], t[1] + 3 * (size_t)nt[1]);
    }
    if (halvesH) cuacd_cuts_free(halvesH);
    const double cutGpu = ms_since(ta);
    parallel_for(seeds.size(), threads, [&](size_t k) {
      Part& p = seeds[k].job->parts[seeds[k].part];
      const cuacd_seed_result& r = best[k];
      if (!(r.valid & 1)) return;
      host::CutResult& c = cutRes[k];
      if (!c.ok) {
        p.stuck = true;
        p.stuckReason = 2;
        return;
      }
      if (c.pos.v.size() < 12 || c.neg.v.size() < 12) {
        p.stuck = true;
        p.stuckReason = 4;
        return;
      }
      if (o.validateCuts && (!host::is_closed(c.pos) || !host::is_closed(c.neg))) {
        p.stuck = true;
        p.stuckReason = 3;
        return;
      }
      cuts[k].ok = true;
      cuts[k].pos = std::move(c.pos);
      cuts[k].neg = std::move(c.neg);
    });
    cutMs += ms_since(ta);
    cutGpuMs += cutGpu;
    // hulls and Hausdorff distances of every new half in one submission
    std::vector<const Mesh*> halves;
    std::vector<cuacd_mesh> halvesDev;  // the same halves in the cut engine's output
    std::vector<double> heps;
    std::vector<size_t> which;
    bool allDev = true;
    for (size_t k = 0; k < seeds.size(); k++)
      if (cuts[k].ok) {
        halves.push_back(&cuts[k].pos);
        halves.push_back(&cuts[k].neg);
        for (int sd = 0; sd < 2; sd++) {
          const Mesh& h = sd == 0 ? cuts[k].pos : cuts[k].neg;
          const float* dv = (const float*)devHalf[k][2 * sd];
          const uint32_t* dt = (const uint32_t*)devHalf[k][2 * sd + 1];
          allDev &= dv != nullptr && dt != nullptr;
          halvesDev.push_back(cuacd_mesh{dv, dt, (uint32_t)h.nv(), (uint32_t)h.nt()});
        }
        heps.insert(heps.end(), 2, seeds[k].job->hullEps);
        which.push_back(k);
      }
    const auto th = Clock::now();
    std::vector<Part> made;
    hulls(halves, heps, true, made, false, true, nullptr, allDev ? &halvesDev : nullptr);
    for (size_t q = 0; q < which.size() && allDev; q++)
      for (int sd = 0; sd < 2; sd++) {
        made[2 * q + sd].dV = halvesDev[2 * q + sd].verts;
        made[2 * q + sd].dT = halvesDev[2 * q + sd].tris;
        made[2 * q + sd].gen = cutGen;
      }
    hullMs += ms_since(th);
    if (o.verbose) {
      size_t nParts = 0, nTris = 0;
      for (Job* j : jobs) nParts += j->parts.size();
      for (const Mesh* m : halves) nTris += m->nt();
      fprintf(stderr,
              "[iter %d] cutting %zu parts, %zu cuts applied, %zu half triangles, %zu parts; tree %.1f ms, hull %.1f ms, "
              "cut %.1f ms (GPU batch and readback %.1f), concave %.1f ms\n",
              iterShown, seeds.size(), which.size(), nTris, nParts + which.size(), treeMs, hullMs, cutMs, cutGpuMs,
              concaveMs);
    }
    // per job, in cutting order: the positive half replaces the part, the
    // negative half is appended
    for (size_t q = 0; q < which.size(); q++) {
      const Seed& sd = seeds[which[q]];
      if (o.verbose >= 2) {
        // every applied cut, enough to replay the loop on the host
        const cuacd_seed_result& r = best[which[q]];
        fprintf(stderr, "[cut] iter %d part %zu nt %zu plane %.9g %.9g %.9g %.9g -> %zu + %zu\n", sd.job->iter,
                sd.part, sd.job->parts[sd.part].mesh.nt(), r.plane[0], r.plane[1], r.plane[2], r.plane[3],
                made[2 * q].mesh.nt(), made[2 * q + 1].mesh.nt());
      }
      made[2 * q].id = nextId++;
      made[2 * q + 1].id = nextId++;
      sd.job->parts[sd.part] = std::move(made[2 * q]);
      sd.job->parts.push_back(std::move(made[2 * q + 1]));
    }
    return true;
  }

  // ---- merge pass (merge.ts:189-303), all jobs' rounds in lockstep --------

  static void bbox_of(const Mesh& m, float lo[3], float hi[3]) { host::bbox(m, lo, hi); }

  static bool tri_coplanar(const Mesh& m, size_t t, const Plane& p, double tol) {
    for (int e = 0; e < 3; e++) {
      const float* v = &m.v[3 * (size_t)m.t[t + e]];
      if (std::fabs(p.a * v[0] + p.b * v[1] + p.c * v[2] + p.d) > tol) return false;
    }
    return true;
  }

  static double coplanar_area(const Mesh& m, const Plane& p, double tol) {
    double area = 0;
    for (size_t t = 0; t < m.t.size(); t += 3) {
      if (!tri_coplanar(m, t, p, tol)) continue;
      const float* A = &m.v[3 * (size_t)m.t[t]];
      const float* B = &m.v[3 * (size_t)m.t[t + 1]];
      const float* C = &m.v[3 * (size_t)m.t[t + 2]];
      const double abx = (double)B[0] - A[0], aby = (double)B[1] - A[1], abz = (double)B[2] - A[2];
      const double acx = (double)C[0] - A[0], acy = (double)C[1] - A[1], acz = (double)C[2] - A[2];
      area += 0.5 * std::hypot(aby * acz - abz * acy, abz * acx - abx * acz, abx * acy - aby * acx);
    }
    return area;
  }

  // seamPlane (merge.ts:112-140): a face plane of A's hull with B's hull on
  // its outer side, carrying the most coplanar mesh area of A and B
  static bool seam_plane(const Part& A, const Part& B, double tol, Plane& out) {
    const std::vector<float>& hv = A.hull.v;
    const std::vector<uint32_t>& ht = A.hull.t;
    const std::vector<float>& bv = B.hull.v;
    std::vector<std::array<int64_t, 4>> seen;
    bool found = false;
    double bestArea = 0;
    auto jsround = [](double x) { return (int64_t)std::floor(x + 0.5); };
    for (size_t t = 0; t < ht.size(); t += 3) {
      const size_t i0 = 3 * (size_t)ht[t], i1 = 3 * (size_t)ht[t + 1], i2 = 3 * (size_t)ht[t + 2];
      const double e1x = (double)hv[i1] - hv[i0], e1y = (double)hv[i1 + 1] - hv[i0 + 1], e1z = (double)hv[i1 + 2] - hv[i0 + 2];
      const double e2x = (double)hv[i2] - hv[i0], e2y = (double)hv[i2 + 1] - hv[i0 + 1], e2z = (double)hv[i2 + 2] - hv[i0 + 2];
      double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
      const double len = std::hypot(nx, ny, nz);
      if (len < 1e-20) continue;
      nx /= len;
      ny /= len;
      nz /= len;
      const double d = nx * hv[i0] + ny * hv[i0 + 1] + nz * hv[i0 + 2];
      const std::array<int64_t, 4> key{jsround(nx * 2000), jsround(ny * 2000), jsround(nz * 2000), jsround(d * 2000)};
      if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
      seen.push_back(key);
      bool ok = true;
      for (size_t j = 0; j < bv.size(); j += 3)
        if (nx * bv[j] + ny * bv[j + 1] + nz * bv[j + 2] - d < -tol) {
          ok = false;
          break;
        }
      if (!ok) continue;
      const Plane p{nx, ny, nz, -d};
      const double area = coplanar_area(A.mesh, p, tol) + coplanar_area(B.mesh, p, tol);
      if (area > bestArea) {
        bestArea = area;
        out = p;
        found = true;
      }
    }
    return found;
  }

  // filteredConcat (merge.ts:143-157)
  static Mesh filtered_concat(const Mesh& a, const Mesh& b, const std::vector<Plane>& planes, double tol) {
    Mesh m = host::merge_meshes(a, b);
    if (planes.empty()) return m;
    std::vector<uint32_t> keep;
    keep.reserve(m.t.size());
    for (size_t t = 0; t < m.t.size(); t += 3) {
      bool drop = false;
      for (const Plane& p : planes)
        if (tri_coplanar(m, t, p, tol)) {
          drop = true;
          break;
        }
      if (!drop) keep.insert(keep.end(), m.t.begin() + t, m.t.begin() + t + 3);
    }
    m.t.swap(keep);
    return m;
  }

  void merge(std::vector<Job*>& all) {
    const auto tm = Clock::now();
    std::vector<Job*> jobs;
    for (Job* j : all)
      if (o.mergeHulls && j->parts.size() > 1) {
        j->merging = true;
        jobs.push_back(j);
      }
    const double halfT2 = ((double)o.threshold / 2) * ((double)o.threshold / 2);
    for (int round = 0; round < o.mergeRounds; round++) {
      struct Pair {
        Job* job;
        size_t i, j;
      };
      std::vector<Pair> todo;
      std::vector<std::vector<Pair>> cands(jobs.size());
      bool any = false;
      for (size_t q = 0; q < jobs.size(); q++) {
        Job* jb = jobs[q];
        if (!jb->merging) continue;
        if (jb->parts.size() <= 1) {
          jb->merging = false;
          continue;
        }
        any = true;
        jb->st.mergeRounds = round + 1;
        std::vector<std::array<float, 6>> box(jb->parts.size());
        for (size_t i = 0; i < jb->parts.size(); i++) bbox_of(jb->parts[i].mesh, &box[i][0], &box[i][3]);
        for (size_t i = 0; i < jb->parts.size(); i++)
          for (size_t j = i + 1; j < jb->parts.size(); j++) {
            const Part& A = jb->parts[i];
            const Part& B = jb->parts[j];
            const auto key = std::make_pair(std::min(A.id, B.id), std::max(A.id, B.id));
            if (jb->cache.count(key)) {
              cands[q].push_back(Pair{jb, i, j});
              continue;
            }
            if (rv_cost(A.meshVol + B.meshVol, A.hullVol + B.hullVol) >= o.threshold) continue;
            double g2 = 0;
            for (int k = 0; k < 3; k++) {
              const double g = std::max({0.0, (double)box[i][k] - box[j][3 + k], (double)box[j][k] - box[i][3 + k]});
              g2 += g * g;
            }
            if (g2 >= halfT2) continue;
            todo.push_back(Pair{jb, i, j});
            cands[q].push_back(Pair{jb, i, j});
          }
      }
      if (!any) break;
      // merged hulls of the pairs' hull points, one batch for every job
      std::vector<Mesh> pts(todo.size());
      for (size_t k = 0; k < todo.size(); k++) {
        const Part& A = todo[k].job->parts[todo[k].i];
        const Part& B = todo[k].job->parts[todo[k].j];
        pts[k].v = A.hull.v;
        pts[k].v.insert(pts[k].v.end(), B.hull.v.begin(), B.hull.v.end());
      }
      const auto th = Clock::now();
      std::vector<Part> hp;
      {
        std::vector<const Mesh*> ptr(todo.size());
        std::vector<double> peps(todo.size());
        for (size_t k = 0; k < todo.size(); k++) {
          ptr[k] = &pts[k];
          peps[k] = todo[k].job->hullEps;
        }
        const std::function<bool(size_t, double)> underThreshold = [&](size_t k, double hv) {
          const Part& A = todo[k].job->parts[todo[k].i];
          const Part& B = todo[k].job->parts[todo[k].j];
          return rv_cost(A.meshVol + B.meshVol, hv) < o.threshold;
        };
        hulls(ptr, peps, false, hp, true, false, &underThreshold);
      }
      hullMs += ms_since(th);
      const size_t base = evals.size();
      evals.resize(base + todo.size());
      for (size_t k = 0; k < todo.size(); k++) {
        const Part& A = todo[k].job->parts[todo[k].i];
        const Part& B = todo[k].job->parts[todo[k].j];
        PairEval& ev = evals[base + k];
        ev.hullVol = hp[k].hullVol;
        // a merged hull that failed on the GPU leaves the pair unmerged
        ev.cost = std::isnan(ev.hullVol) ? INFINITY : rv_cost(A.meshVol + B.meshVol, ev.hullVol);
        if (std::isnan(ev.hullVol)) todo[k].job->mergeHullFails++;
        ev.hasHull = ev.cost < o.threshold;
        if (ev.hasHull) ev.hull = std::move(hp[k].hull);
        todo[k].job->st.pairsHulled++;
      }
      // Hausdorff(filtered union, merged hull) of pairs still under the threshold
      std::vector<size_t> hdIdx;
      for (size_t k = 0; k < todo.size(); k++)
        if (evals[base + k].hasHull) hdIdx.push_back(k);
      std::vector<Mesh> unions(hdIdx.size());
      std::vector<char> nonEmpty(hdIdx.size(), 0);
      parallel_for(hdIdx.size(), threads, [&](size_t q) {
        const size_t k = hdIdx[q];
        const Part& A = todo[k].job->parts[todo[k].i];
        const Part& B = todo[k].job->parts[todo[k].j];
        PairEval& ev = evals[base + k];
        Plane sp;
        ev.hasSeam = seam_plane(A, B, o.mergePlaneTol, sp);
        if (ev.hasSeam) ev.seam = sp;
        std::vector<Plane> planes;
        if (ev.hasSeam) planes.push_back(ev.seam);
        planes.insert(planes.end(), A.seams.begin(), A.seams.end());
        planes.insert(planes.end(), B.seams.begin(), B.seams.end());
        unions[q] = filtered_concat(A.mesh, B.mesh, planes, o.mergePlaneTol);
        nonEmpty[q] = !unions[q].t.empty();
      });
      std::vector<const Mesh*> ha, hb;
      std::vector<size_t> hk;
      for (size_t q = 0; q < hdIdx.size(); q++)
        if (nonEmpty[q]) {
          ha.push_back(&unions[q]);
          hb.push_back(&evals[base + hdIdx[q]].hull);
          hk.push_back(hdIdx[q]);
        }
      const auto thd = Clock::now();
      std::vector<double> hd;
      hausdorff(ha, hb, hd);
      hdMs += ms_since(thd);
      if (o.verbose)
        fprintf(stderr, "[merge %d] %zu new pairs hulled, %zu Hausdorff pairs; hull %.1f ms, hausdorff %.1f ms\n", round,
                todo.size(), ha.size(), hullMs, hdMs);
      for (size_t q = 0; q < hk.size(); q++) {
        PairEval& ev = evals[base + hk[q]];
        ev.hd = hd[q];
        ev.cost = std::max(ev.cost, hd[q]);
        if (ev.cost >= o.threshold) {
          ev.hasHull = false;
          ev.hull = Mesh();
        }
        todo[hk[q]].job->st.pairsHausdorff++;
      }
      for (size_t k = 0; k < todo.size(); k++) {
        const Part& A = todo[k].job->parts[todo[k].i];
        const Part& B = todo[k].job->parts[todo[k].j];
        todo[k].job->cache[std::make_pair(std::min(A.id, B.id), std::max(A.id, B.id))] = base + k;
      }
      // greedy min-cost matching per job
      for (size_t q = 0; q < jobs.size(); q++) {
        Job* jb = jobs[q];
        if (!jb->merging) continue;
        struct Ranked {
          size_t i, j;
          size_t ev;
        };
        std::vector<Ranked> ranked;
        for (const Pair& c : cands[q]) {
          const Part& A = jb->parts[c.i];
          const Part& B = jb->parts[c.j];
          const size_t e = jb->cache[std::make_pair(std::min(A.id, B.id), std::max(A.id, B.id))];
          if (evals[e].cost < o.threshold && evals[e].hasHull) ranked.push_back(Ranked{c.i, c.j, e});
        }
        std::stable_sort(ranked.begin(), ranked.end(),
                         [&](const Ranked& x, const Ranked& y) { return evals[x.ev].cost < evals[y.ev].cost; });
        std::vector<char> used(jb->parts.size(), 0);
        std::vector<Part> next;
        int merges = 0;
        for (const Ranked& c : ranked) {
          if (used[c.i] || used[c.j]) continue;
          used[c.i] = used[c.j] = 1;
          const Part& A = jb->parts[c.i];
          const Part& B = jb->parts[c.j];
          const PairEval& ev = evals[c.ev];
          Part m;
          m.mesh = host::merge_meshes(A.mesh, B.mesh);
          m.hull = ev.hull;
          m.meshVol = A.meshVol + B.meshVol;
          m.hullVol = ev.hullVol;
          m.hd = ev.hd;
          m.hasHd = true;
          m.seams = A.seams;
          m.seams.insert(m.seams.end(), B.seams.begin(), B.seams.end());
          if (ev.hasSeam) m.seams.push_back(ev.seam);
          m.merged = A.merged + B.merged;
          m.id = nextId++;
          next.push_back(std::move(m));
          merges++;
        }
        if (merges == 0) {
          jb->merging = false;
          continue;
        }
        for (size_t i = 0; i < jb->parts.size(); i++)
          if (!used[i]) next.push_back(std::move(jb->parts[i]));
        jb->parts = std::move(next);
        jb->st.merges += merges;
      }
    }
    mergeMs += ms_since(tm);
  }

  // ---- the whole decomposition of a set of jobs ---------------------------

  // checks, normalisation and the first part (the whole mesh with its hull
  // and Hausdorff distance) of new jobs (decompose.ts:213-253)
  void begin(std::vector<Job*>& jobs) {
    for (Job* j : jobs) {
      if (o.requireClosed && !host::is_closed(j->input))
        throw Failure{CUACD_E_INVALID,
                      "input mesh is not closed (open or non-manifold edges); repair or remesh it first, or set "
                      "requireClosed: false"};
      if (o.normalize) {
        j->mesh = host::normalize(j->input, j->norm);
        j->normalized = true;
      } else {
        j->mesh = j->input;
      }
      float lo[3], hi[3];
      host::bbox(j->input, lo, hi);
      double maxAbs = 0, extent = 0;
      for (int a = 0; a < 3; a++) {
        maxAbs = std::max({maxAbs, std::fabs((double)lo[a]), std::fabs((double)hi[a])});
        extent = std::max(extent, (double)hi[a] - (double)lo[a]);
      }
      if (!(extent > 0)) extent = 1;
      j->hullEps = std::max(2e-5, 64 * 6e-8 * (maxAbs / extent));
    }
    std::vector<const Mesh*> ms;
    std::vector<double> meps;
    for (Job* j : jobs) {
      ms.push_back(&j->mesh);
      meps.push_back(j->hullEps);
    }
    std::vector<Part> made;
    const auto th = Clock::now();
    hulls(ms, meps, true, made, false, true);
    hullMs += ms_since(th);
    for (size_t k = 0; k < jobs.size(); k++) {
      made[k].id = nextId++;
      jobs[k]->parts.push_back(std::move(made[k]));
    }
  }

  // jobs whose cutting is done: the last Hausdorff distances, the merge pass
  // and the parts back in input units (decompose.ts:360-392)
  void finish(std::vector<Job*>& jobs) {
    evals.clear();  // pair evaluations live for one merge pass
    for (Job* j : jobs)
      for (Part& p : j->parts) resolve(p);
    {
      std::vector<Part*> ps;
      for (Job* j : jobs)
        for (Part& p : j->parts) ps.push_back(&p);
      fill_hausdorff(ps);
    }
    merge(jobs);
    for (Job* j : jobs) {
      if (!j->normalized) continue;
      for (Part& p : j->parts) {
        p.mesh = host::denormalize(p.mesh, j->norm);
        p.hull = host::denormalize(p.hull, j->norm);
        for (Plane& s : p.seams) s = host::denormalize_plane(s, j->norm);
      }
    }
  }

  void run(std::vector<Job*>& jobs) {
    begin(jobs);
    while (iterate(jobs)) {
    }
    finish(jobs);
  }

  // engines for concurrent groups of a batch (streams > 1), made on demand
  std::vector<std::unique_ptr<Engine>> peers;
  void reset_timers() {
    evals.clear();
    treeMs = cutMs = concaveMs = hullMs = hdMs = mergeMs = gpuMs = cutGpuMs = 0;
  }
  // The batch split over `streams` engines by triangle count (largest mesh
  // to the least loaded group), each group run on its own host thread; each
  // job records the engine that ran it.
  void run_groups(std::vector<Job*>& jobs, std::vector<Engine*>& ranBy);
};

Engine* make_engine(const cuacd_decompose_opts& o, int* err);

void Engine::run_groups(std::vector<Job*>& jobs, std::vector<Engine*>& ranBy) {
  const int G = (int)std::min<size_t>((size_t)std::max(o.streams, 1), jobs.size());
  ranBy.assign(jobs.size(), this);
  if (G <= 1) {
    reset_timers();
    run(jobs);
    return;
  }
  while ((int)peers.size() < G - 1) {
    int err = 0;
    Engine* p = make_engine(o, &err);
    if (!p) throw Failure{err ? err : CUACD_E_INVALID, std::string("stream engine: ") + cuacd_last_error()};
    peers.emplace_back(p);
  }
  std::vector<size_t> order(jobs.size());
  for (size_t k = 0; k < order.size(); k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return jobs[a]->input.nt() > jobs[b]->input.nt(); });
  std::vector<std::vector<Job*>> groups(G);
  std::vector<uint64_t> load(G, 0);
  for (size_t k : order) {
    const int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    groups[g].push_back(jobs[k]);
    load[g] += jobs[k]->input.nt() + 1;
    ranBy[k] = g == 0 ? this : peers[g - 1].get();
  }
  // the host threads of the merge geometry and hull cleanup are shared out
  const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
  const int per = std::max(2, (int)(hc / (unsigned)G));
  std::vector<Failure> errs(G);
  std::vector<int> bad(G, 0);
  std::vector<std::thread> th;
  for (int g = 0; g < G; g++) {
    Engine* en = g == 0 ? this : peers[g - 1].get();
    en->threads = o.threads > 0 ? o.threads : per;
    th.emplace_back([&, g, en]() {
      try {
        en->reset_timers();
        en->run(groups[g]);
      } catch (const Failure& f) {
        bad[g] = 1;
        errs[g] = f;
      } catch (const std::bad_alloc&) {
        bad[g] = 1;
        errs[g] = Failure{CUACD_E_CAPACITY, "host memory exhausted"};
      } catch (const std::exception& x) {
        // e.g. a worker thread the system would not start
        bad[g] = 1;
        errs[g] = Failure{CUACD_E_CAPACITY, std::string("host error: ") + x.what()};
      }
    });
  }
  for (std::thread& t : th) t.join();
  threads = o.threads > 0 ? o.threads : (int)hc;
  for (int g = 0; g < G; g++)
    if (bad[g]) throw errs[g];
}

// An Engine with its tree built from the options (decompose.ts:128-149).
Engine* make_engine(const cuacd_decompose_opts& o, int* err) {
  if (o.width % 3 != 0 || o.width2 % 3 != 0) {
    *err = set_error(CUACD_E_INVALID, "width and width2 must be multiples of 3");
    return nullptr;
  }
  if (!(o.threshold > 0) || o.maxNCutting < 1 || o.maxIters < 0 || o.mergeRounds < 0) {
    *err = set_error(CUACD_E_INVALID, "decomposer: invalid option");
    return nullptr;
  }
  std::unique_ptr<Engine> e(new Engine());
  e->o = o;
  cuacd_tree_config cfg = o.tree;
  cfg.width = o.width;
  cfg.width2 = o.width2;
  cfg.depth = o.depth;
  cfg.nConcaveEdges = o.nConcaveEdges;
  cfg.minEdgeDist = std::min(o.threshold / 4.0f, 0.015f);
  int rc = 0;
  e->tree = cuacd_tree_create(&cfg, &rc);
  if (!e->tree) {
    *err = rc ? rc : CUACD_E_INVALID;
    return nullptr;
  }
  e->o.tree = cfg;
  cuacd_set_profile(e->tree, o.profile);
  e->planeSlots = cuacd_plane_slots(e->tree);
  const unsigned hc = std::thread::hardware_concurrency();
  e->threads = o.threads > 0 ? o.threads : (int)std::max(1u, hc);
  *err = CUACD_OK;
  return e.release();
}

// ---------------------------------------------------------------------------
// Serving: continuous batching of decompositions under a device-memory
// budget. Requests wait in a queue (of at most maxQueue; a submission to a
// full queue is refused) and are admitted in arrival order while the device
// bytes of the server's trees, with the pools grown for every admitted
// request's working set, stay within the budget (one request is always
// admitted when none runs). A request's working set is the pool space of one
// lookahead run with its mesh as the seed: every job of level l splits a
// copy of at most the seed plus the intersection points (the halves hold the
// split triangles of the crossing edges), level 0 has width + planeSlots jobs
// per seed and each deeper level width2 times its parent level's; the
// estimate takes the seed's vertices and triangles once per job, with half
// again for the crossings. Every step runs one iteration of every admitted
// decomposition together (one tree launch per threshold, its pools grown
// beforehand so the launch needs no split), then finishes the ones with
// nothing left to cut (merge pass included), so a request that arrives while
// others are on the GPU joins them at the next step. A decomposition's parts
// do not depend on what else was admitted with it.
// bytes of pools with these capacities (vertex floats, triangle u32, open
// edges of 32 bytes, scratch u32)
static uint64_t pool_bytes(const uint64_t* c) { return 4 * c[0] + 4 * c[1] + 32 * c[2] + 4 * c[3]; }

// Pool space of one lookahead run with an (nv, nt) seed. Level l has J_l
// jobs (J_0 = width + planeSlots, J_l+1 = width2 J_l); a job's two children
// hold up to 2.5 nv + 64 vertices together (the children keep the parent's
// vertices on their side plus the intersection points), the children of the
// levels that keep topology (all but the last) 1.5 nt + 64 triangles and
// 16 sqrt(nt) + 64 open rim edges; a level's plan scratch is 2 words per
// parent vertex of each of its jobs. The oracle's tree runs on pools of
// exactly these sizes without overflow (tests/test_pool_estimate.py).
static void pool_working_set(int width, int width2, int depth, int planeSlots, uint64_t nv, uint64_t nt,
                             uint64_t* need) {
  uint64_t jobs = (uint64_t)width + (uint64_t)planeSlots, all = 0, topo = 0, last = 0;
  for (int l = 0; l < depth; l++) {
    all += jobs;
    if (l + 1 < depth) topo += jobs;
    last = jobs;
    jobs *= (uint64_t)width2;
  }
  const uint64_t rim = 16 * (uint64_t)std::ceil(std::sqrt((double)nt)) + 64;
  need[0] = all * 3 * (5 * nv / 2 + 64) + 3 * nv + 4096;
  need[1] = topo * 3 * (3 * nt / 2 + 64) + 3 * nt + 4096;
  need[2] = topo * rim + 4096;
  need[3] = 2 * last * (3 * nv / 2 + 64) + 4096;
}

struct Request {
  uint64_t ticket = 0;
  std::unique_ptr<Job> job;
  Clock::time_point submitted;
  float threshold = 0;
  uint64_t need[4] = {0, 0, 0, 0};  // working set in the pools: vertex floats, triangle u32, open edges, scratch u32
  uint64_t aux = 0;                  // allowance for the cut, concave-plane and Hausdorff buffers
  uint64_t bytes() const { return pool_bytes(need) + aux; }
};

class Server {
 public:
  cuacd_decompose_opts base{};
  uint64_t budget = 0;   // device bytes the server may hold
  size_t maxQueue = 0;   // 0: unbounded
  size_t maxActive = 0;  // running requests at most (slots); 0: unbounded
  int planeSlots = 0;
  std::map<uint32_t, std::unique_ptr<Engine>> engines;  // by threshold bits
  std::vector<Request> queue;                           // FIFO
  size_t queueHead = 0;
  std::vector<Request> active;
  std::map<uint64_t, std::unique_ptr<Result>> done;
  std::map<uint64_t, std::pair<int, std::string>> failed;
  uint64_t nextTicket = 1;
  uint64_t rejected = 0, peakBytes = 0, admittedTotal = 0;

  static uint32_t key_of(float thr) {
    uint32_t key;
    std::memcpy(&key, &thr, 4);
    return key;
  }
  Engine* engine_for(float thr) {
    const uint32_t key = key_of(thr);
    auto it = engines.find(key);
    if (it != engines.end()) return it->second.get();
    cuacd_decompose_opts o = base;
    o.threshold = thr;
    int err = 0;
    Engine* e = make_engine(o, &err);
    if (!e) throw Failure{err, cuacd_last_error()};
    engines.emplace(key, std::unique_ptr<Engine>(e));
    return e;
  }
  void working_set(uint64_t nv, uint64_t nt, uint64_t* need) const {
    pool_working_set(base.width, base.width2, base.depth, planeSlots, nv, nt, need);
  }
  // the buffers of the passes outside the tree pools grow with the work of
  // a step: the cut's inputs, classification, hash tables, cap arenas and
  // halves with the parts cut (at most the mesh and its caps), the tables
  // with the seeds, and the merge pass's hull and Hausdorff batches (chunks
  // of up to 1024 pairs) with the parts. A tree counts 64 MB for its batches and
  // each request 64 bytes per input byte, twice the growth measured on
  // icospheres of 1,280 triangles decomposed alone.
  static uint64_t aux_bytes(uint64_t nv, uint64_t nt) { return 64 * 12 * (nv + nt) + (1 << 20); }
  static constexpr uint64_t kTreeBatchBytes = 64ull << 20;
  struct Mem {
    uint64_t nonPool = 0, aux = 0, cap[4] = {0, 0, 0, 0}, need[4] = {0, 0, 0, 0};
    bool built = false;
  };
  // per tree at creation: bytes besides the pools, and the pools'
  // capacities; the hull slabs (up to hullBudgetBytes) and the buffers of
  // the cut, concave-plane and Hausdorff passes grow later
  uint64_t createdNonPool = 0, createdCap[4] = {0, 0, 0, 0}, hullBudget = 0;
  uint64_t mem_total(const Mem& x) const {
    const uint64_t fixed = std::max(x.nonPool, createdNonPool + hullBudget + kTreeBatchBytes + x.aux);
    uint64_t c[4];
    for (int k = 0; k < 4; k++) c[k] = std::max(x.cap[k], x.need[k]);
    return fixed + pool_bytes(c);
  }
  // device bytes of every tree (one not built yet counts as built), with
  // its pools grown to the working sets of the active requests and `extra`
  // device bytes of an engine's trees: its tree and, once a hull outgrew
  // that tree's bound, the larger tree that rebuilds such hulls
  static uint64_t engine_bytes(const Engine& e, uint64_t* caps4) {
    uint64_t held = 0, extra = 0;
    cuacd_tree_memory(e.tree, &held, caps4);
    if (e.bigTree) cuacd_tree_memory(e.bigTree, &extra, nullptr);
    return held + extra;
  }
  std::map<uint32_t, Mem> memory(const Request* extra) const {
    std::map<uint32_t, Mem> m;
    for (const auto& kv : engines) {
      Mem& x = m[kv.first];
      const uint64_t held = engine_bytes(*kv.second, x.cap);
      x.nonPool = held - pool_bytes(x.cap);
      x.built = true;
    }
    auto add = [&](const Request& r) {
      Mem& x = m[key_of(r.threshold)];
      if (!x.built)
        for (int k = 0; k < 4; k++) x.cap[k] = createdCap[k];
      for (int k = 0; k < 4; k++) x.need[k] += r.need[k];
      x.aux += r.aux;
    };
    for (const Request& r : active)
      if (r.job) add(r);
    if (extra) add(*extra);
    return m;
  }
  uint64_t projected(const Request* extra) const {
    uint64_t n = 0;
    for (const auto& kv : memory(extra)) n += mem_total(kv.second);
    return n;
  }
  bool engine_busy(uint32_t key) const {
    for (const Request& r : active)
      if (r.job && key_of(r.threshold) == key) return true;
    return false;
  }

  void complete(Request& r) {
    std::unique_ptr<Result> res(new Result());
    cuacd_decompose_stats s = r.job->st;
    s.nParts = (int32_t)r.job->parts.size();
    s.totalMs = ms_since(r.submitted);
    res->stats.push_back(s);
    res->parts.push_back(std::move(r.job->parts));
    done.emplace(r.ticket, std::move(res));
  }

  int step(int* completed) {
    int nDone = 0;
    // admission by device memory; a tree with no active request gives its
    // pools back (it is built again when a request needs it) when the next
    // request would not fit beside them
    std::vector<size_t> admitted;
    while (queueHead < queue.size()) {
      Request& q = queue[queueHead];
      if (maxActive && active.size() >= maxActive) break;
      if (!active.empty()) {
        if (projected(&q) > budget) {
          bool freed = false;
          for (auto it = engines.begin(); it != engines.end();) {
            if (!engine_busy(it->first)) {
              it = engines.erase(it);
              freed = true;
            } else {
              ++it;
            }
          }
          if (!freed || projected(&q) > budget) break;
        }
      }
      engine_for(q.threshold);
      active.push_back(std::move(q));
      admitted.push_back(active.size() - 1);
      admittedTotal++;
      queueHead++;
    }
    if (queueHead == queue.size()) {
      queue.clear();
      queueHead = 0;
    }
    // new jobs: a mesh that is not closed fails alone
    std::map<Engine*, std::vector<Job*>> fresh;
    for (size_t k : admitted) {
      Request& r = active[k];
      if (base.requireClosed && !host::is_closed(r.job->input)) {
        failed[r.ticket] = {CUACD_E_INVALID, "input mesh is not closed (open or non-manifold edges)"};
        r.job.reset();
        continue;
      }
      fresh[engine_for(r.threshold)].push_back(r.job.get());
    }
    for (auto& kv : fresh) kv.first->begin(kv.second);
    // the pools of each tree grow to its requests' working sets, so one
    // launch per threshold runs the whole step
    for (const auto& kv : memory(nullptr)) {
      auto it = engines.find(kv.first);
      if (it == engines.end()) continue;
      uint64_t c[4];
      for (int k = 0; k < 4; k++) c[k] = std::min<uint64_t>(std::max(kv.second.cap[k], kv.second.need[k]), 0xffffffffull);
      const int rc = cuacd_tree_reserve_pools(it->second->tree, c);
      if (rc != CUACD_OK) throw Failure{rc, cuacd_last_error()};
    }
    uint64_t held = 0;
    for (const auto& kv : engines) held += engine_bytes(*kv.second, nullptr);
    // one iteration of every admitted decomposition, per threshold
    std::map<Engine*, std::vector<Job*>> groups;
    for (Request& r : active)
      if (r.job) groups[engine_for(r.threshold)].push_back(r.job.get());
    for (auto& kv : groups) kv.first->iterate(kv.second);
    // the buffers of the cut and concave passes grow inside the step
    uint64_t after = 0;
    for (const auto& kv : engines) after += engine_bytes(*kv.second, nullptr);
    peakBytes = std::max({peakBytes, held, after});
    // decompositions with nothing left to cut finish together
    std::map<Engine*, std::vector<Job*>> fin;
    for (Request& r : active)
      if (r.job && r.job->cutting_done) fin[engine_for(r.threshold)].push_back(r.job.get());
    for (auto& kv : fin) kv.first->finish(kv.second);
    std::vector<Request> keep;
    for (Request& r : active) {
      if (!r.job) continue;
      if (r.job->cutting_done) {
        complete(r);
        nDone++;
      } else {
        keep.push_back(std::move(r));
      }
    }
    active.swap(keep);
    if (completed) *completed = nDone;
    return CUACD_OK;
  }
};

}  // namespace dec
}  // namespace cuacd

using namespace cuacd;
using namespace cuacd::dec;

extern "C" {

void cuacd_decompose_opts_default(cuacd_decompose_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->threshold = 0.05f;
  o->maxIters = 100;
  o->width = 30;
  o->width2 = 3;
  o->depth = 2;
  o->maxNCutting = 16;
  o->nConcaveEdges = 16;
  o->concaveEps = 0.005f;
  o->concaveThreshold = 3.49f;
  o->concaveIters = 10;
  o->normalize = 1;
  o->requireClosed = 1;
  o->validateCuts = 1;
  o->refineRounds = 2;
  o->refineProbes = 8;
  o->mergeHulls = 1;
  o->mergeRounds = 32;
  o->mergePlaneTol = 1e-3f;
  o->profile = 0;
  o->threads = 0;
  o->verbose = 0;
  o->streams = 1;
  cuacd_tree_config_default(&o->tree);
}

void* cuacd_decomposer_create(const cuacd_decompose_opts* o, int* err) {
  auto setErr = [&](int c) {
    if (err) *err = c;
  };
  if (!o) {
    setErr(set_error(CUACD_E_INVALID, "cuacd_decomposer_create: null options"));
    return nullptr;
  }
  int rc = 0;
  Engine* e = make_engine(*o, &rc);
  setErr(rc);
  return e;
}

void cuacd_decomposer_destroy(void* d) { delete static_cast<Engine*>(d); }

int cuacd_decompose(void* d, const cuacd_mesh* meshes, int n, int batched, void** result) {
  if (!d || !meshes || n < 1 || !result) return set_error(CUACD_E_INVALID, "cuacd_decompose: invalid argument");
  Engine* e = static_cast<Engine*>(d);
  *result = nullptr;
  std::vector<std::unique_ptr<Job>> jobs;
  for (int k = 0; k < n; k++) {
    const cuacd_mesh& m = meshes[k];
    if ((m.nv && !m.verts) || (m.nt && !m.tris)) return set_error(CUACD_E_INVALID, "cuacd_decompose: null mesh arrays");
    std::unique_ptr<Job> j(new Job());
    j->input.v.assign(m.verts, m.verts + 3 * (size_t)m.nv);
    j->input.t.assign(m.tris, m.tris + 3 * (size_t)m.nt);
    jobs.push_back(std::move(j));
  }
  std::unique_ptr<Result> res(new Result());
  try {
    e->reset_timers();
    const auto t0 = Clock::now();
    std::vector<Engine*> ranBy(jobs.size(), e);
    if (batched) {
      std::vector<Job*> all;
      for (auto& j : jobs) all.push_back(j.get());
      e->run_groups(all, ranBy);
    } else {
      for (auto& j : jobs) {
        std::vector<Job*> one{j.get()};
        e->evals.clear();
        e->run(one);
      }
    }
    const double total = ms_since(t0);
    for (size_t k = 0; k < jobs.size(); k++) {
      Job* j = jobs[k].get();
      const Engine* en = ranBy[k];
      cuacd_decompose_stats s = j->st;
      s.nParts = (int32_t)j->parts.size();
      s.totalMs = total;
      s.treeMs = en->treeMs;
      s.cutMs = en->cutMs;
      s.concaveMs = en->concaveMs;
      s.hullMs = en->hullMs;
      s.hausdorffMs = en->hdMs;
      s.mergeMs = en->mergeMs;
      s.gpuMs = en->gpuMs;
      res->stats.push_back(s);
      res->parts.push_back(std::move(j->parts));
    }
    e->evals.clear();
  } catch (const Failure& f) {
    e->evals.clear();
    return set_error(f.code, f.msg.c_str());
  } catch (const std::bad_alloc&) {
    e->evals.clear();
    return set_error(CUACD_E_CAPACITY, "cuacd_decompose: host memory exhausted");
  } catch (const std::exception& x) {
    e->evals.clear();
    return set_error(CUACD_E_CAPACITY, (std::string("cuacd_decompose: host error: ") + x.what()).c_str());
  }
  *result = res.release();
  return CUACD_OK;
}

void cuacd_merge_opts_default(cuacd_merge_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->threshold = 0.05f;
  o->maxRounds = 32;
  o->planeTol = 1e-3;
  o->hullEps = 2e-5;
}

static bool part_from(const cuacd_part_in& in, Part& p) {
  if ((in.mesh.nv && !in.mesh.verts) || (in.mesh.nt && !in.mesh.tris) || (in.hull.nv && !in.hull.verts) ||
      (in.hull.nt && !in.hull.tris) || (in.nSeams && !in.seams))
    return false;
  for (uint64_t k = 0; k < 3ull * in.mesh.nt; k++)
    if (in.mesh.tris[k] >= in.mesh.nv) return false;
  for (uint64_t k = 0; k < 3ull * in.hull.nt; k++)
    if (in.hull.tris[k] >= in.hull.nv) return false;
  p.mesh.v.assign(in.mesh.verts, in.mesh.verts + 3 * (size_t)in.mesh.nv);
  p.mesh.t.assign(in.mesh.tris, in.mesh.tris + 3 * (size_t)in.mesh.nt);
  p.hull.v.assign(in.hull.verts, in.hull.verts + 3 * (size_t)in.hull.nv);
  p.hull.t.assign(in.hull.tris, in.hull.tris + 3 * (size_t)in.hull.nt);
  p.meshVol = in.meshVol;
  p.hullVol = in.hullVol;
  p.hasHd = !std::isnan(in.hausdorff);
  p.hd = p.hasHd ? in.hausdorff : 0.0;
  for (uint32_t k = 0; k < in.nSeams; k++)
    p.seams.push_back(Plane{in.seams[4 * k], in.seams[4 * k + 1], in.seams[4 * k + 2], in.seams[4 * k + 3]});
  p.merged = in.merged > 0 ? in.merged : 1;
  return true;
}

int cuacd_merge_hulls(void* d, const cuacd_part_in* parts, int n, const cuacd_merge_opts* mo, void** result,
                      cuacd_merge_stats* stats) {
  if (!d || !result || n < 0 || (n > 0 && !parts)) return set_error(CUACD_E_INVALID, "cuacd_merge_hulls: invalid argument");
  Engine* e = static_cast<Engine*>(d);
  *result = nullptr;
  cuacd_merge_opts mopt;
  cuacd_merge_opts_default(&mopt);
  if (mo) mopt = *mo;
  if (!(mopt.threshold > 0) || mopt.maxRounds < 0 || !(mopt.planeTol >= 0))
    return set_error(CUACD_E_INVALID, "cuacd_merge_hulls: invalid options");
  Job j;
  j.hullEps = mopt.hullEps;
  for (int k = 0; k < n; k++) {
    Part p;
    if (!part_from(parts[k], p)) return set_error(CUACD_E_INVALID, "cuacd_merge_hulls: bad part arrays");
    p.id = e->nextId++;
    j.parts.push_back(std::move(p));
  }
  std::unique_ptr<Result> res(new Result());
  const cuacd_decompose_opts saved = e->o;
  e->o.threshold = mopt.threshold;
  e->o.mergeRounds = mopt.maxRounds;
  e->o.mergePlaneTol = (float)mopt.planeTol;
  e->o.mergeHulls = 1;
  e->o.verbose = mopt.verbose;
  try {
    e->reset_timers();
    const auto t0 = Clock::now();
    std::vector<Job*> jobs{&j};
    e->merge(jobs);
    e->evals.clear();
    cuacd_merge_stats st{};
    st.rounds = j.st.mergeRounds;
    st.merges = j.st.merges;
    st.pairsHulled = j.st.pairsHulled;
    st.pairsHausdorff = j.st.pairsHausdorff;
    st.hullFallbacks = j.mergeHullFails;
    st.hullMs = e->hullMs;
    st.hausdorffMs = e->hdMs;
    st.totalMs = ms_since(t0);
    if (stats) *stats = st;
    cuacd_decompose_stats ds = j.st;
    ds.nParts = (int32_t)j.parts.size();
    ds.totalMs = st.totalMs;
    ds.mergeMs = e->mergeMs;
    res->stats.push_back(ds);
    res->parts.push_back(std::move(j.parts));
  } catch (const Failure& f) {
    e->o = saved;
    e->evals.clear();
    return set_error(f.code, f.msg.c_str());
  } catch (const std::bad_alloc&) {
    e->o = saved;
    e->evals.clear();
    return set_error(CUACD_E_CAPACITY, "cuacd_merge_hulls: host memory exhausted");
  } catch (const std::exception& x) {
    e->o = saved;
    e->evals.clear();
    return set_error(CUACD_E_CAPACITY, (std::string("cuacd_merge_hulls: host error: ") + x.what()).c_str());
  }
  e->o = saved;
  *result = res.release();
  return CUACD_OK;
}

int cuacd_seam_plane(const cuacd_part_in* a, const cuacd_part_in* b, double tol, double* out4) {
  if (!a || !b || !out4) return set_error(CUACD_E_INVALID, "cuacd_seam_plane: invalid argument");
  Part A, B;
  if (!part_from(*a, A) || !part_from(*b, B)) return set_error(CUACD_E_INVALID, "cuacd_seam_plane: bad part arrays");
  Plane p{0, 0, 0, 0};
  if (!Engine::seam_plane(A, B, tol, p)) return 0;
  out4[0] = p.a;
  out4[1] = p.b;
  out4[2] = p.c;
  out4[3] = p.d;
  return 1;
}

int cuacd_filtered_concat(const cuacd_mesh* a, const cuacd_mesh* b, const double* planes, int nPlanes, double tol,
                          uint32_t* outTris, int cap) {
  if (!a || !b || nPlanes < 0 || (nPlanes > 0 && !planes) || cap < 0 || (cap > 0 && !outTris))
    return set_error(CUACD_E_INVALID, "cuacd_filtered_concat: invalid argument");
  Mesh ma, mb;
  ma.v.assign(a->verts, a->verts + 3 * (size_t)a->nv);
  ma.t.assign(a->tris, a->tris + 3 * (size_t)a->nt);
  mb.v.assign(b->verts, b->verts + 3 * (size_t)b->nv);
  mb.t.assign(b->tris, b->tris + 3 * (size_t)b->nt);
  for (uint32_t x : ma.t)
    if (x >= a->nv) return set_error(CUACD_E_INVALID, "cuacd_filtered_concat: triangle index out of range");
  for (uint32_t x : mb.t)
    if (x >= b->nv) return set_error(CUACD_E_INVALID, "cuacd_filtered_concat: triangle index out of range");
  std::vector<Plane> pl;
  for (int k = 0; k < nPlanes; k++) pl.push_back(Plane{planes[4 * k], planes[4 * k + 1], planes[4 * k + 2], planes[4 * k + 3]});
  const Mesh m = Engine::filtered_concat(ma, mb, pl, tol);
  const int nt = (int)m.nt();
  if (nt > cap) return set_error(CUACD_E_CAPACITY, "cuacd_filtered_concat: output buffer too small");
  std::copy(m.t.begin(), m.t.end(), outTris);
  return nt;
}

int cuacd_result_meshes(const void* r) { return r ? (int)static_cast<const Result*>(r)->parts.size() : 0; }

int cuacd_result_parts(const void* r, int mesh) {
  const Result* R = static_cast<const Result*>(r);
  if (!R || mesh < 0 || (size_t)mesh >= R->parts.size()) return set_error(CUACD_E_INVALID, "cuacd_result_parts: bad mesh");
  return (int)R->parts[(size_t)mesh].size();
}

int cuacd_result_part(const void* r, int mesh, int part, cuacd_part_view* out) {
  const Result* R = static_cast<const Result*>(r);
  if (!R || !out || mesh < 0 || (size_t)mesh >= R->parts.size() || part < 0 ||
      (size_t)part >= R->parts[(size_t)mesh].size())
    return set_error(CUACD_E_INVALID, "cuacd_result_part: bad index");
  const Part& p = R->parts[(size_t)mesh][(size_t)part];
  out->verts = p.mesh.v.data();
  out->tris = p.mesh.t.data();
  out->hullVerts = p.hull.v.data();
  out->hullTris = p.hull.t.data();
  out->seams = p.seams.empty() ? nullptr : &p.seams[0].a;
  out->nv = (uint32_t)p.mesh.nv();
  out->nt = (uint32_t)p.mesh.nt();
  out->hullNv = (uint32_t)p.hull.nv();
  out->hullNt = (uint32_t)p.hull.nt();
  out->nSeams = (uint32_t)p.seams.size();
  out->stuck = p.stuck ? 1 : 0;
  out->stuckReason = p.stuckReason;
  out->merged = p.merged;
  out->meshVol = p.meshVol;
  out->hullVol = p.hullVol;
  out->hausdorff = p.hasHd ? p.hd : NAN;
  return CUACD_OK;
}

int cuacd_result_stats(const void* r, int mesh, cuacd_decompose_stats* out) {
  const Result* R = static_cast<const Result*>(r);
  if (!R || !out || mesh < 0 || (size_t)mesh >= R->stats.size())
    return set_error(CUACD_E_INVALID, "cuacd_result_stats: bad mesh");
  *out = R->stats[(size_t)mesh];
  return CUACD_OK;
}

void cuacd_result_free(void* r) { delete static_cast<Result*>(r); }

// ---- serving -----------------------------------------------------------

void* cuacd_server_create(const cuacd_decompose_opts* o, uint64_t admitBytes, int32_t maxActive, int32_t maxQueue,
                          int* err) {
  if (!o || maxQueue < 0 || maxActive < 0) {
    if (err) *err = set_error(CUACD_E_INVALID, "cuacd_server_create: null options or negative bound");
    return nullptr;
  }
  std::unique_ptr<Server> s(new Server());
  s->base = *o;
  s->maxQueue = (size_t)maxQueue;
  s->maxActive = (size_t)maxActive;
  if (admitBytes == 0) {
    uint64_t total = 0;
    const int rc = cuacd_device_memory(&total, nullptr);
    if (rc != CUACD_OK) {
      if (err) *err = rc;
      return nullptr;
    }
    admitBytes = total / 5 * 4;  // 20 % headroom
  }
  s->budget = admitBytes;
  try {
    Engine* e = s->engine_for(o->threshold);  // validates the options and builds the first tree
    s->planeSlots = e->planeSlots;
    uint64_t held = 0;
    cuacd_tree_memory(e->tree, &held, s->createdCap);
    s->createdNonPool = held - pool_bytes(s->createdCap);
    s->hullBudget = e->o.tree.hullBudgetBytes;
  } catch (const Failure& f) {
    if (err) *err = set_error(f.code, f.msg.c_str());
    return nullptr;
  }
  if (err) *err = CUACD_OK;
  return s.release();
}

void cuacd_server_destroy(void* s) { delete static_cast<Server*>(s); }

int cuacd_server_submit(void* sv, const cuacd_mesh* m, float threshold, uint64_t* ticket) {
  Server* s = static_cast<Server*>(sv);
  if (!s || !m || !ticket || (m->nv && !m->verts) || (m->nt && !m->tris))
    return set_error(CUACD_E_INVALID, "cuacd_server_submit: invalid argument");
  for (size_t k = 0; k < 3 * (size_t)m->nt; k++)
    if (m->tris[k] >= m->nv) return set_error(CUACD_E_INVALID, "cuacd_server_submit: triangle index out of range");
  Request r;
  s->working_set(m->nv, m->nt, r.need);
  r.aux = Server::aux_bytes(m->nv, m->nt);
  if (r.bytes() > s->budget)
    return set_error(CUACD_E_CAPACITY, ("cuacd_server_submit: the mesh's working set (" + std::to_string(r.bytes()) +
                                        " bytes) exceeds the server's device budget")
                                           .c_str());
  if (s->maxQueue && s->queue.size() - s->queueHead >= s->maxQueue) {
    s->rejected++;
    return set_error(CUACD_E_BUSY, "cuacd_server_submit: queue full");
  }
  r.ticket = s->nextTicket++;
  r.job.reset(new Job());
  r.job->input.v.assign(m->verts, m->verts + 3 * (size_t)m->nv);
  r.job->input.t.assign(m->tris, m->tris + 3 * (size_t)m->nt);
  r.submitted = Clock::now();
  r.threshold = threshold > 0 ? threshold : s->base.threshold;
  *ticket = r.ticket;
  s->queue.push_back(std::move(r));
  return CUACD_OK;
}

int cuacd_pool_working_set(const cuacd_tree_config* cfg, uint32_t nv, uint32_t nt, uint64_t* caps4) {
  if (!cfg || !caps4 || cfg->depth < 1 || cfg->width < 0 || cfg->width2 < 0)
    return set_error(CUACD_E_INVALID, "cuacd_pool_working_set: invalid argument");
  pool_working_set(cfg->width, cfg->width2, cfg->depth, std::max(4 * cfg->nConcaveEdges, 32), nv, nt, caps4);
  return CUACD_OK;
}

int cuacd_server_stats(const void* sv, cuacd_server_state* out) {
  const Server* s = static_cast<const Server*>(sv);
  if (!s || !out) return set_error(CUACD_E_INVALID, "cuacd_server_stats: invalid argument");
  std::memset(out, 0, sizeof *out);
  out->budgetBytes = s->budget;
  for (const auto& kv : s->engines) out->deviceBytes += Server::engine_bytes(*kv.second, nullptr);
  out->peakDeviceBytes = std::max(s->peakBytes, out->deviceBytes);
  out->projectedBytes = s->projected(nullptr);
  for (const Request& r : s->active)
    if (r.job) out->workingSetBytes += r.bytes();
  out->admitted = s->admittedTotal;
  out->rejected = s->rejected;
  out->queued = (int32_t)(s->queue.size() - s->queueHead);
  out->active = (int32_t)s->active.size();
  return CUACD_OK;
}

int cuacd_server_step(void* sv, int* completed) {
  Server* s = static_cast<Server*>(sv);
  if (!s) return set_error(CUACD_E_INVALID, "cuacd_server_step: null server");
  try {
    return s->step(completed);
  } catch (const Failure& f) {
    return set_error(f.code, f.msg.c_str());
  } catch (const std::bad_alloc&) {
    return set_error(CUACD_E_CAPACITY, "cuacd_server_step: host memory exhausted");
  } catch (const std::exception& x) {
    return set_error(CUACD_E_CAPACITY, (std::string("cuacd_server_step: host error: ") + x.what()).c_str());
  }
}

int cuacd_server_pending(const void* sv) {
  const Server* s = static_cast<const Server*>(sv);
  return s ? (int)(s->queue.size() - s->queueHead + s->active.size()) : 0;
}

int cuacd_server_take(void* sv, uint64_t ticket, void** result) {
  Server* s = static_cast<Server*>(sv);
  if (!s || !result) return set_error(CUACD_E_INVALID, "cuacd_server_take: invalid argument");
  *result = nullptr;
  auto f = s->failed.find(ticket);
  if (f != s->failed.end()) {
    const int code = f->second.first;
    const std::string msg = f->second.second;
    s->failed.erase(f);
    return set_error(code, msg.c_str());
  }
  auto it = s->done.find(ticket);
  if (it == s->done.end()) return 1;
  *result = it->second.release();
  s->done.erase(it);
  return CUACD_OK;
}

// ---- host geometry entry points ----------------------------------------

namespace {
struct Halves {
  host::Mesh h[2];
};
host::Mesh to_mesh(const cuacd_mesh* m) {
  host::Mesh r;
  r.v.assign(m->verts, m->verts + 3 * (size_t)m->nv);
  r.t.assign(m->tris, m->tris + 3 * (size_t)m->nt);
  return r;
}
}  // namespace

int cuacd_plane_cut(const cuacd_mesh* mesh, const double* plane, void** halves) {
  if (!mesh || !plane || !halves || (mesh->nv && !mesh->verts) || (mesh->nt && !mesh->tris))
    return set_error(CUACD_E_INVALID, "cuacd_plane_cut: invalid argument");
  *halves = nullptr;
  const host::Mesh m = to_mesh(mesh);
  for (uint32_t x : m.t)
    if (x >= m.nv()) return set_error(CUACD_E_INVALID, "cuacd_plane_cut: triangle index out of range");
  host::CutResult r = host::plane_cut(m, Plane{plane[0], plane[1], plane[2], plane[3]});
  if (!r.ok) return set_error(CUACD_E_INVALID, r.reason ? r.reason : "cut failed");
  Halves* h = new Halves();
  h->h[0] = std::move(r.pos);
  h->h[1] = std::move(r.neg);
  *halves = h;
  return CUACD_OK;
}

int cuacd_cut_half(const void* halves, int side, const float** verts, uint32_t* nv, const uint32_t** tris,
                   uint32_t* nt) {
  const Halves* h = static_cast<const Halves*>(halves);
  if (!h || side < 0 || side > 1 || !verts || !nv || !tris || !nt)
    return set_error(CUACD_E_INVALID, "cuacd_cut_half: invalid argument");
  *verts = h->h[side].v.data();
  *nv = (uint32_t)h->h[side].nv();
  *tris = h->h[side].t.data();
  *nt = (uint32_t)h->h[side].nt();
  return CUACD_OK;
}

void cuacd_cut_free(void* halves) { delete static_cast<Halves*>(halves); }

int cuacd_concave_planes(const cuacd_mesh* mesh, int nConcaveEdges, double concaveEps, double concaveThreshold,
                         uint32_t seed, float* out, int cap) {
  if (!mesh || (mesh->nv && !mesh->verts) || (mesh->nt && !mesh->tris) || cap < 0 || (cap > 0 && !out))
    return set_error(CUACD_E_INVALID, "cuacd_concave_planes: invalid argument");
  const host::Mesh m = to_mesh(mesh);
  for (uint32_t x : m.t)
    if (x >= m.nv()) return set_error(CUACD_E_INVALID, "cuacd_concave_planes: triangle index out of range");
  const std::vector<float> p = host::concave_edge_planes(m, nConcaveEdges, concaveEps, concaveThreshold, seed);
  const int n = (int)(p.size() / 4);
  std::copy(p.begin(), p.begin() + 4 * (size_t)std::min(n, cap), out);
  return n;
}

int cuacd_quickhull(const double* pts, int n, double eps, double* vOut, int vCap, uint32_t* tOut, int tCap,
                    int* nvOut) {
  if (n < 0 || (n > 0 && !pts) || vCap < 0 || tCap < 0 || (vCap > 0 && !vOut) || (tCap > 0 && !tOut) || !nvOut)
    return set_error(CUACD_E_INVALID, "cuacd_quickhull: invalid argument");
  std::vector<double> hv;
  std::vector<uint32_t> ht;
  host::quickhull(pts, (size_t)n, eps, hv, ht);
  const int nv = (int)(hv.size() / 3), nt = (int)(ht.size() / 3);
  *nvOut = nv;
  if (nv > vCap || nt > tCap) return set_error(CUACD_E_CAPACITY, "cuacd_quickhull: output buffers too small");
  std::copy(hv.begin(), hv.end(), vOut);
  std::copy(ht.begin(), ht.end(), tOut);
  return nt;
}

int cuacd_clean_hull_faces(const cuacd_mesh* mesh, const uint32_t* tris, uint32_t nt, double eps, uint32_t* out,
                           int cap) {
  if (!mesh || (mesh->nv && !mesh->verts) || (nt && !tris) || cap < 0 || (cap > 0 && !out))
    return set_error(CUACD_E_INVALID, "cuacd_clean_hull_faces: invalid argument");
  for (size_t i = 0; i < 3 * (size_t)nt; i++)
    if (tris[i] >= mesh->nv) return set_error(CUACD_E_INVALID, "cuacd_clean_hull_faces: triangle index out of range");
  const std::vector<uint32_t> c = host::clean_hull_faces(mesh->verts, mesh->nv, tris, 3 * (size_t)nt, eps);
  const int n = (int)(c.size() / 3);
  if (n > cap) return set_error(CUACD_E_CAPACITY, "cuacd_clean_hull_faces: output buffer too small");
  std::copy(c.begin(), c.end(), out);
  return n;
}

}  // extern "C"
