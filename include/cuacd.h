/* cuacd.h — C ABI of the cuacd GB300 engine (libcuacd.so).
 *
 * The engine replaces the WebGPU hot path of cuacd-web: the lookahead tree
 * that GpuTree drives (src/gpu/tree.ts with the plan / scan / emit / hull /
 * record / evaluate kernels of src/gpu/shaders.ts), the sampled Hausdorff
 * kernel (src/gpu/hausdorff_shader.ts) and the GPU hull and Hausdorff
 * batches of the merge pass (src/merge.ts:357-416). Every entry point below
 * names the reference interface it stands in for.
 *
 * Conventions
 *   - Plain pointers and sizes only. Inputs are borrowed for the duration of
 *     the call and copied; outputs are caller-allocated.
 *   - Device meshes: cuacd_tree_run / _prepare, cuacd_tree_hull_meshes,
 *     cuacd_tree_plane_cuts and cuacd_tree_concave_planes also take meshes
 *     whose two buffers are device memory of the handle's device (for
 *     instance the halves cuacd_cuts_half_device returns): they are copied
 *     on the device, in the handle's stream order, and their indices are not
 *     checked on the host. The Hausdorff entry points take host meshes (the
 *     sample counts follow each mesh's area, computed on the host).
 *   - Return codes: CUACD_OK (0) or a negative CUACD_E_* code; the message
 *     of the last failure on the calling thread is cuacd_last_error().
 *   - Recoverable conditions of a tree run (pool overflow, hull failures,
 *     too many parts per item) are result flags, not errors, as in
 *     TreeRunResult (tree.ts:75-85): the caller halves the batch and retries
 *     (decompose.ts:316-321).
 *   - One handle owns one CUDA stream and its device pools; calls on one
 *     handle must not overlap (the reference serialises GpuTree calls with
 *     await). Different handles may be used from different threads.
 *   - Nothing here aborts the process or traps the device.
 */
#ifndef CUACD_H
#define CUACD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUACD_OK 0
#define CUACD_E_INVALID (-1)  /* bad argument or configuration */
#define CUACD_E_CAPACITY (-2) /* input exceeds a configured pool */
#define CUACD_E_SCRATCH (-3)  /* Hausdorff sample scratch exceeded (tree.ts:345) */
#define CUACD_E_CUDA (-4)     /* CUDA runtime error (allocation, launch) */
#define CUACD_E_NODEVICE (-5) /* no CUDA device */
#define CUACD_E_BUSY (-6)     /* a server's queue is full */

/* Maximum pairs of one Hausdorff call (HD_MAX_PAIRS, tree.ts:12). */
#define CUACD_HD_MAX_PAIRS 1024
/* Visible-face limit of one hull insertion (VIS_MAX, shaders.ts:27). */
#define CUACD_VIS_MAX 2048

/* TreeConfig (tree.ts:14-46). Capacities keep the reference's units:
 * vertexCap in floats (3 per vertex), triCap in u32 (3 per triangle),
 * edgeCap in open edges, scratchWords in u32. */
typedef struct {
  int32_t width;         /* axis-aligned cuts at level 0 (multiple of 3) */
  int32_t width2;        /* axis-aligned cuts at deeper levels (multiple of 3) */
  int32_t depth;         /* full levels, 1..4 */
  int32_t nConcaveEdges; /* edge planes per seed = max(4 * nConcaveEdges, 32) */
  float minEdgeDist;
  int32_t hullMaxVerts;  /* hull export bound per part */
  uint64_t vertexCap;
  uint64_t triCap;
  uint64_t edgeCap;
  uint64_t scratchWords;
  uint64_t hullBudgetBytes; /* bytes of hull scratch slabs in flight */
  int32_t pruneLastLevel;   /* last-level branch and bound (tree.ts:29-30) */
  int32_t warpMaxNv;        /* hulls of parts up to this many points run on one
                               warp each, larger ones on a 256-thread block
                               (0: 1024); the results do not depend on it */
  int32_t hdScreenMinTris;  /* Hausdorff target meshes with at least this many
                               triangles go through the tensor-core screen
                               (0: 256, < 0: never); the results do not
                               depend on it */
  int32_t autotune;         /* 1 (the default): when warpMaxNv is 0, the
                               warp/block thresholds of the hull and of
                               plan/emit are chosen per distribution of part
                               sizes (log2 buckets of the largest, median and
                               total point counts and of the part count): the
                               first runs or hull batches of each distribution
                               try the schedules in turn, later ones use the
                               fastest; the results do not depend on it */
} cuacd_tree_config;

/* Mesh (mesh.ts:7-10): nv vertices (3 floats each), nt triangles (3 u32). */
typedef struct {
  const float* verts;
  const uint32_t* tris;
  uint32_t nv;
  uint32_t nt;
} cuacd_mesh;

/* GpuTree.run opts (tree.ts:449-453) and RefineRequest (tree.ts:60-67). */
typedef struct {
  int32_t depth;        /* <= 0: configured depth */
  int32_t width;        /* < 0: configured width */
  int32_t nEdgeCuts;    /* < 0: every plane slot */
  int32_t refineRounds; /* probe rounds after the tree, 0 = none */
  int32_t refineProbes; /* probes per round (>= 3) */
  int32_t reserved;
  const float* refineSpacing; /* per seed initial half-width, or NULL */
} cuacd_run_opts;

/* SeedResult (tree.ts:69-73). */
typedef struct {
  int32_t bestCut; /* index into the seed's candidate planes, -1 if none */
  float bestCost;  /* +inf when no cut */
  float plane[4];  /* a, b, c, d with a x + b y + c z + d = 0 */
  int32_t valid;
  int32_t reserved;
} cuacd_seed_result;

/* TreeRunResult flags and stats (tree.ts:75-85). */
typedef struct {
  uint32_t overflow;
  uint32_t hullFail;
  uint32_t hullFailCount;
  uint32_t npOverflow;
  uint32_t pruned;
  uint32_t nLevels;
  uint32_t jobsPerLevel[4];
  uint64_t validJobs; /* candidate cuts evaluated (jobs valid after plan, all stages) */
  uint32_t hullSlabWords;
  uint32_t hullChunkSize; /* hull scratch slabs in flight */
  float gpuMs;            /* device time of the run */
  uint32_t reserved;
} cuacd_run_stats;

/* DEFAULT_TREE_CONFIG (tree.ts:33-46), with width2 = 3 (decompose.ts:91). */
void cuacd_tree_config_default(cuacd_tree_config* cfg);

/* new GpuTree(device, cfg) (tree.ts:139-178): validates width/width2 (multiples
 * of 3) and depth (1..4), allocates the device pools on the current device.
 * Returns NULL and sets *err on failure. */
void* cuacd_tree_create(const cuacd_tree_config* cfg, int* err);

/* GpuTree.destroy (tree.ts:813-815). */
void cuacd_tree_destroy(void* tree);

/* cudaMemGetInfo of the current device: total and free bytes (either
 * pointer may be NULL). */
int cuacd_device_memory(uint64_t* total, uint64_t* freeBytes);

/* Device memory of a handle (no counterpart in the reference, whose pools
 * are fixed at construction, tree.ts:150-176): *deviceBytes = bytes held by
 * its pools, tables, hull slabs and the buffers of its GPU cut and
 * concave-plane passes; caps4 = the pools' current capacities in the
 * configuration's units: vertexCap (floats), triCap (u32), edgeCap (open
 * edges, 32 bytes each), scratchWords (u32). Either output may be NULL. */
int cuacd_tree_memory(const void* tree, uint64_t* deviceBytes, uint64_t* caps4);

/* Pool space of one lookahead run with an (nv, nt) seed on a tree of this
 * configuration (no reference counterpart; the server's working-set
 * estimate): caps4 = {vertex floats, triangle u32, open edges, scratch u32}.
 * Level l has J_l jobs (J_0 = width + max(4 nConcaveEdges, 32), J_l+1 =
 * width2 J_l); each job's children hold up to 2.5 nv + 64 vertices, the
 * children of every level but the last 1.5 nt + 64 triangles and
 * 16 sqrt(nt) + 64 open edges, and a level's plan scratch is 2 words per
 * parent vertex per job. A run on pools of these sizes does not overflow. */
int cuacd_pool_working_set(const cuacd_tree_config* cfg, uint32_t nv, uint32_t nt, uint64_t* caps4);

/* The autotuner's state (no reference counterpart): out4[0] = the largest
 * part a warp hulls and out4[1] = the largest parent a warp plans and emits
 * in the last prepared run or hull batch, out4[2] = 1 when that run tries a
 * schedule for its distribution of part sizes, out4[3] = distributions whose
 * trials are complete. */
int cuacd_tree_schedule(const void* tree, int32_t* out4);

/* Grows the pools to at least caps4 = {vertexCap, triCap, edgeCap,
 * scratchWords} (pools never shrink; at most 2^32 - 1 each). Waits for the
 * handle's stream and drops a prepared run. When the device refuses an
 * allocation that pool keeps its old capacity and CUACD_E_CUDA is returned. */
int cuacd_tree_reserve_pools(void* tree, const uint64_t* caps4);

/* GpuTree.planeSlots (tree.ts:759-761): plane slots per seed. */
int cuacd_plane_slots(const void* tree);

/* GpuTree.visMax (tree.ts:809-811). */
int cuacd_vis_max(void);

/* GpuTree.profile (tree.ts:133-134): when on, runs launch kernel by kernel
 * with CUDA events between them instead of replaying a CUDA graph. */
void cuacd_set_profile(void* tree, int on);

/* stats.kernelMs of the last profiled run (tree.ts:82, 610-615): device time
 * per kernel class, summed over levels and rounds, in ms: [0] table reset,
 * [1] plan, [2] scan, [3] emit, [4] hull, [5] record, [6] evaluate. */
int cuacd_tree_kernel_ms(void* tree, float* ms7);

/* Algorithmic bytes of the last run's plan, emit and hull kernels: each
 * candidate reads its parent once (12 nv + 12 nt + 32 ne), writes its
 * children once, and each child's points are read once by its hull. */
int cuacd_tree_kernel_bytes(void* tree, uint64_t* bytes3);

/* Hausdorff tensor-core screen of the last Hausdorff batch on this handle
 * (no reference counterpart): [0] exact point-triangle distances computed,
 * [1] sample-triangle pairs screened, [2] 1 when a tensor-core wait timed out
 * (the batch's distances are then incomplete). */
int cuacd_tree_hd_stats(void* tree, uint64_t* out3);

/* GpuTree.lastHullGpuMs (tree.ts:380): device time of the last completed
 * call on this handle (tree run, hull batch or Hausdorff batch), in ms. */
float cuacd_tree_last_gpu_ms(void* tree);

/* GpuTree.run (tree.ts:449-661). edgePlanes holds planesPerSeed planes
 * (4 floats) per seed; zero planes are skipped; planes beyond planeSlots are
 * ignored. out receives nSeeds results. */
int cuacd_tree_run(void* tree, const cuacd_mesh* seeds, int nSeeds, const float* edgePlanes, int planesPerSeed,
                   const cuacd_run_opts* opts, cuacd_seed_result* out, cuacd_run_stats* stats);

/* The two halves of cuacd_tree_run for device-resident reruns: prepare
 * uploads seeds and planes (tree.ts:470-557); launch enqueues the whole tree,
 * evaluate and refinement rounds on the handle's stream, starting from the
 * prepared seeds (tree.ts:559-594); collect waits and reads the results
 * (tree.ts:596-661). launch may be called any number of times after one
 * prepare. */
int cuacd_tree_prepare(void* tree, const cuacd_mesh* seeds, int nSeeds, const float* edgePlanes, int planesPerSeed,
                       const cuacd_run_opts* opts);
int cuacd_tree_launch(void* tree);
int cuacd_tree_collect(void* tree, cuacd_seed_result* out, cuacd_run_stats* stats);

/* GpuTree.hausdorff (tree.ts:318-372): bidirectional sampled Hausdorff of n
 * pairs (n <= CUACD_HD_MAX_PAIRS). Returns CUACD_E_SCRATCH when the pairs'
 * sample capacity exceeds scratchWords (the reference throws an Error whose
 * message contains "scratch"; merge.ts:405 halves the batch on it). */
int cuacd_tree_hausdorff(void* tree, const cuacd_mesh* a, const cuacd_mesh* b, int n, float* out);

/* GpuTree.hullMeshes (tree.ts:382-443): exact convex hulls of n meshes or
 * point sets (nt = 0). For mesh k, up to exportStride u32 of outward hull
 * triangles over its own vertex indices go to trisOut + k * exportStride,
 * the triangle count to ntOut[k], the volume to volOut[k], and status[k] is
 * 0, or the reference's failure code (lastHullFails, tree.ts:668, 752):
 * 1 visible-set overflow, 2 face slots exhausted, 3 slab too small,
 * 8 fewer than 4 faces, 9 other. hullStage 1/2/3 stop after the seeds,
 * the seed insertion or the first assignment (tests/bench_hull.ts:2-4).
 * trisOut may be NULL (noExport). */
int cuacd_tree_hull_meshes(void* tree, const cuacd_mesh* meshes, int n, int hullStage, uint32_t* trisOut,
                           uint32_t exportStride, float* volOut, uint32_t* ntOut, int32_t* status);

/* GpuTree.hullsWithHausdorff (tree.ts:671-756): hulls as above plus the
 * Hausdorff distance of each mesh to its hull, in one submission. */
int cuacd_tree_hulls_with_hausdorff(void* tree, const cuacd_mesh* meshes, int n, uint32_t* trisOut,
                                    uint32_t exportStride, float* volOut, uint32_t* ntOut, float* hdOut,
                                    int32_t* status);

/* Debug readers of the last run's tables, in the reference's word layouts
 * (shaders.ts:41-60): items 20 words, parts 16 words, jobs 24 words. Part
 * offsets keep the reference's units (vOff in floats, tOff in u32, eOff in
 * edges). GpuTree.readPart / readPlane / levels (tree.ts:764-807, 621-639). */
int cuacd_tree_read_items(void* tree, uint32_t first, uint32_t n, uint32_t* out);
int cuacd_tree_read_parts(void* tree, uint32_t first, uint32_t n, uint32_t* out);
int cuacd_tree_read_jobs(void* tree, uint32_t first, uint32_t n, uint32_t* out);
int cuacd_tree_read_part_geometry(void* tree, uint32_t part, float* verts, uint32_t* tris, uint32_t* edges);
int cuacd_tree_read_plane(void* tree, uint32_t index, float* out4);

/* Convex hull of one point set without allocating device memory. No
 * counterpart in the reference: it serves callers that cannot allocate at
 * the moment they need a hull (a host application whose own arena or
 * caching allocator owns the device memory, or an interactive loop that
 * must not stall running work on cudaMalloc / cudaFree). The caller passes
 * device buffers it owns: points (nv * 3 floats), tris (trisCap u32), and
 * one float, one u32 and one i32 for the volume, the triangle count and the
 * status (as cuacd_tree_hull_meshes: 0, or the failure code, 8 for fewer
 * than 4 points or a flat set). A hull of nv points has at most 2 nv - 4
 * triangles, so trisCap must be at least 3 * max(2 nv - 4, 4) u32; a smaller
 * buffer is refused with CUACD_E_CAPACITY before any work is queued (no
 * hull is ever cut short). The kernel's scratch is a fixed array of about
 * 1.7 MiB inside the library, which every GPU that loads the library keeps
 * until exit; it holds at most 4096 points, and larger sets are rejected
 * with CUACD_E_CAPACITY. Work is queued on `stream` (a cudaStream_t of the
 * current device, NULL for the default stream); results are valid once that
 * stream has completed. The first call in a CUDA context (the first on a
 * device, and the first after its context was re-created) looks up the
 * array's device address in that context, so make it before any stream
 * capture. All calls share the one array and each leaves its contents
 * behind: calls that overlap on the GPU (different streams, or different
 * host threads) race and must be serialised. */
int cuacd_hull_points_noalloc(const float* points, uint32_t nv, uint32_t* tris, uint32_t trisCap, float* volume,
                              uint32_t* ntris, int32_t* status, void* stream);

/* planeCut (src/cpu/cut.ts:33-315) of nCuts (mesh, plane) pairs on the GPU,
 * on the tree handle's stream: cut k cuts meshes[meshOfCut[k]] by planes[4k
 * .. 4k + 3] (a x + b y + c z + d = 0). The halves are the host cut's
 * (cuacd_plane_cut) bit for bit: the same vertices in the same order, the
 * same triangles, caps and failures, for open meshes too. flags:
 * CUACD_CUT_CLOSED when the caller vouches that every mesh is closed (each
 * directed edge has a reverse, as the decomposer's parts do), which skips
 * the search for open input edges. On success *halves receives a handle read
 * with cuacd_cuts_half. */
#define CUACD_CUT_CLOSED 1
int cuacd_tree_plane_cuts(void* tree, const cuacd_mesh* meshes, int nMeshes, const int32_t* meshOfCut,
                          const double* planes, int nCuts, int flags, void** halves);
/* Half `side` (0 positive, 1 negative) of cut `cut`: returns 0 with the
 * half's arrays (valid until cuacd_cuts_free), or the cut's failure: 1 the
 * plane does not split the mesh, 2 open boundary chain, 3 boundary chain dead
 * end, 4 boundary chain cycle (the reasons cut.ts throws), 5 an internal
 * scratch bound was exceeded; or a negative error. */
int cuacd_cuts_half(const void* halves, int cut, int side, const float** verts, uint32_t* nv, const uint32_t** tris,
                    uint32_t* nt);
/* The same half in device memory (no counterpart in the reference): the
 * GPU cut's output buffers keep every half of the batch until the next
 * cuacd_tree_plane_cuts (or cuacd_tree_eval_cuts) on the same handle, also
 * after cuacd_cuts_free, so the next steps can take the halves as device
 * meshes (see the conventions on device meshes). Same return as
 * cuacd_cuts_half. */
int cuacd_cuts_half_device(const void* halves, int cut, int side, const float** verts, const uint32_t** tris);
/* concaveEdgePlanes (src/cpu/concave.ts:25-92) of n meshes on the GPU, on
 * the tree handle's stream: mesh k's planes (at most 4 * nConcaveEdges, 4
 * floats each) go to out + 16 * nConcaveEdges * k and their count to
 * counts[k]; seeds[k] is the mesh's reservoir seed. The planes are
 * cuacd_concave_planes' bit for bit. */
int cuacd_tree_concave_planes(void* tree, const cuacd_mesh* meshes, int n, int nConcaveEdges, double concaveEps,
                              double concaveThreshold, const uint32_t* seeds, float* out, int32_t* counts);
/* Device time of the last cuacd_tree_concave_planes, in ms. */
float cuacd_tree_concave_ms(void* tree);

/* The reference's CPU helpers applied to candidate cuts of one mesh
 * (planeCut, convexHull, volumes and rv, hausdorff: src/cpu/cut.ts,
 * src/cpu/hull.ts, src/mesh.ts:58-72, src/part.ts:24-26, src/cpu/
 * hausdorff.ts), on the GPU: the capped cut of every plane in one batch,
 * then one hull + Hausdorff batch over all halves. out8 receives 8 doubles
 * per plane: split (1 or 0), |volume| of the positive and negative half,
 * their hull volumes, their rv costs, and the larger of the two halves'
 * Hausdorff distances to their hulls (samples by hausdorff_shader.ts:57-78).
 * Planes that do not split the mesh leave zeros. */
int cuacd_tree_eval_cuts(void* tree, const cuacd_mesh* mesh, const double* planes, int n, double* out8);
/* Device time of the last cuacd_tree_eval_cuts (cut batch + hull batches). */
float cuacd_tree_eval_cuts_ms(void* tree);
/* Device time of the batch (uploads, kernels and the readback), in ms. */
float cuacd_cuts_gpu_ms(const void* halves);
void cuacd_cuts_free(void* halves);

/* ---- decomposition (src/decompose.ts, src/merge.ts) -------------------- */

/* DecomposeOptions (decompose.ts:26-78) with DEFAULT_OPTIONS (decompose.ts:
 * 83-106). The GPU tree of the decomposer is built from `tree` with width,
 * width2, depth and nConcaveEdges taken from the options and minEdgeDist =
 * min(threshold / 4, 0.015) (decompose.ts:141-147). Hulls and Hausdorff
 * distances always run on the GPU (hullBackend / hausdorffBackend "gpu"). */
typedef struct {
  float threshold;
  int32_t maxIters;
  int32_t width;
  int32_t width2;
  int32_t depth;
  int32_t maxNCutting;
  int32_t nConcaveEdges;
  float concaveEps;
  float concaveThreshold;
  int32_t concaveIters;
  int32_t normalize;     /* centre and scale to extent 2 */
  int32_t requireClosed; /* reject input that is not a closed manifold */
  int32_t validateCuts;  /* a cut whose halves are not closed leaves the part */
  int32_t refineRounds;
  int32_t refineProbes;
  int32_t mergeHulls;
  int32_t mergeRounds;
  float mergePlaneTol;
  int32_t profile;
  int32_t threads; /* host threads for hull cleanup and merge geometry, 0 = all cores */
  int32_t verbose; /* 1: one line per iteration and merge round on stderr;
                      2: also every applied cut (part, plane, half sizes) */
  int32_t streams; /* batched decompositions: meshes are split (by triangle
                      count) over this many engines, each with its own tree,
                      CUDA stream and host thread, so one group's latency-bound
                      levels overlap another's; 0 or 1 = one engine. The
                      parts do not depend on it. */
  cuacd_tree_config tree;
} cuacd_decompose_opts;

/* Part (part.ts:9-22) of a finished decomposition, in input units. The
 * pointers stay valid until cuacd_result_free. hausdorff is NaN when unset.
 * stuckReason: 0 none, 1 no-plane, 2 cut-failed, 3 not-closed, 4 degenerate. */
typedef struct {
  const float* verts;
  const uint32_t* tris;
  const float* hullVerts;
  const uint32_t* hullTris;
  const double* seams; /* 4 doubles per seam plane */
  uint32_t nv, nt, hullNv, hullNt, nSeams;
  int32_t stuck;
  int32_t stuckReason;
  int32_t merged;
  double meshVol;
  double hullVol;
  double hausdorff;
} cuacd_part_view;

/* DecomposeResult.stats and MergeStats (decompose.ts:112-120, merge.ts:
 * 53-66) of one mesh. Times are of the whole call (every mesh of a batched
 * call shares them). candidates = cut candidates the tree evaluated. */
typedef struct {
  int32_t iterations;
  int32_t treeRuns;
  int32_t hullFailRuns;
  int32_t nParts;
  int32_t mergeRounds;
  int32_t merges;
  int32_t pairsHulled;
  int32_t pairsHausdorff;
  uint64_t candidates;
  double totalMs, treeMs, cutMs, concaveMs, hullMs, hausdorffMs, mergeMs, gpuMs;
} cuacd_decompose_stats;

void cuacd_decompose_opts_default(cuacd_decompose_opts* o);
/* new Decomposer(device, opts) (decompose.ts:128-149): validates the options
 * and creates the GPU tree. NULL on failure (err set). */
void* cuacd_decomposer_create(const cuacd_decompose_opts* o, int* err);
void cuacd_decomposer_destroy(void* d);
/* Decomposer.decompose (decompose.ts:213-392) of n meshes. batched = 0 runs
 * them one after another; batched != 0 advances all of them together, so one
 * tree launch per iteration serves the cutting parts of every mesh and hull,
 * Hausdorff and merge batches are shared. The results are the same either
 * way. On success *result receives a handle for the accessors below. */
int cuacd_decompose(void* d, const cuacd_mesh* meshes, int n, int batched, void** result);
int cuacd_result_meshes(const void* result);
int cuacd_result_parts(const void* result, int mesh);
int cuacd_result_part(const void* result, int mesh, int part, cuacd_part_view* out);
int cuacd_result_stats(const void* result, int mesh, cuacd_decompose_stats* out);
void cuacd_result_free(void* result);

/* ---- the merge pass on its own (src/merge.ts:170-303) ------------------- */

/* A part handed to the merge pass (Part, part.ts:9-22): its mesh, its hull
 * (vertices and outward triangles), volumes, the Hausdorff distance (NaN when
 * unknown), the seam planes of earlier merges (4 doubles each) and how many
 * input parts it already holds. */
typedef struct {
  cuacd_mesh mesh;
  cuacd_mesh hull;
  double meshVol;
  double hullVol;
  double hausdorff;
  const double* seams;
  uint32_t nSeams;
  int32_t merged;
} cuacd_part_in;

/* MergeOptions (merge.ts:25-42) with DEFAULT_MERGE_OPTIONS (merge.ts:44-52);
 * hulls and Hausdorff distances always run on the GPU. */
typedef struct {
  float threshold;
  int32_t maxRounds;
  double planeTol;
  double hullEps; /* epsilon of the merged hulls' cleanup (cleanHullFaces) */
  int32_t verbose;
  int32_t reserved;
} cuacd_merge_opts;

/* MergeStats (merge.ts:54-66). hullFallbacks counts merged hulls the GPU
 * could not build (the pair then stays unmerged). */
typedef struct {
  int32_t rounds;
  int32_t merges;
  int32_t pairsHulled;
  int32_t pairsHausdorff;
  int32_t hullFallbacks;
  int32_t reserved;
  double hullMs, hausdorffMs, totalMs;
} cuacd_merge_stats;

void cuacd_merge_opts_default(cuacd_merge_opts* o);
/* mergeHulls(tree, parts, opts) (merge.ts:170-303) on the decomposer's GPU
 * tree: rounds of cheap rejections, merged hulls of the surviving pairs,
 * Hausdorff distances of the seam-filtered unions, greedy min-cost matching.
 * On success *result receives a one-mesh result handle (cuacd_result_parts /
 * cuacd_result_part with mesh 0) holding the merged part list, and *stats the
 * pass's statistics. */
int cuacd_merge_hulls(void* decomposer, const cuacd_part_in* parts, int n, const cuacd_merge_opts* o, void** result,
                      cuacd_merge_stats* stats);
/* seamPlane(a, b, tol) (merge.ts:114-141): writes the plane (4 doubles) and
 * returns 1, or returns 0 when no separating hull face carries mesh area. */
int cuacd_seam_plane(const cuacd_part_in* a, const cuacd_part_in* b, double tol, double* out4);
/* filteredConcat(a, b, planes, tol) (merge.ts:144-157): the concatenation's
 * vertices are a's then b's; writes the kept triangles (over the
 * concatenation, at most cap of them) and returns their count. */
int cuacd_filtered_concat(const cuacd_mesh* a, const cuacd_mesh* b, const double* planes, int nPlanes, double tol,
                          uint32_t* outTris, int cap);

/* Serving (no counterpart in the reference, whose decompose serves one mesh
 * per call): continuous batching of decompositions under a device-memory
 * budget. admitBytes = device bytes the server may hold (0: 80 % of the
 * device's memory); maxActive = decompositions running at once (slots; 0 =
 * no bound besides memory). Requests queue in arrival order (at most maxQueue of them
 * wait, 0 = no bound; a submission to a full queue returns CUACD_E_BUSY and
 * counts as rejected) and are admitted while a slot is free and the server's trees, with their
 * vertex and triangle pools grown to the working sets of every admitted
 * request, fit in the budget (one request is always admitted when none runs;
 * a tree with no running request gives its memory back when the next request
 * would not fit beside it). A request's working set is the pool space of one
 * lookahead run with its mesh (nv vertices, nt triangles) as the seed: level
 * l has J_l jobs (J_0 = width + planeSlots, J_l+1 = width2 J_l), each job's
 * children hold up to 2.5 nv + 64 vertices, the children of every level but
 * the last 1.5 nt + 64 triangles and 16 sqrt(nt) + 64 open edges, and a
 * level's plan scratch is 2 words per parent vertex per job; 64 bytes per
 * input byte are added for the buffers of the cut, concave-plane and
 * Hausdorff passes, and a tree counts its hull slabs at hullBudgetBytes plus
 * 64 MB for the merge pass's hull and Hausdorff batches.
 * Before each step every tree's pools grow to its running requests' working
 * sets. A mesh whose working set alone exceeds the budget is
 * refused with CUACD_E_CAPACITY at submission. Each cuacd_server_step runs
 * one iteration of every admitted decomposition together, one tree launch per
 * threshold, and finishes (merge pass included) the decompositions with
 * nothing left to cut; a request submitted between steps joins at the next
 * one. A decomposition's parts are the same as cuacd_decompose gives it.
 * threshold <= 0 takes the options' threshold; other values get a tree of
 * their own (minEdgeDist follows the threshold). cuacd_server_take returns
 * CUACD_OK with a one-mesh result handle (cuacd_result_* accessors; stats
 * totalMs = time from submission to completion) once the request finished,
 * 1 while it is queued or running, or the request's error. */
typedef struct {
  uint64_t budgetBytes;     /* the device budget */
  uint64_t deviceBytes;     /* device bytes the server's trees hold now */
  uint64_t peakDeviceBytes; /* the most they held at any step */
  uint64_t workingSetBytes; /* working sets of the running requests */
  uint64_t projectedBytes;  /* what admission compares with the budget: the
                               trees with their pools grown to the running
                               requests' working sets, plus allowances for
                               their hull slabs and cut / concave-plane /
                               Hausdorff buffers (at least the bytes held) */
  uint64_t admitted;        /* requests admitted so far */
  uint64_t rejected;        /* submissions refused with a full queue */
  int32_t queued;           /* requests waiting */
  int32_t active;           /* requests running */
} cuacd_server_state;
void* cuacd_server_create(const cuacd_decompose_opts* o, uint64_t admitBytes, int32_t maxActive, int32_t maxQueue,
                          int* err);
void cuacd_server_destroy(void* server);
int cuacd_server_submit(void* server, const cuacd_mesh* mesh, float threshold, uint64_t* ticket);
int cuacd_server_step(void* server, int* completed);
int cuacd_server_pending(const void* server);
int cuacd_server_take(void* server, uint64_t ticket, void** result);
int cuacd_server_stats(const void* server, cuacd_server_state* out);

/* planeCut with caps (src/cpu/cut.ts:33-315) on the host, for callers that
 * apply a cut themselves. plane = a, b, c, d (a x + b y + c z + d = 0). On
 * success the two halves are returned in a handle read with
 * cuacd_cut_half (0 = positive side, 1 = negative side). Returns
 * CUACD_E_INVALID with the reference's reason when the plane does not split
 * the mesh or a boundary loop cannot be closed. */
int cuacd_plane_cut(const cuacd_mesh* mesh, const double* plane, void** halves);
int cuacd_cut_half(const void* halves, int side, const float** verts, uint32_t* nv, const uint32_t** tris,
                   uint32_t* nt);
void cuacd_cut_free(void* halves);

/* concaveEdgePlanes (src/cpu/concave.ts:25-92): writes up to cap planes (4
 * floats each) and returns their count (or a negative error). */
int cuacd_concave_planes(const cuacd_mesh* mesh, int nConcaveEdges, double concaveEps, double concaveThreshold,
                         uint32_t seed, float* out, int cap);

/* The reference's CPU hull, qh_compute (wasm/qh.cpp:16-25 over
 * wasm/quickhull/QuickHull.cpp): double-precision quickhull of n points,
 * eps relative to the largest extreme coordinate. Writes the hull vertices
 * (3 doubles each, at most vCap) and triangles (3 indices each, at most
 * tCap, counter-clockwise seen from outside); returns the triangle count and
 * sets *nvOut, or CUACD_E_CAPACITY when an output does not fit. */
int cuacd_quickhull(const double* pts, int n, double eps, double* vOut, int vCap, uint32_t* tOut, int tCap,
                    int* nvOut);

/* cleanHullFaces (src/cpu/hull.ts:87-155): the faces of an exact grid hull
 * (nt triangles indexing mesh->verts; mesh->tris is not read) rebuilt for
 * output from their own vertices; returns the count of triangles written to
 * out (at most cap) or an error. The decomposer applies it to every output
 * hull with eps = max(2e-5, 64 * 6e-8 * maxAbs / extent) of the input. */
int cuacd_clean_hull_faces(const cuacd_mesh* mesh, const uint32_t* tris, uint32_t nt, double eps, uint32_t* out,
                           int cap);

/* Message of the last failure on the calling thread. */
const char* cuacd_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* CUACD_H */
