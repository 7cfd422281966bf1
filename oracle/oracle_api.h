// oracle_api.h — C structs of the CPU oracle's ctypes interface.
//
// TEST INFRASTRUCTURE ONLY. The field lists match the engine's public
// structs in include/cuacd.h so one set of Python wrappers drives both.
#pragma once
#include <cstdint>

extern "C" {

typedef struct {
  int32_t width, width2, depth, nConcaveEdges;
  float minEdgeDist;
  int32_t hullMaxVerts;
  uint64_t vertexCap, triCap, edgeCap, scratchWords, hullBudgetBytes;
  int32_t pruneLastLevel;
  int32_t reserved;
} orc_config;

typedef struct {
  const float* verts;
  const uint32_t* tris;
  uint32_t nv, nt;
} orc_mesh;

typedef struct {
  int32_t depth;        // <= 0: configured depth
  int32_t width;        // < 0: configured width
  int32_t nEdgeCuts;    // < 0: all plane slots
  int32_t refineRounds;
  int32_t refineProbes;
  int32_t reserved;
  const float* refineSpacing;  // per seed
} orc_run_opts;

typedef struct {
  int32_t bestCut;
  float bestCost;
  float plane[4];
  int32_t valid;
  int32_t reserved;
} orc_seed;

typedef struct {
  uint32_t overflow, hullFail, hullFailCount, npOverflow, pruned;
  uint32_t nLevels;
  uint32_t jobsPerLevel[4];
  uint64_t validJobs;
  uint32_t hullSlabWords, hullChunkSize;
  float gpuMs;
  uint32_t reserved;
} orc_stats;

}
