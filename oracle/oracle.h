// oracle.h — CPU oracle for the cuacd GB300 engine.
//
// TEST INFRASTRUCTURE ONLY. These are plain C++ restatements of the
// reference's GPU kernels (src/gpu/shaders.ts, src/gpu/hausdorff_shader.ts)
// and CPU helpers (src/cpu/*.ts, src/mesh.ts, src/part.ts). Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load them, and only
// as the checker; the engine never does.
#pragma once
#include <cstdint>
#include <vector>

#include "oracle_geom.h"

#define ORC_VIS_MAX 2048u

namespace orc {

float rv_cost(float meshVol, float hullVol);

struct HullOpts {
  int hullStage = 0;       // 1 = seeds only, 2/3 = no full-point insertion (tree.ts:382)
  bool prune = false;      // last-level branch and bound (shaders.ts:1300-1331)
  float prunePartial = 0;  // partial path sum of the parent item
  float pruneUb = 0;       // best completed-path upper bound of the seed
  float meshVol = 0;
};

struct HullResult {
  float hullVol = 0.0f;
  uint32_t status = 0;  // 1 visible-set overflow, 2 face slots exhausted, 3 slab too small
  bool pruned = false;
  bool assigned = false;  // reached the full assignment pass (the kernel records ncand there)
  uint32_t nIns = 0, ncand = 0;
  std::vector<uint32_t> faces;  // alive faces in slot order, (a, b, c) per face
};

HullResult hull_points(const f3* pts, uint32_t nv, uint32_t slabWords, const HullOpts& o);

}  // namespace orc
