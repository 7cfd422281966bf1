// cut_engine.h — host interface of the GPU capped plane cut (cut_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/cuacd.h"

namespace cuacd {
namespace cut {

// One cut: a mesh of the batch and its plane's frame (unit normal n, offset
// d, cap basis u, v; host::plane_frame computes them).
struct CutSpec {
  int32_t mesh;
  double n[3], d, u[3], v[3];
};

// The halves of a batch of cuts, in host memory. status[k] is 0 or
// the cut's failure (1 the plane does not split the mesh, 2 open boundary
// chain, 3 boundary chain dead end, 4 boundary chain cycle, 5 internal
// scratch bound exceeded). For cut k and side s (0 positive, 1 negative)
// the half's vertices start at float 3 * vOff[2k + s], its triangles at u32
// 3 * tOff[2k + s].
struct Halves {
  std::vector<int32_t> status;
  std::vector<uint64_t> vOff, tOff;
  std::vector<uint32_t> nv, nt;
  std::vector<double> vol;  // signed volume of each half (a fixed-order parallel sum)
  float* V = nullptr;     // into host
  uint32_t* T = nullptr;  // into host
  // the same halves on the device, in the engine's output buffers (same
  // offsets), valid until the engine's next batch
  const float* dV = nullptr;
  const uint32_t* dT = nullptr;
  float gpuMs = 0.0f;
  std::vector<uint32_t> host;  // every half's vertices, then every half's triangles
};

struct Engine;
Engine* engine_create();
void engine_destroy(Engine* e);
// device bytes the engine's buffers hold (they grow with the largest batch)
size_t engine_device_bytes(const Engine* e);
// Cuts meshes[cuts[k].mesh] by each plane on `stream`. Mesh indices must be
// in range. closed = the caller vouches that every mesh is closed (each
// directed edge has a reverse), as the decomposer's parts are: the pass that
// finds open input edges is skipped. Returns CUACD_OK or an error code.
int engine_run(Engine* e, cudaStream_t stream, const cuacd_mesh* meshes, int nMeshes, const CutSpec* cuts, int nCuts,
               bool closed, Halves* out);

}  // namespace cut
}  // namespace cuacd
