// concave_engine.h — host interface of the GPU concave-edge planes
// (concave_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cuacd.h"

namespace cuacd {
namespace conc {

struct Engine;
Engine* engine_create();
void engine_destroy(Engine* e);
// device bytes the engine's buffers hold (they grow with the largest batch)
size_t engine_device_bytes(const Engine* e);
// concaveEdgePlanes of every mesh on `stream`: mesh k's planes (at most
// 4 * nConcaveEdges, 4 floats each) go to out + 16 * nConcaveEdges * k and
// their count to counts[k]; seeds[k] is its reservoir seed.
int engine_run(Engine* e, cudaStream_t stream, const cuacd_mesh* meshes, int nMeshes, int nConcaveEdges, double eps,
               double thr, const uint32_t* seeds, float* out, int32_t* counts, float* gpuMs);

}  // namespace conc
}  // namespace cuacd
