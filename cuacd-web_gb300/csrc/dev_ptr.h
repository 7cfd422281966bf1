// dev_ptr.h — whether a mesh buffer lives in device memory. The entry points
// that take meshes accept device buffers of the handle's device as well as
// host buffers: a device mesh is copied on the device (no host round trip);
// a host mesh is staged and uploaded.
#pragma once

#include <cuda_runtime.h>

namespace cuacd {

// device or managed allocations are device memory; host memory, registered
// or not, is not
inline bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace cuacd
