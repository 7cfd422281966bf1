// tree_internal.h — library-internal entry points of the tree handle.
#pragma once

#include "../../include/cuacd.h"

namespace cuacd {

// Host copies of the meshes of the handle's next cuacd_tree_hull_meshes /
// cuacd_tree_hulls_with_hausdorff call (same order): that call may then
// pass the meshes in device memory; their Hausdorff sample counts follow
// the host copies' areas. The copies serve that one call.
int tree_set_host_twins(void* tree, const cuacd_mesh* twins, int n);

}  // namespace cuacd
