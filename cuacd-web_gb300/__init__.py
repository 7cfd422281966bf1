"""cuacd GB300 engine: the lookahead-tree hot path of cuacd-web on sm_103a.

The engine is the C-ABI library ``libcuacd.so`` (include/cuacd.h) built from
``csrc/``. This package mirrors the reference's GpuTree interface
(src/gpu/tree.ts) over that library; the CUDA path is the only path, and
constructing a tree fails loudly when the library is missing.
"""
from .mesh import Mesh, make_box, merge_meshes, unit_cube, l_shape, volume, signed_volume, is_closed, normalize  # noqa: F401
from .part import K_RV, rv_cost, part_cost  # noqa: F401
from ._abi import DEFAULT_TREE_CONFIG  # noqa: F401


def __getattr__(name):
    # the CUDA-backed classes load libcuacd.so on first use
    if name in ("GpuTree", "HD_MAX_PAIRS", "load_library", "library_path"):
        from . import tree

        return getattr(tree, name)
    raise AttributeError(name)
