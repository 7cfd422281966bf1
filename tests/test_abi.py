"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/cuacd.h declares (no device calls: this runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT, pkg

HEADER = os.path.join(ROOT, "include", "cuacd.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cuacd_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build = pkg("build")
    path = build.build()
    assert os.path.exists(path)
    return C.CDLL(path)


def test_header_declares_the_reference_surface():
    syms = declared_symbols()
    for s in ("cuacd_tree_create", "cuacd_tree_destroy", "cuacd_tree_run", "cuacd_tree_hausdorff",
              "cuacd_tree_hull_meshes", "cuacd_tree_hulls_with_hausdorff", "cuacd_plane_slots",
              "cuacd_tree_read_part_geometry", "cuacd_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_config_default_matches_reference(lib):
    A = pkg("_abi")
    c = A.TreeConfig()
    lib.cuacd_tree_config_default(C.byref(c))
    assert (c.width, c.width2, c.depth, c.nConcaveEdges) == (60, 3, 2, 32)
    assert abs(c.minEdgeDist - 0.0125) < 1e-9
    assert c.vertexCap == 64 << 20 and c.triCap == 64 << 20 and c.edgeCap == 1 << 20
    assert c.scratchWords == 48 << 20 and c.hullBudgetBytes == 256 << 20 and c.hullMaxVerts == 4096
    assert lib.cuacd_vis_max() == 2048


def test_struct_layouts():
    A = pkg("_abi")
    assert C.sizeof(A.TreeConfig) == 80
    assert C.sizeof(A.MeshRef) == 24
    assert C.sizeof(A.RunOpts) == 32
    assert C.sizeof(A.SeedResult) == 32
    assert C.sizeof(A.RunStats) == 64
