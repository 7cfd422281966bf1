"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/cuacd.h declares (no device calls: this runs without a GPU)."""
import ctypes as C
import os
import re
import shutil
import subprocess

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


# The byte offsets the Deno FFI shim in INTEGRATION.md writes by hand
# (Deno.UnsafePointer / DataView see C layout): struct, field -> offset, and
# struct sizes, checked against the header compiled by a C compiler.
SHIM_OFFSETS = {
    ("cuacd_tree_config", "width"): 0, ("cuacd_tree_config", "width2"): 4, ("cuacd_tree_config", "depth"): 8,
    ("cuacd_tree_config", "nConcaveEdges"): 12, ("cuacd_tree_config", "minEdgeDist"): 16,
    ("cuacd_tree_config", "hullMaxVerts"): 20, ("cuacd_tree_config", "vertexCap"): 24,
    ("cuacd_tree_config", "triCap"): 32, ("cuacd_tree_config", "edgeCap"): 40,
    ("cuacd_tree_config", "scratchWords"): 48, ("cuacd_tree_config", "hullBudgetBytes"): 56,
    ("cuacd_tree_config", "pruneLastLevel"): 64, ("cuacd_tree_config", "autotune"): 76,
    ("cuacd_mesh", "verts"): 0, ("cuacd_mesh", "tris"): 8, ("cuacd_mesh", "nv"): 16, ("cuacd_mesh", "nt"): 20,
    ("cuacd_run_opts", "depth"): 0, ("cuacd_run_opts", "width"): 4, ("cuacd_run_opts", "nEdgeCuts"): 8,
    ("cuacd_run_opts", "refineRounds"): 12, ("cuacd_run_opts", "refineProbes"): 16,
    ("cuacd_run_opts", "refineSpacing"): 24,
    ("cuacd_decompose_opts", "threshold"): 0, ("cuacd_decompose_opts", "maxIters"): 4,
    ("cuacd_decompose_opts", "width"): 8, ("cuacd_decompose_opts", "depth"): 16,
    ("cuacd_decompose_opts", "mergeHulls"): 60, ("cuacd_decompose_opts", "tree"): 88,
}
SHIM_SIZES = {"cuacd_tree_config": 80, "cuacd_mesh": 24, "cuacd_run_opts": 32, "cuacd_decompose_opts": 168,
              "cuacd_part_view": 96, "cuacd_seed_result": 32}


def test_shim_offsets_match_the_header_in_c(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "cuacd.h"', "int main(void) {"]
    for (st, f) in SHIM_OFFSETS:
        lines.append(f'  printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    for st in SHIM_SIZES:
        lines.append(f'  printf("{st} %zu\\n", sizeof({st}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "offsets.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "offsets"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                                text=True).stdout.splitlines())
    for (st, f), off in SHIM_OFFSETS.items():
        assert int(got[f"{st}.{f}"]) == off, (st, f, got[f"{st}.{f}"], off)
    for st, size in SHIM_SIZES.items():
        assert int(got[st]) == size, (st, got[st], size)
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    assert "cuacd_decompose_opts is 168 bytes" in doc and "new Uint8Array(168)" in doc
