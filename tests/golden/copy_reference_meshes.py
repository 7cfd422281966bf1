"""Copies the reference's own test meshes into this folder as fixtures.

The reference ships three meshes its tests and README use: tests/data/49160.stl
(decompose.test.ts:52-63) and demo/models/{teapot,bunny}_vox64.stl.gz
(README.md:151-157). They are copied byte for byte, so the GPU tests can
decompose them on a machine without the reference tree.

    CUACD_REFERENCE_DIR=<reference checkout> python tests/golden/copy_reference_meshes.py
"""
import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = {"tests/data/49160.stl": "49160.stl",
         "demo/models/teapot_vox64.stl.gz": "teapot_vox64.stl.gz",
         "demo/models/bunny_vox64.stl.gz": "bunny_vox64.stl.gz"}


def main():
    ref = os.environ.get("CUACD_REFERENCE_DIR", "/root/reference")
    for src, dst in FILES.items():
        shutil.copyfile(os.path.join(ref, src), os.path.join(HERE, dst))
        print(dst, os.path.getsize(os.path.join(HERE, dst)))


if __name__ == "__main__":
    main()
