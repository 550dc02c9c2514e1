"""exporter::write3D's mesh files (src/exporter.cpp:70-167) from the
library's host writers against the files the reference itself wrote for
the same mesh (tests/golden/export_n16.npz, on the mesh of
tests/golden/mesh_n16.npz; both made by tests/golden/make_golden.py).
Host code; no GPU needed."""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


def test_obj_and_sunflow_files_are_the_references(gpu, tmp_path):
    ex = np.load(os.path.join(HERE, "golden", "export_n16.npz"))
    mesh = np.load(os.path.join(HERE, "golden", "mesh_n16.npz"))
    v, nr, f = mesh["vertices"], mesh["normals"], mesh["faces"]
    assert hashlib.sha256(v.tobytes() + nr.tobytes() + f.astype(np.int32).tobytes()).hexdigest() \
        == str(ex["mesh_sha256"])
    obj, sc = str(tmp_path / "m.obj"), str(tmp_path / "m.sc")
    gpu.write_mesh_files(obj, sc, v, nr, f, float(ex["wall_thick"]))
    for tag, path in (("obj", obj), ("sunflow", sc)):
        raw = open(path, "rb").read()
        head = bytes(ex[f"{tag}_head"])
        assert raw[:len(head)] == head, tag
        assert len(raw) == int(ex[f"{tag}_bytes"]), tag
        assert hashlib.sha256(raw).hexdigest() == str(ex[f"{tag}_sha256"]), tag


def test_empty_mesh(gpu, tmp_path):
    obj, sc = str(tmp_path / "e.obj"), str(tmp_path / "e.sc")
    gpu.write_mesh_files(obj, sc, np.zeros(0), np.zeros(0), np.zeros(0, np.int32), 1 / 32)
    assert open(obj, "rb").read() == b""
    assert open(sc, "rb").read() == (b"include template.sc\n\nobject { \n shader Liquid \n type "
                                     b"mesh \n name polySurfac \n 0 0 \n}\n")
