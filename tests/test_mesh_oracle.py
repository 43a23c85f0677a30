"""The mesh consumers' oracle against known answers, and the argument checks of
the diso_mesh_* entry points (no GPU)."""
import ctypes
import math
import struct

import numpy as np
import pytest

from oracle import mesh as M


def test_obj_fixed_point_rounding_and_special_values():
    # 1/512 * 1e8 and 3/512 * 1e8 are exact ties (195312.5, 585937.5): to even
    v = np.array([[0.0, 1 / 512, -0.0], [3 / 512, 1e-9, -1e-9], [math.nan, math.inf, -math.inf]], dtype=np.float64)
    f = np.array([[0, 1, 2]])
    assert M.obj_text(v, f) == (b"v 0.00000000 0.00195312 -0.00000000\n"
                                b"v 0.00585938 0.00000000 -0.00000000\n"
                                b"v nan inf -inf\n"
                                b"f 1 2 3\n")
    n = np.eye(3)
    assert M.obj_text(v[:1], np.array([[0, 0, 0, 0]]), n[:1]).endswith(b"vn 1.00000000 0.00000000 0.00000000\n"
                                                                      b"f 1//1 1//1 1//1 1//1\n")


def test_normals_of_a_square_and_its_triangles():
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], dtype=np.float64)
    quad = M.vertex_normals(v, np.array([[0, 1, 2, 3]]))
    tris = M.vertex_normals(v, np.array([[0, 1, 2], [0, 2, 3]]))
    assert np.allclose(quad, [[0, 0, 1]] * 4) and np.allclose(tris, [[0, 0, 1]] * 4)
    assert np.all(M.vertex_normals(np.zeros((2, 3)), np.zeros((0, 3), dtype=np.int64)) == 0)


def test_weld_keeps_the_lowest_index_and_drops_collapsed_faces():
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 0], [1, 1e-4, 0], [0, 1, 0]], dtype=np.float32)
    f = np.array([[0, 1, 4], [2, 3, 4], [0, 2, 4]])
    wv, wf = M.weld(v, f)
    assert wv.tolist() == v[[0, 1, 3, 4]].tolist() and wf.tolist() == [[0, 1, 3], [0, 2, 3]]
    wv, wf = M.weld(v, f, tol=1e-2)  # 1 and 1 + 1e-4 round together
    assert wv.tolist() == v[[0, 1, 4]].tolist() and wf.tolist() == [[0, 1, 2], [0, 1, 2]]


def test_ply_layout():
    v = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8]], dtype=np.float32)
    b = M.ply_bytes(v, np.array([[0, 1, 2]]))
    head, body = b.split(b"end_header\n")
    assert b"element vertex 3\nproperty float x" in head and b"property list uchar int vertex_indices" in head
    assert body[:36] == v.tobytes() and body[36:] == struct.pack("<B3i", 3, 0, 1, 2)


@pytest.fixture(scope="module")
def lib():
    from diso_gb300.build import build

    build()
    from diso_gb300 import _native

    return _native.lib()


def test_mesh_entry_points_check_their_arguments(lib):
    # sizes of the PLY body, and status codes for bad arguments, without a GPU
    assert lib.diso_mesh_ply_bytes(0, 10, 4, 3, 0) == 10 * 12 + 4 * 13
    assert lib.diso_mesh_ply_bytes(1, 10, 4, 4, 1) == 10 * 48 + 4 * 17
    assert lib.diso_mesh_ply_bytes(0, 10, 4, 5, 0) == -1
    n = ctypes.c_int64(0)
    assert lib.diso_mesh_normals(None, None, 0, None, 0, 3, None, None) == 1
    assert lib.diso_mesh_obj(None, None, None, 0, None, 0, 3, None, 0, ctypes.byref(n), None) == 1
    assert lib.diso_mesh_ply(None, None, None, 0, None, 0, 3, None, None) == 1
    assert lib.diso_mesh_weld(None, None, 0, None, 0, 3, 0.0, None, None, ctypes.byref(n), ctypes.byref(n),
                              None) == 1
