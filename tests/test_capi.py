"""C ABI checks that need no GPU: the library builds for sm_103a, loads, and
exports exactly the entry points include/arborx_gb300.h declares."""

import ctypes
import os
import re

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "arborx_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^ABX_API [^;]*?\b(abx_\w+)\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def libpath():
    from arborx_gb300 import build as b

    return b.build()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "abx_bvh_create" in names and "abx_bvh_query_nearest" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(libpath):
    from arborx_gb300 import _lib

    assert set(_lib.SIGNATURES) == set(declared_functions())
    L = _lib.load(libpath)
    # pure host calls, no device work
    assert L.abx_status_string(0) == b"ABX_SUCCESS"
    assert L.abx_status_string(4) == b"ABX_ERROR_BUFFER_OVERFLOW"
    assert L.abx_version().decode().count(".") == 2



def test_forest_arguments_are_checked_on_the_host():
    """Bad forest offsets are refused before any device work (no GPU needed)."""
    import ctypes

    import numpy as np

    from arborx_gb300 import _lib

    L = _lib.load()
    h = ctypes.c_void_p()
    for offsets in ([1, 5], [0, 6, 5], [0, -1]):
        o = np.asarray(offsets, np.int64)
        st = L.abx_forest_create(None, 0, ctypes.c_void_p(16), o.ctypes.data, o.size - 1, ctypes.byref(h))
        assert st == 1 and not h.value  # ABX_ERROR_INVALID_ARGUMENT
    o = np.asarray([0], np.int64)
    assert L.abx_forest_create(None, 0, None, o.ctypes.data, 0, ctypes.byref(h)) == 1
    assert L.abx_forest_create(None, 2, None, o.ctypes.data, 0, ctypes.byref(h)) == 1
    assert L.abx_forest_num_trees(None) == 0 and L.abx_forest_size(None, 0) == 0


def test_tree_file_errors_are_reported_on_the_host(tmp_path):
    """abx_bvh_load refuses a missing file and a file that is not a tree
    before any device work."""
    import ctypes

    from arborx_gb300 import _lib

    L = _lib.load()
    h = ctypes.c_void_p()
    missing = str(tmp_path / "missing.abx").encode()
    assert L.abx_bvh_load(None, missing, ctypes.byref(h)) == 1
    assert not h.value
    bad = tmp_path / "bad.abx"
    bad.write_bytes(b"ABXBVH01" + b"\0" * 8)  # header cut short
    assert L.abx_bvh_load(None, str(bad).encode(), ctypes.byref(h)) == 1
    bad.write_bytes(b"NOTATREE" + b"\0" * 64)
    assert L.abx_bvh_load(None, str(bad).encode(), ctypes.byref(h)) == 1
    assert not h.value
    assert L.abx_bvh_save(None, missing) == 1


def test_tree_file_with_bad_references_is_refused(tmp_path):
    """A tree file whose node references leave the tree (a corrupted or
    hostile file) is refused on the host before anything reaches the device."""
    import ctypes
    import struct

    import numpy as np

    from arborx_gb300 import _lib

    L = _lib.load()
    n = 3

    def write(nodes, leaves):
        hdr = b"ABXBVH01" + struct.pack("<iiq6f", 0, 0, n, 0, 0, 0, 1, 1, 1)
        body = nodes.tobytes() + leaves.tobytes()
        path = tmp_path / "t.abx"
        path.write_bytes(hdr + body)
        return str(path).encode()

    def node(lref, rref, lc, rc):
        a = np.zeros(16, np.int32)
        a[12:16] = [lref, rref, lc, rc]
        return a

    leaves = np.zeros((n, 4), np.float32)
    leaves[:, 3] = np.arange(n, dtype=np.int32).view(np.float32)
    h = ctypes.c_void_p()
    bad_sets = [
        # internal reference past the node array
        np.concatenate([node(5, ~2, 2, 1), node(~0, ~1, 1, 1)]),
        # leaf value past the leaves
        np.concatenate([node(1, ~7, 2, 1), node(~0, ~1, 1, 1)]),
        # bucket count running past the leaves
        np.concatenate([node(1, ~2, 30, 1), node(~0, ~1, 1, 1)]),
    ]
    for nodes in bad_sets:
        assert L.abx_bvh_load(None, write(nodes, leaves), ctypes.byref(h)) == 1
        assert not h.value
    bad_leaves = leaves.copy()
    bad_leaves[1, 3] = np.array([9], np.int32).view(np.float32)[0]
    good_nodes = np.concatenate([node(1, ~2, 2, 1), node(~0, ~1, 1, 1)])
    assert L.abx_bvh_load(None, write(good_nodes, bad_leaves), ctypes.byref(h)) == 1


def test_new_entry_points_check_arguments_on_the_host():
    """Argument checks of the KDOP, gather and host-buffer entry points fail
    before any device work."""
    import ctypes

    from arborx_gb300 import _lib

    L = _lib.load()
    buf = (ctypes.c_float * 64)()
    # KDOP conversion: source must be points or boxes, target a KDOP kind
    assert L.abx_kdop_from_geometry(None, _lib.SPHERE, buf, 1, _lib.KDOP14, buf) == 1
    assert L.abx_kdop_from_geometry(None, _lib.BOX, buf, 1, _lib.BOX, buf) == 1
    assert L.abx_kdop_from_geometry(None, _lib.POINT, None, 1, _lib.KDOP18, buf) == 1
    # row gather: whole 32-bit words, non-null arrays
    assert L.abx_gather_rows(None, buf, 4, 6, buf, 1, buf) == 1
    assert L.abx_gather_rows(None, buf, 4, 0, buf, 1, buf) == 1
    assert L.abx_gather_rows(None, None, 4, 16, buf, 1, buf) == 1
    # KDOP bounds and host-buffer queries need a tree
    assert L.abx_bvh_kdop_bounds(None, buf) == 1
    pol = _lib.TraversalPolicyC(0, 1)
    assert L.abx_bvh_query_nearest_host(None, None, buf, 1, 1, pol, 0, buf, buf, None) == 1
