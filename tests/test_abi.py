"""CPU tests of the C-ABI boundary: the library loads, exports every function
include/lrx.h declares, and its struct layouts match the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

from luxcore_gb300 import build, lrx
from luxcore_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "lrx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lrx_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return lrx.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert names, "no declarations parsed"
    assert sorted(lrx.EXPORTED) == names
    for n in names:
        assert hasattr(lib, n), n


def test_abi_version_and_error_string(lib):
    assert lib.lrx_abi_version() == 4
    assert isinstance(lib.lrx_last_error(), bytes)


def test_struct_layouts():
    assert W.RAY_DTYPE.itemsize == 48 and W.HIT_DTYPE.itemsize == 20
    assert W.RAY_DTYPE.fields["mint"][1] == 24 and W.RAY_DTYPE.fields["flags"][1] == 36
    assert ctypes.sizeof(lrx.MeshDesc) == 24
    assert ctypes.sizeof(lrx.ObjectDesc) == 136
    assert ctypes.sizeof(lrx.BuildOpts) == 20  # ABI 4: + node_layout
    assert ctypes.sizeof(lrx.SceneInfo) == 64
    assert ctypes.sizeof(lrx.TraceConfig) == 32  # ABI 3: + max_visits, deadline_us
    assert ctypes.sizeof(lrx.ServerOpts) == 40  # ABI 4: + max_rays_per_launch


def test_variant_constants_match_the_header():
    src = open(os.path.join(ROOT, "include", "lrx.h")).read()
    defs = dict(re.findall(r"#define (LRX_VARIANT_[A-Z0-9_]+) (0x[0-9a-fA-F]+)u", src))
    assert defs, "no variant defines parsed"
    for name, val in defs.items():
        assert getattr(lrx, name) == int(val, 16), name
    nodes = dict(re.findall(r"#define (LRX_NODES_[A-Z0-9_]+) ([0-9]+)u", src))
    assert set(nodes) == {"LRX_NODES_WIDE8", "LRX_NODES_COMPACT4"}
    for name, val in nodes.items():
        assert getattr(lrx, name) == int(val), name


def test_null_arguments_are_rejected_without_a_device(lib):
    # argument checks run before any CUDA call
    h = ctypes.c_void_p()
    assert lib.lrx_scene_create(None, 0, None, 0, None, None, None) == 1
    assert lib.lrx_trace(None, None, None, 10, 0, None) == 1
    assert lib.lrx_trace_batches(None, 3, None) == 1
    assert lib.lrx_trace_host_batches(None, 3, None) == 1
    assert lib.lrx_scene_create_motion(None, 0, None, 0, None, 2, None, None, ctypes.byref(h)) == 1
    assert lib.lrx_scene_destroy(None) == 0
    assert b"null" in lib.lrx_last_error()
    del h


def test_bad_node_width_is_rejected_without_a_device(lib):
    # build options are checked before any CUDA call too
    h = ctypes.c_void_p()
    for w in (1, 3, 9, 64):
        opts = lrx.BuildOpts(ctypes.sizeof(lrx.BuildOpts), 3, 2, w)
        assert lib.lrx_scene_create(None, 0, None, 0, ctypes.byref(opts), None, ctypes.byref(h)) == 1
        assert b"node_width" in lib.lrx_last_error()
    # 64-byte records take 4-wide trees; an unknown record is refused
    for w, layout in ((8, lrx.LRX_NODES_COMPACT4), (5, lrx.LRX_NODES_COMPACT4), (4, 2)):
        opts = lrx.BuildOpts(ctypes.sizeof(lrx.BuildOpts), 3, 2, w, layout)
        assert lib.lrx_scene_create(None, 0, None, 0, ctypes.byref(opts), None, ctypes.byref(h)) == 1
        assert b"node_layout" in lib.lrx_last_error()
    # a caller of ABI 1-3 passes the 16-byte struct: its options are read,
    # node_layout is not (a bad width is still refused)
    opts = lrx.BuildOpts(16, 3, 2, 9, lrx.LRX_NODES_COMPACT4)
    assert lib.lrx_scene_create(None, 0, None, 0, ctypes.byref(opts), None, ctypes.byref(h)) == 1
    assert b"node_width" in lib.lrx_last_error()


def test_package_has_no_cpu_fallback():
    # the product path must not import the oracle
    for dirpath, _, files in os.walk(os.path.join(ROOT, "luxcore_gb300")):
        for f in files:
            if f.endswith(".py"):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in re.sub(r"#.*", "", src).replace('"""', "").split("import")[0] or \
                    "from oracle" not in src and "import oracle" not in src, f
