"""The LuxRays binding as code: luxcore_gb300/luxrays/gb300accel.{h,cpp} --
GB300Accel (an Accelerator) and GB300Kernel (a HardwareIntersectionKernel)
over liblrx.so -- compiles against the reference's own headers
(include/luxrays/core/accelerator.h, hardwareintersectiondevice.h,
devices/cudadevice.h), with the third-party headers those include (Boost,
cuew, OptiX) replaced by the declaration-only stand-ins in
tests/cpp/refstubs/.  Also checked: the PATHOCL accelerator check
(src/slg/engines/pathoclbase/pathoclbaseoclthreadkernels.cpp:250-262) is
the switch the maintainer patches, and it does not yet accept GB300.
Skipped where the LuxCore source tree is absent (a checkout of this
repository alone)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_tree():
    r = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), "--tree"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else None


def _cuda_include():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "include", "cuda.h")):
            return os.path.join(c, "include")
    return None


@pytest.fixture(scope="module")
def tree():
    t = _reference_tree()
    if t is None:
        pytest.skip("LuxCore source tree not present")
    if _cuda_include() is None or shutil.which("g++") is None:
        pytest.skip("no CUDA headers or g++")
    return t


def test_binding_compiles_against_the_reference_headers(tree, tmp_path):
    obj = tmp_path / "gb300accel.o"
    cmd = ["g++", "-std=c++17", "-Wall", "-Wno-unused-parameter", "-c",
           os.path.join(ROOT, "luxcore_gb300", "luxrays", "gb300accel.cpp"), "-o", str(obj),
           "-I", os.path.join(ROOT, "tests", "cpp", "refstubs"), "-I", os.path.join(tree, "include"),
           "-I", os.path.join(ROOT, "include"), "-I", _cuda_include()]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    syms = subprocess.run(["nm", "-C", str(obj)], capture_output=True, text=True).stdout
    # the virtual interface is defined here, and it calls the C ABI
    for name in ("luxrays::GB300Accel::Init", "luxrays::GB300Accel::Update",
                 "luxrays::GB300Accel::NewHardwareIntersectionKernel", "luxrays::GB300Kernel::EnqueueTraceRayBuffer",
                 "vtable for luxrays::GB300Accel", "vtable for luxrays::GB300Kernel"):
        assert name in syms, name
    for c_entry in ("lrx_scene_create", "lrx_scene_create_motion", "lrx_scene_update_instances", "lrx_trace",
                    "lrx_scene_destroy", "lrx_last_error"):
        assert f"U {c_entry}" in syms, c_entry


def test_the_pathocl_accelerator_check_is_the_switch_to_patch(tree):
    src = open(os.path.join(tree, "src", "slg", "engines", "pathoclbase", "pathoclbaseoclthreadkernels.cpp")).read()
    i = src.index("switch (intersectionDevice->GetAccelerator()->GetType())")
    block = src[i:src.index("}", i)]
    for known in ("case ACCEL_BVH:", "case ACCEL_MBVH:", "case ACCEL_OPTIX:", "default:"):
        assert known in block
    assert "ACCEL_GB300" not in block   # the maintainer adds `case ACCEL_GB300: break;` here
