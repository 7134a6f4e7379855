"""The MEX shim (mesolf_gb300/mex/mex_lfm_convolution_vec.c) compiled against a fake MATLAB
runtime (tests/mex_fake/): the reference's argument validation and error id
(src/cuda/mex_lfm_convolution_vec.cu:296-347) on the CPU, and one valid call on the GPU
against the oracle (relative L2 1e-5)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import mesolf_ref as R

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INVALID = "parallel:gpu:mexGPUExample:InvalidInput"
SINGLE, DOUBLE = 7, 6


@pytest.fixture(scope="module")
def harness(tmp_path_factory, lib):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    out = str(tmp_path_factory.mktemp("mex") / "libmexfake.so")
    libdir = os.path.join(ROOT, "mesolf_gb300")
    subprocess.run(["gcc", "-std=c99", "-O1", "-Wall", "-shared", "-fPIC", "-o", out,
                    os.path.join(ROOT, "tests", "mex_fake", "fake_mex.c"),
                    os.path.join(ROOT, "mesolf_gb300", "mex", "mex_lfm_convolution_vec.c"),
                    "-I", os.path.join(ROOT, "tests", "mex_fake"), "-I", os.path.join(ROOT, "include"),
                    "-L", libdir, "-lmesolf_lf", "-Wl,-rpath," + libdir], check=True)
    h = ctypes.CDLL(out)
    h.harness_call.restype = ctypes.c_int
    return h


def call(h, arrays, out_n=1, shapes=None):
    """arrays: list of (numpy array, class id); shapes (optional) overrides the dimensions
    passed for each array (validation cases that must fail before any data is read).
    Returns (ok, output or (id, message))."""
    n = len(arrays)
    keep = [np.asfortranarray(a) for a, _ in arrays]
    shapes = shapes or [a.shape for a in keep]
    nds = (ctypes.c_int * n)(*[len(sh) for sh in shapes])
    dims = (ctypes.c_int64 * (8 * n))()
    for k, sh in enumerate(shapes):
        for d, s in enumerate(sh):
            dims[8 * k + d] = s
    cls = (ctypes.c_int * n)(*[c for _, c in arrays])
    datas = (ctypes.c_void_p * n)(*[a.ctypes.data for a in keep])
    out = np.zeros(out_n, np.float32)
    eid = ctypes.create_string_buffer(256)
    msg = ctypes.create_string_buffer(1024)
    rc = h.harness_call(n, nds, dims, cls, datas, out.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(out_n),
                        eid, msg)
    if rc:
        return False, (eid.value.decode(), msg.value.decode())
    return True, out


def f32(*shape):
    return np.random.default_rng(sum(shape)).random(shape).astype(np.float32)


@pytest.mark.parametrize("case", ["one_input", "three_inputs", "double_bitmap", "kernels_3d", "bitmap_4d",
                                  "double_kernels"])
def test_shape_and_class_validation(harness, case):
    bm, K = f32(20, 18, 2), f32(7, 7, 15, 15)
    args = {"one_input": [(bm, SINGLE)],
            "three_inputs": [(bm, SINGLE), (K, SINGLE), (bm, SINGLE)],
            "double_bitmap": [(bm.astype(np.float64), DOUBLE), (K, SINGLE)],
            "kernels_3d": [(bm, SINGLE), (K[:, :, :, 0], SINGLE)],
            "bitmap_4d": [(bm[:, :, :, None], SINGLE), (K, SINGLE)],
            "double_kernels": [(bm, SINGLE), (K.astype(np.float64), DOUBLE)]}[case]
    ok, res = call(harness, args)
    assert not ok
    assert res == (INVALID, "Invalid input to mex_lfm_convolution_vec()")


def test_kernel_width_limit_and_grid(harness):
    ok, (eid, msg) = call(harness, [(f32(20, 18), SINGLE), (f32(3, 3, 15, 15), SINGLE)],
                          shapes=[(20, 18), (343, 343, 15, 15)])
    assert not ok and eid == INVALID and "kernel_width_limit=341" in msg
    ok, (eid, msg) = call(harness, [(f32(20, 18), SINGLE), (f32(5, 5, 14, 14), SINGLE)])
    assert not ok and eid == INVALID and "15 x 15" in msg


@pytest.mark.gpu
def test_valid_call_matches_oracle(harness, cuda):
    bm, K = f32(40, 33, 2), f32(9, 9, 15, 15)
    ok, out = call(harness, [(bm, SINGLE), (K, SINGLE)], out_n=bm.size)
    assert ok, out
    got = out.reshape(bm.shape, order="F")
    ref = R.lfm_conv_vec(bm, K)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-5
