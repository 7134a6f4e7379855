"""Recipe: the reference's own MEX kernel, built from its source for the parity tests.

    python oracle/refbuild.py

* ``oracle/_ref/mex_lfm_convolution_vec.cubin``: the reference file
  ``src/cuda/mex_lfm_convolution_vec.cu`` compiled where it lies, unchanged, for sm_103a.
  ``oracle/ref_mex/mlf_ref_compat.h`` is force-included to stand in for the texture
  references CUDA 12 removed (plain bounds-checked loads) and for MATLAB's MEX headers
  (declarations only; the host function is never run).  Built only where the reference
  source exists; elsewhere a cubin built earlier is used as it is.
* ``oracle/_build/libmlf_ref_mex.so``: the launcher (``oracle/ref_mex/ref_mex_launch.cu``)
  that loads that cubin and launches the kernel with the reference's launch geometry.

Test infrastructure only: the product never loads either file.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_ROOT = os.environ.get("MLF_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src", "cuda", "mex_lfm_convolution_vec.cu")
COMPAT = os.path.join(HERE, "ref_mex", "mlf_ref_compat.h")
MEX_HEADERS = os.path.join(ROOT, "tests", "mex_fake")
CUBIN = os.path.join(HERE, "_ref", "mex_lfm_convolution_vec.cubin")
LAUNCH_SRC = os.path.join(HERE, "ref_mex", "ref_mex_launch.cu")
LAUNCH_LIB = os.path.join(HERE, "_build", "libmlf_ref_mex.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_cubin():
    """Compile the reference kernel if its source is here.  Returns the cubin path, or None
    when there is neither the source nor a cubin built earlier."""
    nvcc = _nvcc()
    if os.path.exists(REF_SRC) and nvcc:
        deps = [REF_SRC, COMPAT]
        if not os.path.exists(CUBIN) or os.path.getmtime(CUBIN) < max(os.path.getmtime(d) for d in deps):
            os.makedirs(os.path.dirname(CUBIN), exist_ok=True)
            _run([nvcc, "-cubin", *ARCH, "-O3", "-lineinfo", "-include", COMPAT, "-I", MEX_HEADERS,
                  REF_SRC, "-o", CUBIN])
    return CUBIN if os.path.exists(CUBIN) else None


def build_launcher():
    nvcc = _nvcc()
    if nvcc is None:
        return None
    if not os.path.exists(LAUNCH_LIB) or os.path.getmtime(LAUNCH_LIB) < os.path.getmtime(LAUNCH_SRC):
        os.makedirs(os.path.dirname(LAUNCH_LIB), exist_ok=True)
        _run([nvcc, *ARCH, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-cudart", "static",
              LAUNCH_SRC, "-o", LAUNCH_LIB])
    return LAUNCH_LIB


def build():
    return build_cubin(), build_launcher()


class ReferenceMex:
    """The reference kernel on the current CUDA device (device pointers in, synchronous)."""

    def __init__(self):
        cubin, lib = build()
        if cubin is None or lib is None:
            raise FileNotFoundError("reference MEX cubin or launcher not built")
        self.lib = ctypes.CDLL(lib)
        self.lib.mlf_ref_mex_error.restype = ctypes.c_char_p
        self.lib.mlf_ref_mex_load.argtypes = [ctypes.c_char_p]
        self.lib.mlf_ref_mex_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_double)]
        if self.lib.mlf_ref_mex_load(cubin.encode()):
            raise RuntimeError(self.lib.mlf_ref_mex_error().decode())

    def run(self, bitmap_ptr, W, H, n, kernels_ptr, kw, out_ptr):
        """Returns the device time of the launches in ms."""
        ms = ctypes.c_double(0.0)
        if self.lib.mlf_ref_mex_run(bitmap_ptr, W, H, n, kernels_ptr, kw, out_ptr, ctypes.byref(ms)):
            raise RuntimeError(self.lib.mlf_ref_mex_error().decode())
        return ms.value


if __name__ == "__main__":
    print(build())
