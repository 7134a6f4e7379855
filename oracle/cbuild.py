"""Build recipe for the C/OpenMP oracle port (test infrastructure and CPU baseline only).

    python oracle/cbuild.py          -> oracle/_build/libmlf_oracle.so

Plain gcc, portable flags (no -march=native): the same source builds on x86_64 and on the
Arm hosts of the GPU machines.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mlf_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmlf_oracle.so")


def build():
    os.makedirs(OUT_DIR, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", SRC, "-o", LIB, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        d = ctypes.POINTER(ctypes.c_double)
        i = ctypes.c_int64
        lib.mlf_oracle_threads.restype = ctypes.c_int
        lib.mlf_oracle_forward.argtypes = [d, i, d, i, i, i, i, d]
        lib.mlf_oracle_backward.argtypes = [d, i, d, i, i, i, i, i, i, d]
        lib.mlf_oracle_view_step.argtypes = [d, d, i, d, d, i, i, i, i, i, i, ctypes.c_double]
        lib.mlf_oracle_view_step.restype = ctypes.c_int
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    import numpy as np
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def forward(h, X, N):
    import numpy as np
    h, X = _f64(h), _f64(X)
    Xr, Xc, Z = X.shape
    out = np.zeros((Xr // N, Xc // N), order="F")
    load().mlf_oracle_forward(_p(h), h.shape[0], _p(X), Xr, Xc, Z, N, _p(out))
    return out


def backward(t, R, u, v, N):
    import numpy as np
    t, R = _f64(t), _f64(R)
    Li, Lj = R.shape
    Z = t.shape[2]
    out = np.zeros((Li * N, Lj * N, Z), order="F")
    load().mlf_oracle_backward(_p(t), t.shape[0], _p(R), Li, Lj, u, v, N, Z, _p(out))
    return out


def view_step(h, t, LF, X, u, v, w, N):
    """One RL view step; returns the updated volume (X is not modified)."""
    h, t, LF = _f64(h), _f64(t), _f64(LF)
    Xo = _f64(X).copy(order="F")
    Xr, Xc, Z = Xo.shape
    if load().mlf_oracle_view_step(_p(h), _p(t), h.shape[0], _p(LF), _p(Xo), Xr, Xc, Z, N, u, v, float(w)):
        raise MemoryError("oracle view step: allocation failed")
    return Xo


def threads():
    return int(load().mlf_oracle_threads())


if __name__ == "__main__":
    print(build())
