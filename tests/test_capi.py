"""The C-ABI library builds, loads and exports every symbol the header declares; host-side
argument validation (no GPU compute)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "mesolf_lf.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mlf_[a-z0-9_]+)\s*\(", src)))


def test_header_lists_entry_points():
    fns = header_functions()
    assert "mlf_conv_vec" in fns and "mlf_solver_run" in fns and len(fns) >= 14


def test_library_exports_every_declared_symbol(lib):
    from mesolf_gb300 import _lib
    for name in header_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} missing from the ctypes signature table"
    assert lib.mlf_version() == 3


def _err(lib):
    buf = ctypes.create_string_buffer(512)
    code = lib.mlf_last_error(buf, 512)
    return code, buf.value.decode()


def test_conv_vec_rejects_like_the_mex(lib):
    a = np.zeros(16, np.float32)
    p = a.ctypes.data
    # kw above kernel_width_limit (mex_lfm_convolution_vec.cu:344)
    assert lib.mlf_conv_vec(p, 4, 4, 1, p, 342, 15, p, None) == 1
    assert "kernel_width_limit" in _err(lib)[1]
    # bitmap_n < 1 (:332)
    assert lib.mlf_conv_vec(p, 4, 4, 0, p, 3, 15, p, None) == 1
    assert "at least 1" in _err(lib)[1]
    # null pointers, wrong kernel grid
    assert lib.mlf_conv_vec(None, 4, 4, 1, p, 3, 15, p, None) == 1
    assert lib.mlf_conv_vec(p, 4, 4, 1, p, 3, 13, p, None) == 1
    assert _err(lib)[0] == 1


def test_psf_create_rejects_bad_shapes(lib):
    a = np.zeros(16, np.float32)
    p = a.ctypes.data
    h = ctypes.c_void_p()
    assert lib.mlf_psf_create(p, p, 60, 15, 3, ctypes.byref(h), None) == 1   # even K0
    assert lib.mlf_psf_create(p, p, 61, 14, 3, ctypes.byref(h), None) == 1   # even N
    assert lib.mlf_psf_create(p, p, 61, 15, 0, ctypes.byref(h), None) == 1   # no planes
    # S/N = 19 (K0 = 285) is beyond the supported tap counts
    assert lib.mlf_psf_create(p, p, 285, 15, 1, ctypes.byref(h), None) == 4
    assert "supported" in _err(lib)[1]
    assert lib.mlf_psf_create(None, p, 61, 15, 1, ctypes.byref(h), None) == 1


def test_solver_rejects_null(lib):
    h = ctypes.c_void_p()
    assert lib.mlf_solver_create(None, 165, 165, ctypes.byref(h)) == 1
    assert lib.mlf_solver_run(None, None, 1, 0, None, None, None, None) == 1


def test_python_api_no_cpu_fallback():
    from mesolf_gb300 import MesoLFError, recon_theory_phase_space_LFM_with_filter
    with pytest.raises(MesoLFError):
        recon_theory_phase_space_LFM_with_filter(np.zeros((15, 15)), np.zeros((15, 15, 15, 15, 1)),
                                                 np.zeros((15, 15, 15, 15, 1)), 1, gpuFlag=False)


def test_stats_struct_layout_matches_the_header(tmp_path):
    """The ctypes mirror of mlf_stats has the size and field offsets the C compiler gives
    the header's struct (a mismatch would make the library write past the caller's struct)."""
    import shutil
    import subprocess
    from mesolf_gb300._lib import MLFStats
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = os.path.join(ROOT, "include")
    fields = [f for f, _ in MLFStats._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"mesolf_lf.h\"\nint main(void){\n"
                   "printf(\"%zu\\n\", sizeof(mlf_stats));\n" +
                   "".join(f"printf(\"%zu\\n\", offsetof(mlf_stats, {f}));\n" for f in fields) +
                   "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(MLFStats)
    assert out[1:] == [getattr(MLFStats, f).offset for f in fields]


def test_wait_probe_rejects_limits_before_any_device_work(lib):
    from mesolf_gb300 import _lib
    assert lib.mlf_probe_wait_timeout(0, None) == _lib.MLF_ERR_INVALID
    assert lib.mlf_probe_wait_timeout((1 << 20) + 1, None) == _lib.MLF_ERR_INVALID
