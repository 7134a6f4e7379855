"""Failure detection without a GPU fault: a device wait that nothing satisfies gives up
after its bound, the kernel reports the timeout through a status word and returns, the call
returns MLF_ERR_TIMEOUT, and the context stays usable (the same bounded mbarrier wait guards
every producer / MMA / epilogue hand-off of the tensor-core kernels)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_the_context_survives(cuda, lib):
    import torch
    from mesolf_gb300 import _lib
    assert lib.mlf_probe_wait_timeout(20000, None) == _lib.MLF_ERR_TIMEOUT
    buf = ctypes.create_string_buffer(256)
    assert lib.mlf_last_error(buf, 256) == _lib.MLF_ERR_TIMEOUT
    assert b"bounded wait expired" in buf.value
    # the context still works: torch and the library run afterwards
    a = torch.ones(4096, device=cuda)
    assert float(a.sum()) == 4096.0
    peak = ctypes.c_double()
    assert lib.mlf_probe_fp32_peak(2.0, ctypes.byref(peak), None) == 0
    assert peak.value > 1.0
    # and the wait times out again on a second call
    assert lib.mlf_probe_wait_timeout(1000, None) == _lib.MLF_ERR_TIMEOUT
