"""The measurement helpers the bench's rooflines divide by: the FP64 FMA
rate and the host-link rates. Each returns plausible positive rates on the
GPU and refuses bad arguments without touching the device. Also the
library's self-check of its integer float<->double conversions against the
GPU's conversion instructions."""
from __future__ import annotations

import ctypes

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mara3p_gb300 import _capi
    return _capi


def test_fp64_rate_positive(capi):
    r = ctypes.c_double()
    capi.check(capi.lib.mara_measure_fp64_rate(ctypes.byref(r), torch.cuda.current_stream().cuda_stream))
    # between 1e9 and 1e15 thread-level DFMA per second on any current part
    assert 1e9 < r.value < 1e15


def test_host_link_rates(capi):
    nbytes = 64 << 20
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    g = (ctypes.c_double * 5)()
    capi.check(capi.lib.mara_measure_host_link(host.data_ptr(), dev.data_ptr(), nbytes, g,
                                               torch.cuda.current_stream().cuda_stream))
    assert all(1.0 < v < 10000.0 for v in g), list(g)


def test_host_link_rejects_bad_arguments(capi):
    g = (ctypes.c_double * 5)()
    dev = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    # device memory where pinned host memory is required
    assert capi.lib.mara_measure_host_link(dev.data_ptr(), dev.data_ptr(), 1 << 20, g, None) != 0
    assert b"pinned" in capi.lib.mara_last_error()
    host = torch.empty(1 << 20, dtype=torch.uint8, pin_memory=True)
    assert capi.lib.mara_measure_host_link(host.data_ptr(), dev.data_ptr(), 1000, g, None) != 0
    assert capi.lib.mara_measure_host_link(None, dev.data_ptr(), 1 << 20, g, None) != 0


def test_integer_conversions_match_the_hardware(capi):
    """f2d and its increment form over all 2^32 floats, d2f over 2^32 doubles
    (every high word, hashed low words, exact ties included): no mismatch."""
    bad = (ctypes.c_ulonglong * 3)()
    capi.check(capi.lib.mara_check_conversions(bad, torch.cuda.current_stream().cuda_stream))
    assert list(bad) == [0, 0, 0], list(bad)
