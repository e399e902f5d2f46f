"""The allocation-free minidisk advance (mara_minidisk_advance_noalloc).

Callers that cannot allocate device memory (a host whose pool allocator owns
all of the GPU's memory, a plugin that only receives the caller's buffers)
use this entry point: its scratch is a static device array inside the
library. The test calls it through the C ABI and checks, on two calls in a
row, that it produces what mara_minidisk_advance produces with a
caller-owned workspace: the same kernels on the same inputs, so the states
and clocks must be bit-identical. One case fills the whole static array (a
mesh of exactly the limit, mixed RK2). This file sorts last so that a run
stopping at the first failure has already run every other test; it also
passes alone.
"""
from __future__ import annotations

import ctypes

import pytest

from tests.helpers import REFERENCE_DISK, rel_l1_components

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def md():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import mara3p_gb300.minidisk as m
    return m


def lib_max_cells() -> int:
    return 512 * 512     # MARA_MINIDISK_NOALLOC_MAX_CELLS in include/mara_gb300.h


def clock_buffer(md, sd, u):
    from mara3p_gb300._capi import MinidiskClock, check, lib
    clock = torch.zeros(ctypes.sizeof(MinidiskClock), dtype=torch.uint8, device="cuda")
    check(lib.mara_minidisk_clock_init(ctypes.byref(sd.to_c()), u.data_ptr(), 0.0, clock.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream), "clock_init")
    return clock


@pytest.mark.parametrize("precision,dt_mode,mesh", [(0, 0, (64, 2)), (1, 1, (64, 2)), (1, 1, (128, 2))])
def test_noalloc_matches_workspace_advance_on_two_calls(md, precision, dt_mode, mesh):
    from mara3p_gb300._capi import check, lib
    block_size, depth = mesh
    sd = md.SolverData(**dict(REFERENCE_DISK, block_size=block_size, depth=depth))
    N = sd.cells_per_side
    need = lib.mara_minidisk_workspace_bytes(ctypes.byref(sd.to_c()), 2, precision)
    if N * N == lib_max_cells():
        assert need == 36 * N * N + 64, "the limit case must fill the whole static array (and its binary slot)"
    c = sd.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    u0 = md.initial_conserved(sd, seed=21, amplitude=0.01)
    ua, ub = u0.clone(), u0.clone()
    ca, cb = clock_buffer(md, sd, ua), clock_buffer(md, sd, ub)
    ws = torch.empty(lib.mara_minidisk_workspace_bytes(ctypes.byref(c), 2, precision), dtype=torch.uint8,
                     device="cuda")
    for call, steps in enumerate((3, 4)):
        check(lib.mara_minidisk_advance(ctypes.byref(c), ua.data_ptr(), ca.data_ptr(), steps, 2, precision, dt_mode,
                                        ws.data_ptr(), stream), "advance")
        check(lib.mara_minidisk_advance_noalloc(ctypes.byref(c), ub.data_ptr(), cb.data_ptr(), steps, 2, precision,
                                                dt_mode, stream), "advance_noalloc")
        torch.cuda.synchronize()
        assert torch.equal(ua, ub), (call, rel_l1_components(ub.cpu().numpy(), ua.cpu().numpy()))
        assert torch.equal(ca, cb), f"clocks differ after call {call}"


def test_noalloc_rejects_meshes_above_the_limit(md):
    from mara3p_gb300._capi import lib
    sd = md.SolverData(**dict(REFERENCE_DISK, depth=4))      # 1024^2 > 512^2 cells
    fake = ctypes.c_void_p(0x1000)    # never dereferenced: the size check fails first
    assert lib.mara_minidisk_advance_noalloc(ctypes.byref(sd.to_c()), fake, fake, 1, 2, 0, 0, None) == 1
    assert b"static scratch limit" in lib.mara_last_error()
