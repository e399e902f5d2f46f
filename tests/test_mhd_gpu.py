"""GPU parity of the constrained-transport MHD scheme (through the C ABI)
against the reference's golden fixtures and the oracle.

Tolerances: FP64 relative L1 per component <= 1e-12 after one step and two
RK2 steps (FMA contraction and libm only); div B at rounding; mixed path
(FP32 fluxes/EMFs, FP64 state) relative L1 <= 1e-5 after 20 RK2 steps with
div B still at FP64 rounding."""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

from oracle.oracle import dptr
from tests.helpers import rel_l1_components

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mh():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import mara3p_gb300.mhd as m
    return m


@pytest.fixture(scope="module")
def mhd_golden():
    from pathlib import Path
    return dict(np.load(Path(__file__).resolve().parent / "golden" / "mhd_golden.npz"))


def golden_state(mh, g):
    N, gamma, cfl, theta = g["mhd/params"]
    N = int(N)
    cfg = mh.MhdConfig(N=N, gamma_law_index=gamma, cfl=cfl, plm_theta=theta)
    s = mh.empty_state(cfg)
    s.uc.copy_(torch.from_numpy(g["mhd/uc"].reshape(N, N, N, 5).transpose(3, 0, 1, 2).copy()))
    shapes = [(N + 1, N, N), (N, N + 1, N), (N, N, N + 1)]
    for k in range(3):
        s.bf[k].copy_(torch.from_numpy(g[f"mhd/bf{k + 1}"].reshape(shapes[k])))
    return s


def soa(uc_aos, N):
    return uc_aos.reshape(N, N, N, 5).transpose(3, 0, 1, 2).reshape(5, -1)


@pytest.mark.parametrize("layout", ["soa", "aos"])
def test_advance_ct_fp64_matches_reference(mh, mhd_golden, layout):
    g = mhd_golden
    s = golden_state(mh, g)
    N = s.cfg.N
    uc_in = None
    if layout == "aos":
        uc_in = torch.from_numpy(g["mhd/uc"].copy()).cuda()
    out, clock = mh.advance_ct(s, uc_in=uc_in, layout=layout)
    assert abs(clock.read()["time"] - g["mhd/step_time"][0]) <= 1e-15
    assert rel_l1_components(out.uc.cpu().numpy().reshape(5, -1), soa(g["mhd/step_uc"], N), 5) < 1e-12
    for k in range(3):
        ref = g[f"mhd/step_bf{k + 1}"]
        assert np.abs(out.bf[k].cpu().numpy().ravel() - ref).sum() / np.abs(ref).sum() < 1e-12


def test_rk2_fp64_matches_reference(mh, mhd_golden):
    g = mhd_golden
    s = golden_state(mh, g)
    N = s.cfg.N
    run = mh.Run(s)
    run.advance(2)
    c = run.clock.read()
    assert abs(c["time"] - g["mhd/rk2_time"][0]) <= 1e-15
    assert c["failures"] == 0
    assert rel_l1_components(s.uc.cpu().numpy().reshape(5, -1), soa(g["mhd/rk2_uc"], N), 5) < 1e-12
    for k in range(3):
        ref = g[f"mhd/rk2_bf{k + 1}"]
        assert np.abs(s.bf[k].cpu().numpy().ravel() - ref).sum() / np.abs(ref).sum() < 1e-12


def test_initial_state_matches_oracle(mh, oracle, mhd_golden):
    g = mhd_golden
    N = int(g["mhd/params"][0])
    cfg = mh.MhdConfig(N=N)
    s = mh.initial_state(cfg, seed=3, modes=12)
    assert np.allclose(s.uc.cpu().numpy().reshape(5, -1), soa(g["mhd/uc"], N), rtol=1e-12, atol=1e-13)
    for k in range(3):
        assert np.allclose(s.bf[k].cpu().numpy().ravel(), g[f"mhd/bf{k + 1}"], rtol=1e-12, atol=1e-13)


def test_rk2_fp64_matches_oracle_longer(mh, oracle):
    """32^3, 10 RK2 steps: FP64 GPU vs the oracle, and div B at rounding."""
    oracle.oracle_mhd_rk2.restype = ctypes.c_double
    cfg = mh.MhdConfig(N=32)
    s = mh.initial_state(cfg, seed=11, modes=24)
    N = cfg.N
    uc = np.ascontiguousarray(s.uc.cpu().numpy().reshape(5, -1).T).ravel()
    bf = [b.cpu().numpy().ravel().copy() for b in s.bf]
    run = mh.Run(s)
    run.advance(10)
    t = oracle.oracle_mhd_rk2(N, dptr(uc), *[dptr(b) for b in bf], ctypes.c_double(0.0), 10, ctypes.c_double(1.0 / N),
                              ctypes.c_double(cfg.cfl), ctypes.c_double(cfg.plm_theta), ctypes.c_double(cfg.gamma_law_index))
    assert abs(run.clock.read()["time"] - t) <= 1e-13 * t
    assert rel_l1_components(s.uc.cpu().numpy().reshape(5, -1), soa(uc, N), 5) < 1e-11
    for k in range(3):
        assert np.abs(s.bf[k].cpu().numpy().ravel() - bf[k]).sum() / np.abs(bf[k]).sum() < 1e-11
    b_scale = max(float(b.abs().max()) for b in s.bf)
    assert run.max_div_b() < 1e-13 * b_scale


def test_mhd_128_full_size_fp64_matches_oracle(mh, oracle):
    """The MHD configuration at its own size (128^3, seeded modes, CFL dt):
    three FP64 RK2 steps against the oracle on all host threads at 1e-11,
    with div B at FP64 rounding."""
    oracle.oracle_mhd_rk2_threads.restype = ctypes.c_double
    cfg = mh.MhdConfig(N=128)
    s = mh.initial_state(cfg, seed=1, modes=24)
    N = cfg.N
    uc = np.ascontiguousarray(s.uc.cpu().numpy().reshape(5, -1).T).ravel()
    bf = [b.cpu().numpy().ravel().copy() for b in s.bf]
    run = mh.Run(s)
    run.advance(3)
    t = oracle.oracle_mhd_rk2_threads(N, dptr(uc), *[dptr(b) for b in bf], ctypes.c_double(0.0), 3,
                                      ctypes.c_double(1.0 / N), ctypes.c_double(cfg.cfl),
                                      ctypes.c_double(cfg.plm_theta), ctypes.c_double(cfg.gamma_law_index),
                                      os.cpu_count() or 1)
    assert t > 0.0
    assert abs(run.clock.read()["time"] - t) <= 1e-13 * t
    assert rel_l1_components(s.uc.cpu().numpy().reshape(5, -1), soa(uc, N), 5) < 1e-11
    for k in range(3):
        assert np.abs(s.bf[k].cpu().numpy().ravel() - bf[k]).sum() / np.abs(bf[k]).sum() < 1e-11
    b_scale = max(float(b.abs().max()) for b in s.bf)
    assert run.max_div_b() < 1e-13 * b_scale


def test_mixed_close_to_fp64_and_divergence_free(mh):
    cfg = mh.MhdConfig(N=32)
    a = mh.initial_state(cfg, seed=5, modes=24)
    b = mh.initial_state(cfg, seed=5, modes=24)
    ra, rb = mh.Run(a), mh.Run(b, precision=mh.MIXED)
    ra.advance(20)
    rb.advance(20)
    assert rel_l1_components(b.uc.cpu().numpy().reshape(5, -1), a.uc.cpu().numpy().reshape(5, -1), 5) < 1e-5
    b_scale = max(float(x.abs().max()) for x in b.bf)
    assert rb.max_div_b() < 1e-13 * b_scale
    assert rb.clock.read()["failures"] == 0


def test_advance_checked_restores_and_raises_on_failed_zones(mh):
    """A zone whose energy is set negative on the host fails its recovery
    (the reference throws there): advance_checked puts the state back and
    raises; an unpoisoned run advances normally."""
    from mara3p_gb300._capi import MaraError
    cfg = mh.MhdConfig(N=16)
    s = mh.initial_state(cfg, seed=4, modes=8)
    run = mh.Run(s)
    run.advance_checked(2)
    assert run.clock.read()["iteration"] == 2
    s.uc[4, 3, 4, 5] = -10.0
    before = [s.uc.clone()] + [b.clone() for b in s.bf]
    t0 = run.clock.read()["time"]
    with pytest.raises(MaraError, match="restored"):
        run.advance_checked(1)
    assert torch.equal(s.uc, before[0]) and all(torch.equal(b, b0) for b, b0 in zip(s.bf, before[1:]))
    assert run.clock.read()["time"] == t0


def _mixed_runs(mh, N, steps, chunks, seed=7):
    """(state tensors, clock) of a mixed RK2 run with the fused stage on and off."""
    from mara3p_gb300._capi import check, lib
    out = []
    try:
        for enable in (1, 0):
            check(lib.mara_mhd_fused_stage(enable, chunks), "fused stage")
            s = mh.initial_state(mh.MhdConfig(N=N), seed=seed, modes=24)
            r = mh.Run(s, precision=mh.MIXED)
            r.advance(steps)
            torch.cuda.synchronize()
            out.append(([s.uc.clone()] + [b.clone() for b in s.bf], r.clock.read()))
    finally:
        check(lib.mara_mhd_fused_stage(1, 0), "fused stage")
    return out


@pytest.mark.parametrize("N,steps,chunks", [(32, 6, 0), (32, 3, 32), (64, 4, 5), (96, 2, 7), (128, 3, 0)])
def test_mixed_fused_stage_bit_identical(mh, N, steps, chunks):
    """The fused mixed stage (faces, edge EMFs and both updates in one launch)
    against the face and update kernels over mixed RK2 steps: states, face
    fields and clocks identical bit for bit, at several splittings of the i
    axis (one plane per chunk included) and at the 128^3 configuration."""
    (fa, ca), (fb, cb) = _mixed_runs(mh, N, steps, chunks)
    for x, y in zip(fa, fb):
        assert torch.equal(x, y)
    assert ca["time"] == cb["time"] and ca["dt"] == cb["dt"]
    assert ca["failures"] == cb["failures"] == 0


@pytest.mark.parametrize("layout", ["soa", "aos"])
def test_mixed_fused_single_stage_bit_identical(mh, layout):
    """advance_ct (one forward-Euler stage, input in either layout) with the
    fused stage on and off: identical outputs."""
    from mara3p_gb300._capi import check, lib
    N = 64
    s = mh.initial_state(mh.MhdConfig(N=N), seed=9, modes=24)
    uc_in = s.uc.reshape(5, -1).t().contiguous() if layout == "aos" else None
    outs = []
    try:
        for enable in (1, 0):
            check(lib.mara_mhd_fused_stage(enable, 0), "fused stage")
            out, clock = mh.advance_ct(s, uc_in=uc_in, layout=layout, precision=mh.MIXED)
            torch.cuda.synchronize()
            outs.append(([out.uc] + list(out.bf), clock.read()["time"]))
    finally:
        check(lib.mara_mhd_fused_stage(1, 0), "fused stage")
    for x, y in zip(outs[0][0], outs[1][0]):
        assert torch.equal(x, y)
    assert outs[0][1] == outs[1][1]


def test_fused_stage_switch_rejects_bad_arguments(mh):
    from mara3p_gb300._capi import lib
    assert lib.mara_mhd_fused_stage(2, 0) != 0
    assert lib.mara_mhd_fused_stage(1, -1) != 0
    assert lib.mara_mhd_fused_stage(1, 0) == 0


def test_mixed_fused_unaligned_face_arrays(mh):
    """Face arrays that are 8- but not 16-byte aligned (allowed at the C ABI)
    take the fused path's element copies: the same outputs as aligned copies
    of the same data."""
    import ctypes as ct

    from mara3p_gb300._capi import check, lib
    N = 32
    s = mh.initial_state(mh.MhdConfig(N=N), seed=13, modes=24)
    cfg = s.cfg.to_c()
    ws = torch.empty(lib.mara_mhd_workspace_bytes(ct.byref(cfg), 1, mh.MIXED), dtype=torch.uint8, device="cuda")
    outs = []
    for offset in (0, 1):
        bins, bouts = [], []
        for b in s.bf:
            buf = torch.zeros(b.numel() + 2, dtype=torch.float64, device="cuda")
            buf[offset:offset + b.numel()] = b.reshape(-1)
            bins.append(buf[offset:offset + b.numel()])
            bouts.append(torch.zeros(b.numel() + 2, dtype=torch.float64, device="cuda")[offset:offset + b.numel()])
        uc_out = torch.empty_like(s.uc)
        clock = mh.Clock()
        check(lib.mara_mhd_advance_ct(ct.byref(cfg), s.uc.data_ptr(), N ** 3, 1, *[b.data_ptr() for b in bins],
                                      uc_out.data_ptr(), *[b.data_ptr() for b in bouts], clock.buf.data_ptr(),
                                      mh.MIXED, ws.data_ptr(), torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        assert offset == 0 or bins[0].data_ptr() % 16 == 8
        outs.append([uc_out] + bouts)
    for x, y in zip(*outs):
        assert torch.equal(x, y)


def test_advance_checked_on_the_fused_path(mh):
    """The rollback of advance_checked with the mixed fused stage (N = 32):
    a poisoned zone is counted by the first stage's recovery, the state and
    clock are put back, and an unpoisoned three-step call (odd, so the face
    fields end in the workspace scratch and are copied back) advances."""
    from mara3p_gb300._capi import MaraError
    s = mh.initial_state(mh.MhdConfig(N=32), seed=6, modes=8)
    run = mh.Run(s, precision=mh.MIXED)
    run.advance_checked(3)
    c = run.clock.read()
    assert c["iteration"] == 3 and c["failures"] == 0
    s.uc[4, 5, 6, 7] = -10.0
    before = [s.uc.clone()] + [b.clone() for b in s.bf]
    t0 = c["time"]
    with pytest.raises(MaraError, match="restored"):
        run.advance_checked(2)
    assert torch.equal(s.uc, before[0]) and all(torch.equal(b, b0) for b, b0 in zip(s.bf, before[1:]))
    assert run.clock.read()["time"] == t0
