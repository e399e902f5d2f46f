"""GPU parity of the minidisk path, through the C ABI, against the oracle and
the reference's golden fixtures.

Tolerances (relative L1 per component, sum|gpu - ref| / sum|ref|):
  plain FP64 path: 1e-12 after one step, 1e-9 after 1000 steps (only FMA
  contraction and CUDA-vs-glibc libm rounding differ);
  integer-like / order-free operations (primitive recovery, PLM slopes,
  initial state): bit-exact.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

from oracle.oracle import dptr, params
from tests.golden.make_golden import MINIDISK_CASES
from tests.helpers import REFERENCE_DISK, LARGE_DISK, SMALL_PARAMS, params_from_vector, rel_l1_components

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FP64_ONE_STEP = 1e-12
FP64_1000_STEPS = 1e-9


@pytest.fixture(scope="module")
def md():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import mara3p_gb300.minidisk as m
    return m


def sd_from(md, p):
    return md.SolverData(**{name: getattr(p, name) for name, _ in p._fields_})


def to_gpu(a, shape):
    return torch.from_numpy(np.ascontiguousarray(a).reshape(shape)).cuda()


@pytest.mark.parametrize("case", list(MINIDISK_CASES))
def test_substep_fp64_matches_reference(md, golden, case):
    p = params_from_vector(golden[f"{case}/params"], float(golden[f"{case}/theta"][0]))
    sd = sd_from(md, p)
    N = sd.cells_per_side
    u0 = to_gpu(golden[f"{case}/u0"], (3, N, N))
    t, dt = golden[f"{case}/t"]
    out = md.substep(sd, u0, float(t), float(dt)).cpu().numpy()
    assert rel_l1_components(out, golden[f"{case}/substep"]) < FP64_ONE_STEP


@pytest.mark.parametrize("case", list(MINIDISK_CASES))
def test_rk2_device_clock_matches_reference(md, golden, case):
    p = params_from_vector(golden[f"{case}/params"], float(golden[f"{case}/theta"][0]))
    sd = sd_from(md, p)
    N = sd.cells_per_side
    run = md.Run(sd, to_gpu(golden[f"{case}/u0"], (3, N, N)).clone(), time=0.0, rk_order=2,
                 precision=md.FP64, dt_mode=md.DT_FORMULA)
    run.advance(5)
    torch.cuda.synchronize()
    assert rel_l1_components(run.u.cpu().numpy(), golden[f"{case}/rk2_5"]) < FP64_ONE_STEP * 10
    assert abs(run.time - golden[f"{case}/rk2_5_time"][0]) < 1e-15


def test_block_updated_conserved_dropin(md, golden):
    p = params_from_vector(golden["block/params"])
    sd = sd_from(md, p)
    n = sd.block_size
    level, bi, bj = (int(x) for x in golden["block/index"])
    t, dt = golden["block/time_dt"]
    u1 = md.updated_conserved(to_gpu(golden["block/uc"], (n, n, 3)), to_gpu(golden["block/pe"], (n + 4, n + 4, 3)),
                              float(t), float(dt), (level, bi, bj), sd)
    got = u1.cpu().numpy().reshape(-1, 3).T
    ref = golden["block/u1"].reshape(-1, 3).T
    assert rel_l1_components(got, ref) < FP64_ONE_STEP


@pytest.mark.parametrize("theta", [1.5, 2.0])
@pytest.mark.parametrize("axis", [0, 1])
def test_estimate_gradient_bitexact(md, golden, theta, axis):
    pe = golden["block/pe"]
    g = md.estimate_gradient(to_gpu(pe, pe.shape), axis, theta).cpu().numpy()
    assert np.array_equal(g, golden[f"gradient/theta{theta}/axis{axis}"])


def test_recover_primitive_bitexact(md, oracle, golden):
    uc = golden["block/uc"]
    got = md.recover_primitive_array(to_gpu(uc, uc.shape)).cpu().numpy()
    ref = np.zeros_like(uc)
    oracle.oracle_minidisk_recover_primitive(dptr(uc), ctypes.c_int64(uc.size // 3), dptr(ref))
    assert np.array_equal(got, ref)


def test_recover_primitive_empty(md):
    out = md.recover_primitive_array(torch.empty((0, 3), dtype=torch.float64, device="cuda"))
    assert out.shape == (0, 3)


@pytest.mark.parametrize("amplitude", [0.0, 0.01])
def test_initial_conserved_bitexact(md, oracle, amplitude):
    sd = md.SolverData(**REFERENCE_DISK)
    u = md.initial_conserved(sd, seed=77, amplitude=amplitude).cpu().numpy()
    ref = np.zeros(u.size)
    oracle.oracle_minidisk_initial_conserved(ctypes.byref(params(sd)), ctypes.c_uint64(77), ctypes.c_double(amplitude),
                                             dptr(ref))
    assert np.array_equal(u.ravel(), ref)


def test_reference_disk_physics_one_step_and_1000_steps_fp64(md, oracle):
    """Plain FP64 GPU vs the oracle on the same seeded input: one RK2 step at
    1e-12 and 1000 RK2 steps at 1e-9 (64^2 mesh, the 256^2 disk's physics)."""
    sd = md.SolverData(**SMALL_PARAMS)
    u0 = md.initial_conserved(sd, seed=5, amplitude=0.01)
    ref = u0.cpu().numpy().ravel().copy()
    run = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_FORMULA)
    run.advance(1)
    t = oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(0.0), 1, 2, 0, 8)
    assert rel_l1_components(run.u.cpu().numpy(), ref) < FP64_ONE_STEP
    run.advance(999)
    t = oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(t), 999, 2, 0, 8)
    assert rel_l1_components(run.u.cpu().numpy(), ref) < FP64_1000_STEPS
    assert abs(run.time - t) <= 1e-12 * t


def test_reference_disk_full_size_one_step(md, oracle):
    """Config 1 itself (256^2, 4x4 blocks of 64^2): one RK2 step at 1e-12."""
    sd = md.SolverData(**REFERENCE_DISK)
    u0 = md.initial_conserved(sd, seed=1, amplitude=0.01)
    ref = u0.cpu().numpy().ravel().copy()
    run = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_FORMULA)
    run.advance(2)
    oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(0.0), 2, 2, 0, 8)
    assert rel_l1_components(run.u.cpu().numpy(), ref) < FP64_ONE_STEP


THREADS = os.cpu_count() or 1


def test_reference_disk_full_size_1000_steps_fp64(md, oracle):
    """The reference-sized disk at its own size and physics (256^2, 4x4 blocks of
    64^2, theta 1.5, CFL dt): one RK2 step at 1e-12 and 1000 RK2 steps at
    1e-9 against the oracle, with the clocks' times alike."""
    sd = md.SolverData(**dict(REFERENCE_DISK, plm_theta=1.5))
    u0 = md.initial_conserved(sd, seed=1, amplitude=0.01)
    ref = u0.cpu().numpy().ravel().copy()
    run = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_CFL)
    run.advance(1)
    t = oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(0.0), 1, 2, 1, THREADS)
    assert rel_l1_components(run.u.cpu().numpy(), ref) < FP64_ONE_STEP
    run.advance(999)
    t = oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(t), 999, 2, 1, THREADS)
    assert np.isfinite(ref).all()
    assert rel_l1_components(run.u.cpu().numpy(), ref) < FP64_1000_STEPS
    assert abs(run.time - t) <= 1e-12 * t


def test_large_disk_full_size_one_step_fp64(md, oracle):
    """The large disk itself (4096^2, theta 1.5, q 0.5, e 0.1, Mach 20, CFL
    dt): one FP64 RK2 step at 1e-12 against the oracle on all host threads,
    and the CFL dt (an FP64 reduction over all 16.8 M cells) at 1e-14."""
    sd = md.SolverData(**LARGE_DISK)
    u0 = md.initial_conserved(sd, seed=1, amplitude=0.01)
    ref = u0.cpu().numpy().ravel().copy()
    run = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_CFL)
    run.advance(1)
    dt_ref = oracle.oracle_minidisk_dt_cfl(ctypes.byref(params(sd)), dptr(ref))
    t = oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(0.0), 1, 2, 1, THREADS)
    c = run.clock_state()
    assert abs(c.dt - dt_ref) <= 1e-14 * dt_ref
    assert abs(c.time - t) <= 1e-14 * t
    assert rel_l1_components(run.u.cpu().numpy(), ref) < FP64_ONE_STEP


def test_cfl_dt_matches_oracle(md, oracle):
    sd = md.SolverData(**SMALL_PARAMS)
    u0 = md.initial_conserved(sd, seed=3, amplitude=0.01)
    run = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_CFL)
    run.advance(1)
    dt_gpu = run.clock_state().dt
    dt_ref = oracle.oracle_minidisk_dt_cfl(ctypes.byref(params(sd)), dptr(u0.cpu().numpy().ravel().copy()))
    assert abs(dt_gpu - dt_ref) <= 1e-14 * dt_ref
    # the fused reduction of the new state seeds the next step's dt
    run.advance(1)
    ref = run.u.cpu().numpy().ravel().copy()
    u_prev = u0.cpu().numpy().ravel().copy()
    oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(u_prev), ctypes.c_double(0.0), 2, 2, 1, 8)
    assert rel_l1_components(ref, u_prev) < FP64_ONE_STEP * 10


def test_rk1_fp64_matches_oracle(md, oracle):
    sd = md.SolverData(**SMALL_PARAMS)
    u0 = md.initial_conserved(sd, seed=9, amplitude=0.01)
    ref = u0.cpu().numpy().ravel().copy()
    run = md.Run(sd, u0.clone(), rk_order=1, precision=md.FP64, dt_mode=md.DT_FORMULA)
    run.advance(3)
    oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(0.0), 3, 1, 0, 8)
    assert rel_l1_components(run.u.cpu().numpy(), ref) < FP64_ONE_STEP


@pytest.mark.parametrize("rk_order,steps,block_size", [(1, 20, 16), (2, 200, 16), (2, 200, 8)])
def test_mixed_precision_close_to_fp64(md, rk_order, steps, block_size):
    """Mixed path (FP32 fluxes/sources, FP64 accumulation) vs plain FP64 GPU:
    density and momentum relative L1 below 1e-6 (forward Euler with PLM is
    not stable for long runs, so RK1 runs 20 steps). 64^2 meshes run the
    warp-strip sweep kernel, 32^2 meshes the tiled one."""
    sd = md.SolverData(**dict(SMALL_PARAMS, block_size=block_size))
    u0 = md.initial_conserved(sd, seed=11, amplitude=0.01)
    a = md.Run(sd, u0.clone(), rk_order=rk_order, precision=md.FP64, dt_mode=md.DT_FORMULA)
    b = md.Run(sd, u0.clone(), rk_order=rk_order, precision=md.MIXED, dt_mode=md.DT_FORMULA)
    a.advance(steps)
    b.advance(steps)
    assert torch.isfinite(a.u).all()
    err = rel_l1_components(b.u.cpu().numpy(), a.u.cpu().numpy())
    assert err < 1e-6, err
    assert a.time == b.time


def test_mixed_long_horizon_large_disk_physics(md):
    """The mixed path against the plain FP64 path over 2000 CFL steps of the
    large-minidisk physics (q 0.5, e 0.1, Mach 20, theta 1.5) on a 1024^2
    mesh of the same domain: density and momentum relative L1 at most 1e-6.
    (The primitive velocity is an FMA-corrected quotient: with the biased
    single-MUFU reciprocal the 4096^2 configuration was 4.8e-6 from FP64
    after 1000 steps, with the corrected quotient 7.4e-7.)"""
    sd = md.SolverData(**dict(LARGE_DISK, depth=4))
    u0 = md.initial_conserved(sd, seed=1234, amplitude=0.01)
    a = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_CFL)
    b = md.Run(sd, u0.clone(), rk_order=2, precision=md.MIXED, dt_mode=md.DT_CFL)
    a.advance(2000)
    b.advance(2000)
    assert torch.isfinite(a.u).all() and torch.isfinite(b.u).all()
    err = rel_l1_components(b.u.cpu().numpy(), a.u.cpu().numpy())
    assert err <= 1e-6, err
    assert abs(a.time - b.time) <= 1e-6 * a.time


@pytest.mark.parametrize("block_size,depth", [(64, 3), (100, 2), (128, 5)])
def test_sweep_tma_ring_bit_identical(md, block_size, depth):
    """Rows staged by bulk tensor copies and by per-lane asynchronous copies
    (the default) give bit-identical states and clocks: meshes of 512^2,
    400^2 (strips of both kinds) and 4096^2."""
    from mara3p_gb300._capi import lib
    sd = md.SolverData(**dict(LARGE_DISK, block_size=block_size, depth=depth))
    u0 = md.initial_conserved(sd, seed=31, amplitude=0.01)
    out = []
    try:
        for tma in (1, 0):
            assert lib.mara_minidisk_sweep_tma(tma) in (0, 1)
            run = md.Run(sd, u0.clone(), rk_order=2, precision=md.MIXED, dt_mode=md.DT_CFL)
            run.advance(6)
            torch.cuda.synchronize()
            out.append((run.u.clone(), run.clock.clone()))
    finally:
        lib.mara_minidisk_sweep_tma(0)
    assert torch.equal(out[0][0], out[1][0])
    assert torch.equal(out[0][1], out[1][1])
    assert lib.mara_minidisk_sweep_tma(2) == -1


def test_mass_conservation_full_size(md):
    """Size-independent property at the large disk's size (4096^2): with sinks,
    buffer and viscosity off, the flux divergence telescopes and total mass
    is conserved to rounding, in both precisions."""
    sd = md.SolverData(block_size=64, depth=6, domain_radius=8.0, softening_length=0.05, mach_number=20.0,
                       sink_rate=0.0, buffer_rate=0.0, nu=0.0, sink_radius=0.05, eccentricity=0.1, mass_ratio=0.5)
    u0 = md.initial_conserved(sd, seed=2, amplitude=0.01)
    m0 = u0[0].sum().item()
    for precision in (md.MIXED, md.FP64):
        run = md.Run(sd, u0.clone(), rk_order=2, precision=precision, dt_mode=md.DT_CFL)
        run.advance(2)
        assert abs(run.u[0].sum().item() - m0) < 1e-11 * m0


@pytest.mark.parametrize("block_size,depth", [(64, 0), (66, 0), (96, 1), (100, 1), (64, 2), (80, 2)])
def test_sweep_column_forms_bit_identical(md, block_size, depth):
    """The 1-column sweep and the 2-column sweep (a column pair per lane)
    give bit-identical states and clocks: the mixed path
    rounds every operation explicitly. Meshes whose cell size is not a power
    of two (96, 200, 320) catch any rewritten product; N = 66 leaves a
    6-column last strip. (Odd N puts a cell centre on the origin, where the
    reference's initial state divides by r = 0, so it is not a minidisk mesh.)"""
    from mara3p_gb300._capi import lib
    sd = md.SolverData(**dict(REFERENCE_DISK, block_size=block_size, depth=depth, plm_theta=1.5))
    u0 = md.initial_conserved(sd, seed=5, amplitude=0.01)
    out = []
    try:
        for cols in (1, 2):
            assert lib.mara_minidisk_sweep_columns(cols) in (0, 1, 2)
            for rk in (1, 2):
                run = md.Run(sd, u0.clone(), rk_order=rk, precision=md.MIXED, dt_mode=md.DT_CFL)
                run.advance(6 if rk == 2 else 3)
                torch.cuda.synchronize()
                out.append((cols, rk, run.u.clone(), run.clock_state()))
    finally:
        lib.mara_minidisk_sweep_columns(0)
    for (c1, rk1, u1, k1), (c2, rk2, u2, k2) in zip(out[:2], out[2:]):
        assert rk1 == rk2 and c1 == 1 and c2 == 2
        assert torch.isfinite(u1).all()
        assert torch.equal(u1, u2), (block_size, depth, rk1, float((u1 - u2).abs().max()))
        assert (k1.time, k1.dt, k1.max_wavespeed, k1.iteration) == (k2.time, k2.dt, k2.max_wavespeed, k2.iteration)
    assert lib.mara_minidisk_sweep_columns(3) == -1


@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
@pytest.mark.parametrize("dt_mode_name", ["DT_CFL", "DT_FORMULA"])
def test_graph_replay_matches_direct_advance(md, precision, dt_mode_name):
    """Run.use_graph replays captured steps: the same bits, clock and time as
    advancing directly (including a remainder shorter than one replay)."""
    sd = md.SolverData(**dict(REFERENCE_DISK, block_size=64, depth=1, plm_theta=1.5))
    u0 = md.initial_conserved(sd, seed=21, amplitude=0.01)
    kw = dict(rk_order=2, precision=getattr(md, precision), dt_mode=getattr(md, dt_mode_name))
    direct = md.Run(sd, u0.clone(), **kw)
    direct.advance(4 + 13)
    replay = md.Run(sd, u0.clone(), **kw)
    replay.use_graph(4)                 # advances 4 steps while preparing
    replay.advance(13)                  # 3 replays + 1 direct step
    torch.cuda.synchronize()
    assert torch.isfinite(direct.u).all()
    assert torch.equal(direct.u, replay.u)
    a, b = direct.clock_state(), replay.clock_state()
    assert (a.time, a.dt, a.iteration) == (b.time, b.dt, b.iteration)
    with pytest.raises(ValueError):
        replay.use_graph(0)


@pytest.mark.parametrize("dt_mode_name", ["DT_CFL", "DT_FORMULA"])
@pytest.mark.parametrize("steps", [1, 3])
def test_host_call_pinned_matches_pageable(md, dt_mode_name, steps):
    """mara_minidisk_advance_host with pinned host buffers (mixed RK2: the
    clock init reads the caller's state over the host link while copying it,
    and the last stage writes into the caller's output) gives the same bits
    and time as with pageable buffers (plain copies); the input is left
    alone, and an output that aliases the input works. FP64 takes the copy
    path in both cases."""
    from mara3p_gb300._capi import check, lib
    sd = md.SolverData(**dict(REFERENCE_DISK, block_size=64, depth=2, plm_theta=1.5))
    c = sd.to_c()
    N = sd.cells_per_side
    u0 = md.initial_conserved(sd, seed=3, amplitude=0.01).cpu()
    dt_mode = getattr(md, dt_mode_name)
    stream = torch.cuda.current_stream().cuda_stream
    for prec in (md.MIXED, md.FP64):
        ws = torch.empty(lib.mara_minidisk_host_workspace_bytes(ctypes.byref(c), 2, prec), dtype=torch.uint8,
                         device="cuda")
        outs = []
        for pinned, alias in ((False, False), (True, False), (True, True)):
            hin = torch.empty((3, N, N), dtype=torch.float64, pin_memory=pinned)
            hin.copy_(u0)
            hout = hin if alias else torch.full((3, N, N), float("nan"), dtype=torch.float64, pin_memory=pinned)
            t = ctypes.c_double()
            check(lib.mara_minidisk_advance_host(ctypes.byref(c), hin.data_ptr(), hout.data_ptr(), 0.5, steps, 2,
                                                 prec, dt_mode, ctypes.byref(t), ws.data_ptr(), stream))
            if not alias:
                assert torch.equal(hin, u0)
            outs.append((hout.clone(), t.value))
        assert torch.isfinite(outs[0][0]).all() and outs[0][1] > 0.5
        for u, t in outs[1:]:
            assert torch.equal(u, outs[0][0]), (prec, steps, dt_mode_name)
            assert t == outs[0][1]


@pytest.mark.parametrize("block_size,depth", [(64, 2), (100, 1), (80, 3)])
def test_sweep_launch_shapes_bit_identical(md, block_size, depth):
    """Every launch shape of the single-mesh sweep (warps per block, waves of
    strip segments, down to 16-row segments and ragged last segments) gives
    the same bits: the segments only change which warp computes a cell."""
    from mara3p_gb300._capi import lib
    sd = md.SolverData(**dict(REFERENCE_DISK, block_size=block_size, depth=depth, plm_theta=1.5))
    u0 = md.initial_conserved(sd, seed=9, amplitude=0.01)
    out = []
    try:
        for shape in ((0, 0), (4, 1), (1, 1), (2, 3), (1, 7), (4, 16)):
            assert lib.mara_minidisk_sweep_shape(*shape) == 0
            run = md.Run(sd, u0.clone(), rk_order=2, precision=md.MIXED, dt_mode=md.DT_CFL)
            run.advance(4)
            torch.cuda.synchronize()
            out.append((shape, run.u.clone(), run.clock_state()))
    finally:
        lib.mara_minidisk_sweep_shape(0, 0)
    (s0, u0r, k0) = out[0]
    assert torch.isfinite(u0r).all()
    for shape, u, k in out[1:]:
        assert torch.equal(u, u0r), shape
        assert (k.time, k.dt, k.iteration) == (k0.time, k0.dt, k0.iteration), shape
    for bad in ((3, 1), (8, 1), (-1, 0), (4, 17), (1, -2)):
        assert lib.mara_minidisk_sweep_shape(*bad) == -1


@pytest.mark.parametrize("block_size,depth", [(20, 2), (50, 1), (40, 3), (130, 0)])
def test_ragged_meshes_fp64_rk2_and_mixed(md, oracle, block_size, depth):
    """Meshes whose size is not a multiple of the 16 x 32 tiles or the 28/60
    column strips (80, 100, 320, 130): FP64 RK2 against the oracle, and the
    mixed path within its error budget of the FP64 path. 320 and 130 also
    contain TMA-loaded interior tiles next to wrapped boundary tiles."""
    sd = md.SolverData(**dict(REFERENCE_DISK, block_size=block_size, depth=depth, plm_theta=1.5))
    u0 = md.initial_conserved(sd, seed=4, amplitude=0.01)
    ref = u0.cpu().numpy().ravel().copy()
    a = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_FORMULA)
    a.advance(3)
    oracle.oracle_minidisk_advance(ctypes.byref(params(sd)), dptr(ref), ctypes.c_double(0.0), 3, 2, 0, 8)
    assert rel_l1_components(a.u.cpu().numpy(), ref) < FP64_ONE_STEP
    b = md.Run(sd, u0.clone(), rk_order=2, precision=md.MIXED, dt_mode=md.DT_FORMULA)
    b.advance(3)
    assert rel_l1_components(b.u.cpu().numpy(), a.u.cpu().numpy()) < 1e-6
