"""Minidisk time series: the rate vector (sink, buffer and gravity sums, disk
mass and angular momentum, torques, power), its time integrals, and the
binary's orbital elements and their implied rates.

CPU: mara_two_body_elements against the reference's own
recover_orbital_elements (tests/golden/two_body_golden.npz) and its
known-answer test (src/physics_two_body.hpp:477-490); element rates against
the analytic rate of a tangential force; the oracle's rate vector against the
mass balance of the reference's own substep.

GPU: the FP64 reduction (standalone kernel) and the sums fused into the mixed
sweep kernels against the oracle; integrals, RK weights and mass balance of
whole runs; diagnostics leave the state bit-identical.

Tolerances: FP64 sums differ from the oracle only in summation order
(1e-10 of the entry's group scale); the mixed path sums FP32 per-cell
contributions of the FP32 state (2e-5 of the group scale).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import MinidiskParams, dptr
from tests.helpers import params_from_vector

ROOT = Path(__file__).resolve().parents[1]
# entries compared on one scale: sink mass, sink momentum, forces, buffer,
# disk mass, angular momentum; torques and power (sums of products of the
# forces with the binary's positions and velocities, which cancel) on the
# force scale
GROUPS = [(0, 2), (2, 6), (6, 10), (10, 11), (11, 12), (12, 13), (13, 16)]


@pytest.fixture(scope="module")
def two_body():
    return dict(np.load(ROOT / "tests" / "golden" / "two_body_golden.npz"))


@pytest.fixture(scope="module")
def mdh():
    """The host-only part of the minidisk API (no GPU needed)."""
    import mara3p_gb300.minidisk as m
    return m


def close_by_group(got, ref, tol):
    got, ref = np.asarray(got), np.asarray(ref)
    for a, b in GROUPS:
        scale = np.abs(ref[6:10]).max() if a == 13 else np.abs(ref[a:b]).max()
        assert np.abs(got[a:b] - ref[a:b]).max() <= tol * scale, (a, b, got[a:b], ref[a:b])


# ---------------------------------------------------------------- CPU
def test_elements_match_reference(mdh, two_body):
    from mara3p_gb300._capi import MaraError
    for st, t, ref, status in zip(two_body["two_body/state"], two_body["two_body/t"],
                                  two_body["two_body/recovered"], two_body["two_body/status"]):
        if status:
            with pytest.raises(MaraError, match="not a bound orbit"):
                mdh.two_body_elements(list(st), float(t))
            continue
        got = np.array(list(mdh.two_body_elements(list(st), float(t)).values()))
        assert np.array_equal(got, ref)


def test_elements_known_answer(mdh, two_body):
    # test_two_body: elements (1, 1, 1, 0.5) at t = 0 recover e and a to 1e-10
    states = two_body["two_body/state"]
    el = two_body["two_body/elements"]
    # on-orbit states come first for each (elements, time) pair: index 2 * (row * len(times) + time)
    nt = len(two_body["two_body/times"])
    st = states[2 * (1 * nt + 0)]
    got = mdh.two_body_elements(list(st), 0.0)
    assert abs(got["e"] - el[1, 3]) < 1e-10 and abs(got["a"] - el[1, 0]) < 1e-10


def test_element_rates_of_a_tangential_force(mdh):
    # circular equal-mass binary (a = M = 1): forces f along each velocity do
    # work P = f (|v1| + |v2|); a = -M1 M2 / 2E gives da/dt = 2 a^2 P / (M1 M2)
    sd = mdh.SolverData(omega_frame=0.0, mass_ratio=1.0, eccentricity=0.0)
    st = mdh.binary_state(sd, 0.3)
    f = 1e-4
    rate = [0.0] * 16
    for k in range(2):
        vx, vy = st[5 * k + 3], st[5 * k + 4]
        v = np.hypot(vx, vy)
        rate[6 + 2 * k] = f * vx / v
        rate[7 + 2 * k] = f * vy / v
    P = f * (np.hypot(st[3], st[4]) + np.hypot(st[8], st[9]))
    got = mdh.element_rates(st, 0.3, rate)
    assert got["a"] == pytest.approx(2.0 * P / (0.5 * 0.5), rel=1e-6)
    assert abs(got["M"]) < 1e-12 and abs(got["q"]) < 1e-12
    assert mdh.element_rates(st, 0.3, [0.0] * 16) == {"a": 0.0, "M": 0.0, "q": 0.0, "e": 0.0}


def test_element_rates_of_accretion(mdh):
    # accretion onto body 2 only, at rest relative to it: M and q grow
    sd = mdh.SolverData(omega_frame=0.0, mass_ratio=0.5, eccentricity=0.2)
    st = mdh.binary_state(sd, 1.1)
    rate = [0.0] * 16
    rate[1] = 1e-3
    rate[4], rate[5] = 1e-3 * st[8], 1e-3 * st[9]   # accreted momentum = mass rate * body velocity
    got = mdh.element_rates(st, 1.1, rate)
    m1, m2 = st[0], st[5]
    assert got["M"] == pytest.approx(1e-3, rel=1e-6)
    assert got["q"] == pytest.approx(1e-3 / m1, rel=1e-6)


@pytest.mark.parametrize("case", ["config1_like", "eccentric_unequal", "inviscid_defaults"])
def test_oracle_rates_balance_the_reference_mass_change(oracle, golden, case):
    # periodic mesh: fluxes cancel in the mesh total, so one reference substep
    # changes the disk mass by dt * (buffer - sink 1 - sink 2)
    p = params_from_vector(golden[f"{case}/params"], float(golden[f"{case}/theta"][0]))
    N = p.block_size << p.depth
    dl = 2.0 * p.domain_radius / N
    t, dt = golden[f"{case}/t"]
    u0 = np.ascontiguousarray(golden[f"{case}/u0"])
    r = np.zeros(16)
    oracle.oracle_minidisk_rates(ctypes.byref(p), dptr(u0), ctypes.c_double(t), dptr(r))
    u1 = golden[f"{case}/substep"].reshape(3, N, N)
    dm = (u1[0] - u0.reshape(3, N, N)[0]).sum() * dl * dl / dt
    expected = r[10] - r[0] - r[1]
    assert abs(dm - expected) <= 1e-9 * (abs(r[10]) + abs(r[0]) + abs(r[1])) + 1e-12 * r[11] / dt
    assert r[11] == pytest.approx((u0.reshape(3, N, N)[0]).sum() * dl * dl, rel=1e-13)


# ---------------------------------------------------------------- GPU
torch = pytest.importorskip("torch")

RUN_PARAMS = dict(block_size=32, depth=2, omega_frame=1.0, mach_number=10.0, nu=1e-3, domain_radius=2.0,
                  softening_length=0.05, eccentricity=0.2, mass_ratio=0.5, sink_radius=0.05, sink_rate=10.0,
                  buffer_rate=100.0, buffer_scale=0.2, cfl=0.3, plm_theta=2.0)


@pytest.fixture(scope="module")
def md():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import mara3p_gb300.minidisk as m
    return m


def seeded(md, oracle, p, seed=11, amp=0.05):
    N = p.block_size << p.depth
    u = np.zeros(3 * N * N)
    oracle.oracle_minidisk_initial_conserved(ctypes.byref(p), ctypes.c_uint64(seed), ctypes.c_double(amp), dptr(u))
    return u


def oracle_rates(oracle, p, u, t):
    r = np.zeros(16)
    oracle.oracle_minidisk_rates(ctypes.byref(p), dptr(np.ascontiguousarray(u)), ctypes.c_double(t), dptr(r))
    return r


def sd_of(md, p):
    return md.SolverData(**{name: getattr(p, name) for name, _ in p._fields_})


@pytest.mark.gpu
@pytest.mark.parametrize("t", [0.0, 0.83])
def test_fp64_rates_match_oracle(md, oracle, t):
    p = MinidiskParams(**RUN_PARAMS)
    u = seeded(md, oracle, p)
    N = p.block_size << p.depth
    got = md.rates(sd_of(md, p), torch.from_numpy(u.reshape(3, N, N)).cuda(), t)
    close_by_group([got[k] for k in md.DIAG_NAMES], oracle_rates(oracle, p, u, t), 1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("rk_order", [1, 2])
def test_fp64_run_diagnostics(md, oracle, rk_order):
    p = MinidiskParams(**RUN_PARAMS)
    sd = sd_of(md, p)
    N = p.block_size << p.depth
    u0 = seeded(md, oracle, p)
    plain = md.Run(sd, torch.from_numpy(u0.reshape(3, N, N)).cuda(), rk_order=rk_order)
    run = md.Run(sd, torch.from_numpy(u0.reshape(3, N, N)).cuda(), rk_order=rk_order, diagnostics=True)
    plain.advance(1)
    run.advance(1)
    assert torch.equal(plain.u, run.u)
    d = run.diagnostics()
    dt = run.clock_state().dt
    assert d["steps"] == 1
    r0 = np.array([d["rate"][0][k] for k in md.DIAG_NAMES])
    close_by_group(r0, oracle_rates(oracle, p, u0, 0.0), 1e-10)
    if rk_order == 2:
        # stage 2 sees the forward-Euler state at t + dt
        u1 = np.zeros_like(u0)
        oracle.oracle_minidisk_substep(ctypes.byref(p), dptr(u0), dptr(u1), ctypes.c_double(0.0), ctypes.c_double(dt), 4)
        r1 = np.array([d["rate"][1][k] for k in md.DIAG_NAMES])
        close_by_group(r1, oracle_rates(oracle, p, u1, dt), 1e-10)
        expected = dt * (0.5 * (r0 + r1))
    else:
        expected = dt * r0
    integral = np.array([d["integral"][k] for k in md.DIAG_NAMES])
    keep = [k for k in range(16) if k not in (11, 12)]
    assert np.allclose(integral[keep], expected[keep], rtol=1e-14, atol=0.0)
    assert integral[11] == r0[11] and integral[12] == r0[12]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mass_balance_over_many_steps(md, oracle, precision):
    p = MinidiskParams(**RUN_PARAMS)
    sd = sd_of(md, p)
    N = p.block_size << p.depth
    dl = 2.0 * p.domain_radius / N
    u0 = seeded(md, oracle, p)
    run = md.Run(sd, torch.from_numpy(u0.reshape(3, N, N)).cuda(), rk_order=2,
                 precision=md.FP64 if precision == "fp64" else md.MIXED, diagnostics=True)
    for _ in range(4):
        run.advance(10)
    d = run.diagnostics()
    assert d["steps"] == 40
    I = d["integral"]
    dm = (run.u[0].sum().item() - u0.reshape(3, N, N)[0].sum()) * dl * dl
    expected = I["buffer_mass"] - I["sink_mass_1"] - I["sink_mass_2"]
    scale = abs(I["buffer_mass"]) + abs(I["sink_mass_1"]) + abs(I["sink_mass_2"])
    # FP64: the update's own sources; mixed: FP32 sums of FP32 increments
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert abs(dm - expected) <= tol * scale + 1e-13 * I["disk_mass"]


@pytest.mark.gpu
@pytest.mark.parametrize("columns", [1, 2])
def test_mixed_fused_sums_match_oracle(md, oracle, columns):
    p = MinidiskParams(**dict(RUN_PARAMS, block_size=64))   # 256^2: the sweep kernels
    sd = sd_of(md, p)
    N = p.block_size << p.depth
    u0 = seeded(md, oracle, p)
    prev = md.lib.mara_minidisk_sweep_columns(columns)
    try:
        plain = md.Run(sd, torch.from_numpy(u0.reshape(3, N, N)).cuda(), precision=md.MIXED)
        run = md.Run(sd, torch.from_numpy(u0.reshape(3, N, N)).cuda(), precision=md.MIXED, diagnostics=True)
        plain.advance(1)
        run.advance(1)
    finally:
        md.lib.mara_minidisk_sweep_columns(prev)
    assert torch.equal(plain.u, run.u)
    d = run.diagnostics()
    r0 = np.array([d["rate"][0][k] for k in md.DIAG_NAMES])
    close_by_group(r0, oracle_rates(oracle, p, u0, 0.0), 2e-5)
    dt = run.clock_state().dt
    u1 = np.zeros_like(u0)
    oracle.oracle_minidisk_substep(ctypes.byref(p), dptr(u0), dptr(u1), ctypes.c_double(0.0), ctypes.c_double(dt), 4)
    r1 = np.array([d["rate"][1][k] for k in md.DIAG_NAMES])
    close_by_group(r1, oracle_rates(oracle, p, u1, dt), 2e-5)


@pytest.mark.gpu
def test_reset_and_accumulation_across_calls(md, oracle):
    p = MinidiskParams(**RUN_PARAMS)
    sd = sd_of(md, p)
    N = p.block_size << p.depth
    u0 = seeded(md, oracle, p)
    a = md.Run(sd, torch.from_numpy(u0.reshape(3, N, N)).cuda(), diagnostics=True)
    b = md.Run(sd, torch.from_numpy(u0.reshape(3, N, N)).cuda(), diagnostics=True)
    a.advance(6)
    for _ in range(3):
        b.advance(2)
    da, db = a.diagnostics(), b.diagnostics()
    assert da["steps"] == db["steps"] == 6
    for k in md.DIAG_NAMES:
        assert da["integral"][k] == pytest.approx(db["integral"][k], rel=1e-13, abs=1e-300)
    b.reset_diagnostics()
    assert b.diagnostics()["steps"] == 0 and all(v == 0.0 for v in b.diagnostics()["integral"].values())
