"""GPU parity of the spherical-track SRHD scheme (sedov2d) through the C ABI.

Against the reference's own sedov:: functions (tests/golden/sedov_golden.npz):
the primitives, radial slopes, radial Godunov data, polar faces and the
advanced state of one forward-Euler advance, and RK2 / RK3 runs of three
steps. Against the oracle (oracle/sedov_oracle.cpp, itself bit-identical to
the reference on the fixtures): larger track sets over many steps, a single
track, two-cell tracks, and a failing recovery.

Tolerances: the arithmetic is the reference's FP64 evaluation order; the
device's sin, cos, tan and pow differ from the host's by an ulp or two, which
enters the cell volumes and face areas: one advance 1e-12, three RK steps
1e-11 (relative L1 per array), twenty steps on 60 tracks 1e-9. Merge
indexes of the polar faces are exact.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import dptr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CASES = ["uniform_plm", "focused_swirl", "focused_pcm"]


@pytest.fixture(scope="module")
def sd():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import mara3p_gb300.sedov as s
    return s


@pytest.fixture(scope="module")
def sedov_golden():
    return dict(np.load(ROOT / "tests" / "golden" / "sedov_golden.npz"))


def rel_l1(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300)


def load(sd, g, name):
    k = lambda s: g[f"sedov/{name}/{s}"]  # noqa: E731
    T = int(k("T")[0])
    tr = sd.Tracks(k("ncells"), k("theta"), k("radii"), k("u"))
    return k, T, tr


@pytest.mark.parametrize("name", CASES)
def test_stage_parts_match_reference(sd, sedov_golden, name):
    k, T, tr = load(sd, sedov_golden, name)
    C, F = tr.cells, tr.cells + T
    gi, go = k("ghost_in")[:5 * T], k("ghost_out")[:5 * T]
    out = tr.stage(float(k("dt")[0]), gi, go, use_plm=bool(k("use_plm")[0]))
    assert tr.failure_count() == 0
    assert rel_l1(out["prim"].cpu().numpy().T, k("euler/prim").reshape(C, 5)) < 1e-12
    assert rel_l1(out["grad"].cpu().numpy().T, k("euler/grad").reshape(C, 5)) < 1e-12
    assert rel_l1(out["radial"].cpu().numpy().T, k("euler/radial").reshape(F, 6)) < 1e-12
    polar = k("euler/polar").reshape(-1, 8)
    NP = len(polar)
    assert tr.polar_offsets()[-1] == NP
    got = out["polar"].cpu().numpy()[:, :NP].T
    idx = out["polar_index"].cpu().numpy()[:, :NP].T
    # a transverse face is valid where both merge counters name a cell; zero-
    # length faces (tracks sharing a radius) are valid with zero area
    nc = k("ncells")
    iface = np.searchsorted(np.array(tr.polar_offsets()[:-1]), np.arange(NP), side="right") - 1
    nl, nr = nc[iface] + 1, nc[iface + 1] + 1
    valid = (idx[:, 0] >= 0) & (idx[:, 0] + 1 < nl) & (idx[:, 1] >= 0) & (idx[:, 1] + 1 < nr)
    assert np.array_equal(idx[valid, 0], polar[valid, 6]) and np.array_equal(idx[valid, 1], polar[valid, 7])
    assert np.all(polar[~valid] == 0.0) and np.all(got[~valid] == 0.0)
    assert rel_l1(got[valid, :5], polar[valid, :5]) < 1e-12
    assert rel_l1(got[:, 5], polar[:, 5]) < 1e-12
    assert rel_l1(got[:, :5] * got[:, 5:6], polar[:, :5] * polar[:, 5:6]) < 1e-12
    assert rel_l1(out["radii"].cpu().numpy(), k("euler/radii")) < 1e-14
    assert rel_l1(out["u"].cpu().numpy().T, k("euler/u").reshape(C, 5)) < 1e-12
    # stage leaves its input alone
    assert torch.equal(tr.radii.cpu(), torch.from_numpy(k("radii")))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("rk", [1, 2, 3])
def test_rk_runs_match_reference(sd, sedov_golden, oracle, name, rk):
    k, T, tr = load(sd, sedov_golden, name)
    dt, plm = float(k("dt")[0]), bool(k("use_plm")[0])
    for _ in range(3):
        tr.advance(dt, k("ghost_in"), k("ghost_out"), rk_order=rk, use_plm=plm)
    radii, u = tr.host_state()
    if rk == 1:
        # the reference fixtures hold RK2 and RK3; RK1 runs against the oracle
        ref_r, ref_u = k("radii").copy(), k("u").copy()
        nc = np.ascontiguousarray(k("ncells"), dtype=np.int64)
        for _ in range(3):
            assert oracle.oracle_sedov_advance_rk(ctypes.c_int32(T), nc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                                  dptr(k("theta")), dptr(ref_r), dptr(ref_u), dptr(k("ghost_in")),
                                                  dptr(k("ghost_out")), ctypes.c_double(dt), ctypes.c_int32(1),
                                                  ctypes.c_int32(int(plm))) == 0
    else:
        ref_r, ref_u = k(f"rk{rk}_3/radii"), k(f"rk{rk}_3/u")
    assert tr.failure_count() == 0
    assert rel_l1(radii, ref_r) < 1e-13
    assert rel_l1(u, ref_u.reshape(-1, 5)) < 1e-11


def make_tracks(sd, oracle, T, aspect, r1, seed, u3=0.0, focus=0.3):
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, T + 1)
    theta = np.pi * (x + focus * (x - 1) * x) / (1 + 2 * focus * (x - 1) * x)
    radii, ncells, cons = [], [], []
    oracle.oracle_sedov_cell_volume.restype = ctypes.c_double
    for j in range(T):
        rf = sd.generate_radial_track(1.0, r1, theta[j], theta[j + 1], aspect)
        n = len(rf) - 1
        rc = 0.5 * (rf[:-1] + rf[1:])
        pr = np.zeros((n, 5))
        pr[:, 0] = rc ** -2 * (1 + 0.05 * rng.uniform(-1, 1, n))
        pr[:, 1] = 0.4 + 0.05 * rng.uniform(-1, 1, n)
        pr[:, 2] = 0.02 * rng.uniform(-1, 1, n)
        pr[:, 3] = u3 * rng.uniform(-1, 1, n)
        pr[:, 4] = 1e-3 * pr[:, 0] + np.where(rc < 1.5, 0.3, 0.0)
        uc = np.zeros(5 * n)
        oracle.oracle_srhd_conserved_density(dptr(np.ascontiguousarray(pr.ravel())), ctypes.c_int64(n),
                                             ctypes.c_double(4.0 / 3.0), dptr(uc))
        dv = np.array([oracle.oracle_sedov_cell_volume(ctypes.c_double(rf[i]), ctypes.c_double(rf[i + 1]),
                                                       ctypes.c_double(theta[j]), ctypes.c_double(theta[j + 1]))
                       for i in range(n)])
        radii.append(rf)
        ncells.append(n)
        cons.append((uc.reshape(n, 5) * dv[:, None]).ravel())
    th = np.repeat(theta, 2)[1:-1].copy()
    gin = np.tile([2.0, 0.8, 0.0, 0.0, 0.1], (3, T, 1)).ravel()
    gout = np.tile([0.01, 0.1, 0.0, 0.0, 1e-4], (3, T, 1)).ravel()
    return np.array(ncells, np.int64), th, np.concatenate(radii), np.concatenate(cons), gin, gout


def oracle_run(oracle, ncells, th, radii, u, gin, gout, dt, rk, plm, steps):
    r, uu = radii.copy(), u.copy()
    T = len(ncells)
    for _ in range(steps):
        rc = oracle.oracle_sedov_advance_rk(ctypes.c_int32(T), ncells.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                            dptr(th), dptr(r), dptr(uu), dptr(gin), dptr(gout), ctypes.c_double(dt),
                                            ctypes.c_int32(rk), ctypes.c_int32(int(plm)))
        assert rc == 0
    return r, uu


@pytest.mark.parametrize("u3", [0.0, 0.03])
def test_many_tracks_many_steps_match_oracle(sd, oracle, u3):
    ncells, th, radii, u, gin, gout = make_tracks(sd, oracle, 60, 0.25, 4.0, 7, u3=u3)
    tr = sd.Tracks(ncells, th, radii, u)
    dt = 0.3 * tr.min_spacing()
    assert dt == pytest.approx(0.3 * min(np.diff(radii[o:o + n + 1]).min()
                                         for o, n in zip(np.concatenate([[0], np.cumsum(ncells + 1)[:-1]]), ncells)),
                               rel=0, abs=0)
    for _ in range(20):
        tr.advance(dt, gin, gout, rk_order=2)
    r_ref, u_ref = oracle_run(oracle, ncells, th, radii, u, gin, gout, dt, 2, True, 20)
    r_gpu, u_gpu = tr.host_state()
    assert tr.failure_count() == 0
    assert rel_l1(r_gpu, r_ref) < 1e-12
    assert rel_l1(u_gpu, u_ref.reshape(-1, 5)) < 1e-9


@pytest.mark.parametrize("T,aspect", [(1, 0.1), (3, 0.9)])
def test_single_track_and_short_tracks(sd, oracle, T, aspect):
    # one track: no transverse faces; aspect 0.9 on 3 tracks: 2-cell tracks
    ncells, th, radii, u, gin, gout = make_tracks(sd, oracle, T, aspect, 3.0, 3, focus=0.0)
    assert ncells.min() >= 2
    tr = sd.Tracks(ncells, th, radii, u)
    dt = 0.2 * tr.min_spacing()
    for _ in range(3):
        tr.advance(dt, gin, gout, rk_order=3)
    r_ref, u_ref = oracle_run(oracle, ncells, th, radii, u, gin, gout, dt, 3, True, 3)
    r_gpu, u_gpu = tr.host_state()
    assert rel_l1(r_gpu, r_ref) < 1e-13
    assert rel_l1(u_gpu, u_ref.reshape(-1, 5)) < 1e-11


def test_failed_recovery_is_counted(sd, oracle):
    # a cell whose energy is far below its rest mass: the reference's recovery
    # throws; the GPU counts the failure and carries on
    ncells, th, radii, u, gin, gout = make_tracks(sd, oracle, 4, 0.5, 3.0, 5)
    u = u.copy()
    D = u[5 * 3]
    u[5 * 3 + 1: 5 * 3 + 5] = [0.5 * D, 0.0, 0.0, -0.5 * D]   # Newton does not converge
    r_out, u_out = np.zeros_like(radii), np.zeros_like(u)
    assert oracle.oracle_sedov_advance(ctypes.c_int32(4), ncells.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                       dptr(th), dptr(radii), dptr(u), dptr(gin), dptr(gout), ctypes.c_double(1e-3),
                                       ctypes.c_int32(1), dptr(r_out), dptr(u_out), None, None, None, None) == 1
    tr = sd.Tracks(ncells, th, radii, u)
    tr.advance(1e-3, gin, gout)
    assert tr.failure_count() >= 1


def test_bad_arguments(sd):
    from mara3p_gb300._capi import MaraError, lib
    with pytest.raises(ValueError):
        sd.Tracks([1, 3], [[0, 1], [1, 2]], np.ones(6), np.ones(20))
    assert lib.mara_sedov_workspace_bytes(0, 10) < 0
    tr = sd.Tracks([2, 2], [0.0, 1.5, 1.5, np.pi], np.tile([1.0, 1.5, 2.0], 2), np.ones(20))
    with pytest.raises(MaraError, match="rk_order"):
        tr.advance(1e-3, np.zeros(40), np.zeros(40), rk_order=4)


def oracle_remesh_all(oracle, ncells, th, radii, u, amax, amin, inner):
    """sedov::remesh of every track through the oracle; new (ncells, radii, u)."""
    oracle.oracle_sedov_remesh.restype = ctypes.c_int64
    out_n, out_r, out_u = [], [], []
    fo = np.concatenate([[0], np.cumsum(ncells + 1)])
    co = np.concatenate([[0], np.cumsum(ncells)])
    for j, n in enumerate(ncells):
        rf = np.zeros(n + 2)
        rf[:n + 1] = radii[fo[j]:fo[j + 1]]
        uc = np.zeros(5 * (n + 1))
        uc[:5 * n] = u[5 * co[j]:5 * co[j + 1]]
        m = oracle.oracle_sedov_remesh(ctypes.c_int64(n), ctypes.c_double(th[2 * j]), ctypes.c_double(th[2 * j + 1]),
                                       dptr(rf), dptr(uc), ctypes.c_double(amax), ctypes.c_double(amin),
                                       ctypes.c_double(inner))
        assert m > 0
        out_n.append(m)
        out_r.append(rf[:m + 1])
        out_u.append(uc[:5 * m])
    return np.array(out_n, np.int64), np.concatenate(out_r), np.concatenate(out_u)


def test_remesh_matches_reference_fixtures(sd, sedov_golden):
    names = sorted({k.split("/")[1] for k in sedov_golden if k.startswith("remesh/")})
    for nm in names:
        k = lambda s: sedov_golden[f"remesh/{nm}/{s}"]  # noqa: E731
        rf, u = k("radii"), k("u")
        amax, amin, inner, t0, t1 = k("bounds")
        tr = sd.Tracks([len(rf) - 1], [t0, t1], rf, u)
        m = tr.remesh(amax, amin, inner)
        assert m == int(k("cells_out")[0]), nm
        radii, uu = tr.host_state()
        assert np.array_equal(radii, k("radii_out")), nm
        assert np.array_equal(uu.ravel(), k("u_out")), nm
        assert tr.failure_count() == 0


def test_remesh_many_tracks_match_oracle(sd, oracle):
    ncells, th, radii, u, gin, gout = make_tracks(sd, oracle, 40, 0.5, 3.0, 12)
    rng = np.random.default_rng(3)
    fo = np.concatenate([[0], np.cumsum(ncells + 1)])
    radii = radii.copy()
    for j in range(40):
        # squeeze or stretch one interior face of most tracks
        n = ncells[j]
        if j % 5 == 4:
            continue
        f = fo[j] + rng.integers(2, n - 1)
        lo, hi = radii[f - 1], radii[f + 1]
        radii[f] = lo + (hi - lo) * rng.choice([0.03, 0.97, 0.5])
    tr = sd.Tracks(ncells, th, radii, u)
    m = tr.remesh(2.0, 0.5, 1.0)
    ref_n, ref_r, ref_u = oracle_remesh_all(oracle, ncells, th, radii, u, 2.0, 0.5, 1.0)
    assert m == ref_n.sum()
    assert np.array_equal(tr.ncells, ref_n)
    r_gpu, u_gpu = tr.host_state()
    assert np.array_equal(r_gpu, ref_r) and np.array_equal(u_gpu.ravel(), ref_u)


def test_advance_and_remesh_loop_matches_oracle(sd, oracle):
    """The driver's loop (problems/sedov2d.cpp:700-712): an RK2 advance, then
    remesh of every track, for 15 steps; tracks change length as their faces
    move."""
    ncells, th, radii, u, gin, gout = make_tracks(sd, oracle, 24, 0.4, 3.0, 21)
    tr = sd.Tracks(ncells, th, radii, u)
    dt = 0.3 * tr.min_spacing()
    nc, rr, uu = ncells.copy(), radii.copy(), u.copy()
    for _ in range(15):
        tr.advance(dt, gin, gout, rk_order=2)
        tr.remesh(2.0, 0.5, 1.0)
        rr, uu = oracle_run(oracle, nc, th, rr, uu, gin, gout, dt, 2, True, 1)
        nc, rr, uu = oracle_remesh_all(oracle, nc, th, rr, uu, 2.0, 0.5, 1.0)
        assert np.array_equal(tr.ncells, nc)
    r_gpu, u_gpu = tr.host_state()
    assert tr.failure_count() == 0
    assert rel_l1(r_gpu, rr) < 1e-12
    assert rel_l1(u_gpu, uu.reshape(-1, 5)) < 1e-9
    assert nc.sum() != ncells.sum() or not np.array_equal(nc, ncells)   # the loop did remesh
