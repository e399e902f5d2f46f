"""GPU parity of the 2D SRHD shock-tube scheme against the oracle (which
composes the reference's pinned srhd recovery, HLLE/HLLC and PLM), the
pointwise Riemann solvers against the reference's golden fluxes, and the
effect of the learned / warm-start pressure guesses on the FP64 Newton work.

Tolerances: FP64 relative L1 per component <= 1e-12 after one RK2 step,
<= 1e-10 after 20; mixed (FP32 fluxes, FP64 state and recovery) <= 1e-5;
seeded recoveries change the state by no more than the Newton stopping rule
allows (<= 1e-9 after 10 steps)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle.oracle import dptr
from tests.helpers import rel_l1_components

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
G = 4.0 / 3.0


@pytest.fixture(scope="module")
def sr():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import mara3p_gb300.srhd as s
    return s


def oracle_run(oracle, N, steps, floor=1e-10, hllc=0):
    oracle.oracle_srhd_tube_advance_solver.restype = ctypes.c_double
    u = np.zeros(4 * N * N)
    oracle.oracle_srhd_tube_initial(N, ctypes.c_double(np.pi / 6), ctypes.c_double(10.0), ctypes.c_double(13.33),
                                    ctypes.c_double(1.0), ctypes.c_double(1e-6), ctypes.c_double(G), dptr(u))
    fails, rejected = ctypes.c_int64(0), ctypes.c_int64(0)
    t = oracle.oracle_srhd_tube_advance_solver(N, dptr(u), ctypes.c_double(0.0), steps, ctypes.c_double(0.3),
                                               ctypes.c_double(1.5), ctypes.c_double(G), ctypes.c_double(floor), hllc,
                                               ctypes.byref(fails), ctypes.byref(rejected))
    return u.reshape(4, -1), t, fails.value


@pytest.mark.parametrize("riemann", ["hlle", "hllc"])
@pytest.mark.parametrize("steps,tol", [(1, 1e-12), (20, 1e-10)])
def test_fp64_matches_oracle(sr, oracle, steps, tol, riemann):
    N = 64
    tube = sr.ShockTube(N=N)
    tube.advance(steps, riemann=riemann)
    ref, t, fails = oracle_run(oracle, N, steps, hllc=int(riemann == "hllc"))
    c = tube.clock_state()
    assert fails == 0 and c["failures"] == 0
    assert c["riemann_rejected"] == 0
    assert abs(c["time"] - t) <= 1e-14 * t
    assert rel_l1_components(tube.u.cpu().numpy().reshape(4, -1), ref, 4) < tol


@pytest.mark.parametrize("solver", ["hlle", "hllc"])
@pytest.mark.parametrize("axis", [1, 2, 3])
def test_pointwise_riemann_matches_reference_golden(sr, srhd_golden, solver, axis):
    """mara_srhd_riemann reproduces the reference's riemann_solver fluxes
    (tests/golden, made by the reference's own code) bit for bit."""
    pl = torch.from_numpy(srhd_golden["srhd_riemann/pl"].reshape(-1, 5)).cuda()
    pr = torch.from_numpy(srhd_golden["srhd_riemann/pr"].reshape(-1, 5)).cuda()
    f, status = sr.riemann(pl, pr, axis, G, solver)
    assert int(status.sum()) == 0
    ref = srhd_golden[f"srhd_riemann/{solver}/axis{axis}"].reshape(-1, 5)
    assert np.array_equal(f.cpu().numpy(), ref)


def test_pointwise_riemann_edge_cases(sr, oracle):
    """Supersonic faces (either side), a state at rest against vacuum-like
    pressure, and mirrored states; HLLE and HLLC against the oracle."""
    pl = np.array([[1.0, 5.0, 0.0, 0.0, 1.0], [1.0, -5.0, 0.0, 0.0, 1.0], [10.0, 0.0, 0.0, 0.0, 13.33],
                   [1.0, 0.3, -0.2, 0.1, 1.0], [1e-4, 2.0, 1.0, 0.5, 1e-6]])
    pr = np.array([[1.0, 5.0, 0.0, 0.0, 1.0], [1.0, -5.0, 0.0, 0.0, 1.0], [1.0, 0.0, 0.0, 0.0, 1e-6],
                   [1.0, -0.3, 0.2, -0.1, 1.0], [1e-3, -1.0, 0.5, 0.0, 1e-5]])
    for solver in ("hlle", "hllc"):
        for axis in (1, 2, 3):
            f, status = sr.riemann(torch.from_numpy(pl).cuda(), torch.from_numpy(pr).cuda(), axis, G, solver)
            ref = np.zeros_like(pl)
            bad = oracle.oracle_srhd_riemann(dptr(np.ascontiguousarray(pl)), dptr(np.ascontiguousarray(pr)),
                                             ctypes.c_int64(len(pl)), axis, ctypes.c_double(G),
                                             int(solver == "hllc"), dptr(ref))
            assert int(status.sum()) == bad
            ok = status.cpu().numpy() == 0
            assert np.array_equal(f.cpu().numpy()[ok], ref[ok]), (solver, axis)


def test_initial_state_matches_oracle(sr, oracle):
    N = 64
    tube = sr.ShockTube(N=N)
    ref, _, _ = oracle_run(oracle, N, 0)
    assert np.array_equal(tube.u.cpu().numpy().reshape(4, -1), ref)


def test_mixed_close_to_fp64(sr):
    a, b = sr.ShockTube(N=64), sr.ShockTube(N=64)
    a.advance(20)
    b.advance(20, precision=1)
    assert b.clock_state()["failures"] == 0
    assert rel_l1_components(b.u.cpu().numpy().reshape(4, -1), a.u.cpu().numpy().reshape(4, -1), 4) < 1e-5


@pytest.fixture(scope="module")
def net(sr, oracle):
    from tests.test_srhd_gpu import seeded_zones
    _, cons = seeded_zones(oracle, 1 << 17, seed=99)
    c = torch.from_numpy(cons.reshape(-1, 5).T.copy()).cuda()
    rec = sr.recover_primitive(c, G)
    m = sr.PressureGuess()
    m.prepare(c, rec.prim, seed=2)
    m.train(steps=1500, batch=8192, lr=2e-3, seed=2)
    return m


def test_seeded_recoveries_keep_the_state_and_cut_newton_work(sr, net):
    N = 128
    base = sr.ShockTube(N=N)
    learned = sr.ShockTube(N=N)
    warm = sr.ShockTube(N=N)
    base.advance(10)
    learned.advance(10, guess=sr.GUESS_MLP, mlp=net, refine32=2)
    warm.advance(10, guess=sr.GUESS_PREVIOUS)
    ub = base.u.cpu().numpy().reshape(4, -1)
    for other in (learned, warm):
        assert other.clock_state()["failures"] == 0
        assert rel_l1_components(other.u.cpu().numpy().reshape(4, -1), ub, 4) < 1e-9
    # in the tube most cells are at rest, where the reference's start already
    # converges in two iterations; both guesses still cut the Newton work
    nb, nl, nw = (t.clock_state()["newton"] for t in (base, learned, warm))
    assert nl < nb, (nb, nl)
    assert nw < nb, (nb, nw)
