"""The sedov driver's safety mode (problems/sedov2d.cpp:697-741) around the
GPU tracks: failure handling on the host, tested on the CPU with scripted
failures and on the GPU with a state poisoned on the host."""
from __future__ import annotations

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")


class ScriptedTracks:
    """Stands in for sedov.Tracks on the CPU: the state is a number that each
    advance increases by dt; advances whose (1-based) attempt number is in
    `fail` report one failed zone."""

    def __init__(self, fail=()):
        self.state, self.attempt, self.fail, self.calls, self.f, self.remeshes = 0.0, 0, set(fail), [], 0, 0

    def min_spacing(self):
        return 1.0

    def snapshot(self):
        return {"state": self.state}

    def restore(self, snap):
        self.state = snap["state"]

    def reset_failures(self):
        self.f = 0

    def advance(self, dt, ghost_in, ghost_out, rk_order, use_plm):
        self.attempt += 1
        self.calls.append((dt, use_plm))
        self.state += dt
        self.f = 1 if self.attempt in self.fail else 0

    def remesh(self, *args):
        self.remeshes += 1

    def failure_count(self):
        return self.f


def driver(tracks):
    from mara3p_gb300 import sedov
    return sedov.Driver(tracks, lambda t: (None, None), cfl=0.5)


def test_steps_without_failures():
    tr = ScriptedTracks()
    d = driver(tr)
    for _ in range(3):
        assert not d.step()["rolled_back"]
    assert d.iteration == 3 and d.time == pytest.approx(1.5) and tr.remeshes == 3
    assert all(use_plm for _, use_plm in tr.calls)


def test_failure_rolls_back_to_the_backup_and_retries_in_safety_mode():
    tr = ScriptedTracks(fail={3})
    d = driver(tr)
    d.step(); d.step()                      # iterations 1, 2
    r = d.step()                            # fails at iteration 2
    assert r["rolled_back"] and d.safety
    assert d.iteration == 1 and tr.state == pytest.approx(0.5)   # the state before the last successful step
    r = d.step()                            # safety mode: dt x 1e-3, PLM off
    assert r["safety"] and not r["rolled_back"] and d.iteration == 2 and not d.safety
    assert tr.calls[-1] == (pytest.approx(0.5e-3), False)
    assert tr.remeshes == 3                 # the failed advance skipped its remesh
    d.step()
    assert d.iteration == 3 and tr.calls[-1] == (0.5, True)


def test_second_failure_at_the_same_iteration_is_final():
    from mara3p_gb300._capi import MaraError
    tr = ScriptedTracks(fail={3, 5})
    d = driver(tr)
    d.step(); d.step(); d.step(); d.step()  # success, success, fail at 2 -> back to 1, safety success -> 2
    before = tr.state
    with pytest.raises(MaraError, match="cannot be retried"):
        d.step()                            # fails at iteration 2 again
    assert tr.state == before and d.iteration == 2


def test_failed_safety_step_retries_once_more_then_raises():
    from mara3p_gb300._capi import MaraError
    tr = ScriptedTracks(fail={3, 4, 5})
    d = driver(tr)
    d.step(); d.step()
    assert d.step()["rolled_back"]          # iteration 2 fails -> iteration 1
    assert d.step()["rolled_back"]          # the safety step from 1 fails: 1 is not the last failed iteration
    assert d.iteration == 1 and d.safety
    with pytest.raises(MaraError):
        d.step()                            # fails at iteration 1 again


def test_failure_at_iteration_zero_is_final():
    from mara3p_gb300._capi import MaraError
    tr = ScriptedTracks(fail={1})
    d = driver(tr)
    with pytest.raises(MaraError):
        d.step()
    assert tr.state == 0.0 and d.iteration == 0


def wind(T, r):
    return np.tile([r ** -2, 0.4, 0.0, 0.0, 1e-3 * r ** -2], (1, T, 1))


@pytest.mark.gpu
def test_gpu_driver_recovers_from_a_poisoned_state():
    """Two steps, then one cell's energy is set to NaN on the host: that step
    fails (the recovery counts it where the reference throws), the driver
    restores the state before the previous step and redoes it in safety
    mode, and the run goes on without failures."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mara3p_gb300 import sedov
    ncells, theta, radii, u = sedov.seeded_tracks(48, seed=5)
    tr = sedov.Tracks(ncells, theta, radii, u)
    T = tr.T
    d = sedov.Driver(tr, lambda t: (wind(T, 1.0), wind(T, 1.8)), cfl=0.5)
    assert not d.step()["rolled_back"]
    assert not d.step()["rolled_back"]
    dt_normal = 0.5 * tr.min_spacing()
    tr.u[4, tr.cells // 2] = math.nan
    r = d.step()
    assert r["rolled_back"] and r["failures"] > 0 and d.iteration == 1 and d.safety
    r = d.step()
    assert r["safety"] and not r["rolled_back"] and d.iteration == 2
    assert r["dt"] == pytest.approx(1e-3 * dt_normal, rel=0.05)
    for _ in range(3):
        assert not d.step()["rolled_back"]
    assert d.iteration == 5 and tr.failure_count() == 0
    assert torch.isfinite(tr.u).all() and torch.isfinite(tr.radii).all()


@pytest.mark.gpu
def test_gpu_driver_poisoned_initial_state_is_final():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mara3p_gb300 import sedov
    from mara3p_gb300._capi import MaraError
    ncells, theta, radii, u = sedov.seeded_tracks(16, seed=6)
    tr = sedov.Tracks(ncells, theta, radii, u)
    tr.u[4, 3] = math.nan
    poisoned = tr.u.clone()
    d = sedov.Driver(tr, lambda t: (wind(tr.T, 1.0), wind(tr.T, 1.8)))
    with pytest.raises(MaraError):
        d.step()
    assert torch.equal(torch.nan_to_num(tr.u, nan=-1.0), torch.nan_to_num(poisoned, nan=-1.0))
