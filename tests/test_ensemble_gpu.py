"""Batched minidisk ensembles on the GPU: every member's state and clock after
an ensemble advance equal, bit for bit, those of the single-mesh advance of
that member, in both precisions and for any launch shape, tuned or not."""
from __future__ import annotations

import ctypes

import pytest
import torch

from mara3p_gb300 import ensemble as ens
from mara3p_gb300.minidisk import DT_CFL, DT_FORMULA, FP64, MIXED, Run, SolverData, initial_conserved

pytestmark = pytest.mark.gpu

BASE = SolverData(block_size=64, depth=0, domain_radius=4.0, softening_length=0.05, sink_radius=0.05, sink_rate=10.0,
                  buffer_rate=10.0, buffer_scale=0.1, mach_number=10.0, nu=1e-3, cfl=0.3, plm_theta=1.5)


def members():
    return [
        BASE,
        BASE.with_(depth=1, mass_ratio=0.4, eccentricity=0.3, mach_number=22.0, nu=2e-4),
        BASE.with_(block_size=96, mass_ratio=0.7, eccentricity=0.1, mach_number=14.0),
        BASE.with_(block_size=100, depth=1, mass_ratio=0.2, eccentricity=0.45, mach_number=28.0, nu=5e-4),
        BASE.with_(depth=2, mass_ratio=1.0, eccentricity=0.05, mach_number=18.0, nu=8e-4),
    ]


def initial(ms):
    return [initial_conserved(sd, seed=11 + m, amplitude=0.01) for m, sd in enumerate(ms)]


def single(sd, u0, clock0, steps, rk, precision, dt_mode):
    run = Run(sd, u0.clone(), rk_order=rk, precision=precision, dt_mode=dt_mode)
    run.clock.copy_(clock0)
    run.advance(steps)
    torch.cuda.synchronize()
    return run.u, run.clock_state()


def clock_bytes(e: ens.Ensemble, m: int) -> torch.Tensor:
    size = ctypes.sizeof(ens.MinidiskClock)
    return e.clocks[m * size:(m + 1) * size].clone()


def rel_max(a: torch.Tensor, b: torch.Tensor) -> float:
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("precision", [FP64, MIXED])
@pytest.mark.parametrize("rk", [1, 2])
@pytest.mark.parametrize("steps", [4, 5])
def test_members_match_single_mesh_advance(precision, rk, steps):
    ms = members()
    u0 = initial(ms)
    with ens.Ensemble(ms, [u.clone() for u in u0], rk_order=rk, precision=precision, dt_mode=DT_CFL,
                      autotune=0) as e:
        clocks0 = [clock_bytes(e, m) for m in range(len(ms))]
        e.advance(steps)
        torch.cuda.synchronize()
        got = e.clock_states()
        for m, sd in enumerate(ms):
            u1, c1 = single(sd, u0[m], clocks0[m], steps, rk, precision, DT_CFL)
            assert got[m].iteration == c1.iteration == steps
            # both precisions round every operation the same way in both paths: bit-identical
            assert torch.equal(e.states[m], u1), (m, rel_max(e.states[m], u1))
            assert got[m].time == c1.time and got[m].dt == c1.dt
            assert torch.isfinite(e.states[m]).all()


def test_launch_shapes_agree_and_split_advances_equal_one():
    ms = members()
    u0 = initial(ms)
    shapes = [dict(blocks_per_sm=1, chunks_per_warp=1, cols_per_lane=1, register_variant=0),
              dict(blocks_per_sm=2, chunks_per_warp=4, cols_per_lane=1, register_variant=1),
              dict(blocks_per_sm=3, chunks_per_warp=8, cols_per_lane=1, register_variant=2),
              dict(blocks_per_sm=2, chunks_per_warp=1, cols_per_lane=2, register_variant=0),
              dict(blocks_per_sm=1, chunks_per_warp=2, cols_per_lane=2, register_variant=2)]
    results = []
    for k, shape in enumerate(shapes):
        with ens.Ensemble(ms, [u.clone() for u in u0], precision=MIXED, dt_mode=DT_CFL, autotune=0) as e:
            e.set_config(**shape)
            assert {f: e.config[f] for f in shape} == shape
            if k == 0:
                e.advance(3)
                e.advance(2)
            else:
                e.advance(5)
            torch.cuda.synchronize()
            results.append([u.clone() for u in e.states])
    for other in results[1:]:
        for a, b in zip(results[0], other):
            assert torch.equal(a, b), rel_max(b, a)


def test_tuner_picks_a_timed_shape_and_keeps_results():
    ms = members()
    u0 = initial(ms)
    with ens.Ensemble(ms, [u.clone() for u in u0], precision=MIXED, dt_mode=DT_CFL, autotune=2) as e:
        cfg = e.config
        assert cfg["stage_ms"] > 0.0
        assert cfg["blocks_per_sm"] >= 1 and cfg["chunks_per_warp"] in (1, 2, 4, 8)
        assert cfg["cols_per_lane"] in (1, 2)
        assert cfg["register_variant"] in (0, 1, 2)
        # the tuner only wrote scratch: the clocks and states are as created
        clocks0 = [clock_bytes(e, m) for m in range(len(ms))]
        for a, b in zip(e.states, u0):
            assert torch.equal(a, b)
        e.advance(4)
        torch.cuda.synchronize()
        for m, sd in enumerate(ms):
            u1, _ = single(sd, u0[m], clocks0[m], 4, 2, MIXED, DT_CFL)
            assert torch.equal(e.states[m], u1)
    # a second ensemble of the same mesh sizes reuses the tuned shape
    with ens.Ensemble(ms, [u.clone() for u in u0], precision=MIXED, dt_mode=DT_CFL, autotune=1) as e2:
        assert e2.config == cfg


def test_mixed_members_stay_within_the_fp64_error_budget():
    ms = members()
    u0 = initial(ms)
    out = {}
    for precision in (FP64, MIXED):
        with ens.Ensemble(ms, [u.clone() for u in u0], precision=precision, dt_mode=DT_FORMULA, autotune=0) as e:
            e.advance(10)
            torch.cuda.synchronize()
            out[precision] = [u.clone() for u in e.states]
    for a, b in zip(out[MIXED], out[FP64]):
        rel_l1 = float((a[0] - b[0]).abs().sum() / b[0].abs().sum())
        assert rel_l1 < 1e-6


def test_seeded_ensemble_runs():
    ms = ens.seeded_members(3, 6, BASE, sizes=(64, 128, 192))
    with ens.Ensemble(ms, precision=MIXED, dt_mode=DT_CFL, autotune=1) as e:
        e.advance(3)
        torch.cuda.synchronize()
        assert all(c.iteration == 3 for c in e.clock_states())
        assert all(torch.isfinite(u).all() for u in e.states)
        assert e.cells == sum(sd.cells_per_side ** 2 for sd in ms)


def test_bad_config_is_rejected_and_the_old_one_kept():
    ms = members()[:2]
    with ens.Ensemble(ms, precision=MIXED, autotune=0) as e:
        before = e.config
        from mara3p_gb300._capi import MaraError
        with pytest.raises(MaraError):
            e.set_config(blocks_per_sm=1000)
        with pytest.raises(MaraError):
            e.set_config(cols_per_lane=3)
        with pytest.raises(MaraError):
            e.set_config(register_variant=4)
        assert e.config == before
        e.advance(2)
        torch.cuda.synchronize()
        assert all(c.iteration == 2 for c in e.clock_states())
