"""The ensemble's work-list planner and argument checks (host only, no GPU).

The planner cuts the column strips (28 columns for the 1-column sweep, 60 for
the 2-column one) of every member mesh, rows laid end to end, into equal chunks; the persistent sweep launch gives one chunk to each
warp (or hands chunks out dynamically). Every row of every strip must be
covered exactly once, in order, and the chunks must be balanced."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from mara3p_gb300 import ensemble
from mara3p_gb300._capi import MaraError, check, lib
from mara3p_gb300.minidisk import FP64, MIXED, SolverData


def _strips(n: int, cols: int = 1) -> int:
    w = ensemble.STRIP_COLUMNS[cols]
    return (n + w - 1) // w


def _coverage(sizes, items, cols=1):
    seen = {}
    for m, sy, i0, i1 in items:
        assert 0 <= m < len(sizes)
        assert 0 <= sy < _strips(sizes[m], cols)
        assert 0 <= i0 < i1 <= sizes[m]
        seen.setdefault((m, sy), []).append((i0, i1))
    for m, n in enumerate(sizes):
        for sy in range(_strips(n, cols)):
            ranges = seen.pop((m, sy))
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:])), "rows of a strip in order, no gap or overlap"
    assert not seen


@pytest.mark.parametrize("sizes,chunks", [
    ([128, 256, 512, 1024], 608),
    ([1024] * 3 + [128] * 7, 2432),
    ([64], 1),
    ([64], 7),
    ([100, 64, 300], 57),
    ([4096], 3648),
    ([128], 5000),           # more chunks than rows: some chunks stay empty
])
@pytest.mark.parametrize("cols", [1, 2])
def test_plan_covers_every_row_once_and_balances(sizes, chunks, cols):
    items, first = ensemble.plan(sizes, chunks, cols)
    _coverage(sizes, items, cols)
    assert first[0] == 0 and first[-1] == len(items)
    assert np.all(np.diff(first) >= 0)
    # the items, in chunk order, follow the members' strips end to end
    order = [(m, sy, i0) for m, sy, i0, _ in items]
    assert order == sorted(order)
    rows = np.array([sum(int(i1 - i0) for _, _, i0, i1 in items[first[c]:first[c + 1]]) for c in range(chunks)])
    total = sum(_strips(n, cols) * n for n in sizes)
    assert rows.sum() == total
    target = total / chunks
    if target >= 8:
        # a chunk differs from the target by at most a short strip tail (< 4 rows) plus rounding
        assert np.all(np.abs(rows - target) <= 5), (rows.min(), rows.max(), target)


def test_plan_items_never_shorter_than_a_tail_unless_the_strip_is():
    items, _ = ensemble.plan([1024, 512], 977)
    lens = items[:, 3] - items[:, 2]
    assert lens.min() >= 1
    # a piece shorter than 4 rows can only start a chunk, never end a strip
    for m, sy, i0, i1 in items[lens < 4]:
        assert i1 != [1024, 512][m]


@pytest.mark.parametrize("sizes,chunks,width", [([], 4, 28), ([64], 0, 28), ([0], 4, 28), ([70000], 4, 28),
                                                ([64], 4, 32)])
def test_plan_rejects_bad_arguments(sizes, chunks, width):
    s = np.ascontiguousarray(sizes if sizes else [64], dtype=np.int32)
    n = lib.mara_minidisk_ensemble_plan(s.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(sizes), chunks,
                                        width, None, 0, None)
    assert n == -1
    assert b"mara_minidisk_ensemble_plan" in lib.mara_last_error()


def test_seeded_members_follow_the_distribution():
    base = SolverData(domain_radius=4.0)
    ms = ensemble.seeded_members(7, 256, base)
    assert ms == ensemble.seeded_members(7, 256, base)
    sizes = {m.cells_per_side for m in ms}
    assert sizes == set(ensemble.MESH_SIZES)
    assert all(m.block_size == 64 for m in ms)
    q = np.array([m.mass_ratio for m in ms])
    e = np.array([m.eccentricity for m in ms])
    mach = np.array([m.mach_number for m in ms])
    nu = np.array([m.nu for m in ms])
    assert q.min() >= 0.1 and q.max() <= 1.0
    assert e.min() >= 0.0 and e.max() <= 0.5
    assert mach.min() >= 10 and mach.max() <= 30
    assert nu.min() >= 1e-4 and nu.max() <= 1e-3
    assert all(m.domain_radius == 4.0 for m in ms)


def _create(params, count, states, clocks=1, rk=2, precision=MIXED, dt_mode=1, autotune=0):
    arr = (type(params[0]) * max(1, len(params)))(*params)
    ptrs = (ctypes.c_void_p * max(1, len(states)))(*states)
    h = ctypes.c_void_p()
    return lib.mara_minidisk_ensemble_create(arr, count, ptrs, clocks, rk, precision, dt_mode, autotune,
                                             ctypes.byref(h))


def test_create_rejects_bad_arguments_before_any_device_work():
    p = SolverData(block_size=32, depth=0).to_c()
    fake = 4096          # never dereferenced: every case fails in the host-side checks
    assert _create([p], 0, [fake]) == 1
    assert _create([p], 1, [fake], rk=3) == 1
    assert _create([p], 1, [fake], precision=5) == 1
    assert _create([p], 1, [fake], dt_mode=7) == 1
    assert _create([p], 1, [fake], autotune=3) == 1
    assert _create([p], 1, [None]) == 1
    assert _create([p], 1, [fake + 8]) == 1            # misaligned state
    assert _create([p], 1, [fake]) == 1                 # mixed needs N >= 64
    assert b"at least 64" in lib.mara_last_error()
    bad = SolverData(mach_number=0.0).to_c()
    assert _create([bad], 1, [fake], precision=FP64) == 1
    with pytest.raises(MaraError):
        check(_create([p], 1, [fake]), "create")
