"""The spherical-track SRHD oracle (oracle/sedov_oracle.cpp) against the
reference's own sedov:: scheme (tests/golden/sedov_golden.npz, made by
make_golden.py through oracle/_ref): one forward-Euler advance with every
intermediate array (primitives, radial gradients, radial Godunov data with
contact speeds, polar faces with areas and cell indexes), and RK2 / RK3 runs
of three steps. Same evaluation order on both sides, so bit for bit."""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import dptr

ROOT = Path(__file__).resolve().parents[1]
CASES = ["uniform_plm", "focused_swirl", "focused_pcm"]


@pytest.fixture(scope="module")
def sedov_golden():
    return dict(np.load(ROOT / "tests" / "golden" / "sedov_golden.npz"))


def case(g, name):
    k = lambda s: g[f"sedov/{name}/{s}"]  # noqa: E731
    T = int(k("T")[0])
    nc = np.ascontiguousarray(k("ncells"), dtype=np.int64)
    return k, T, nc, int(nc.sum())


def i64p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


@pytest.mark.parametrize("name", CASES)
def test_euler_advance_and_parts_match_reference(oracle, sedov_golden, name):
    k, T, nc, C = case(sedov_golden, name)
    F = C + T
    NP = int(sum(nc[j] + nc[j + 1] + 1 for j in range(T - 1)))
    ro, uo = np.zeros(F), np.zeros(5 * C)
    parts = [np.zeros(5 * C), np.zeros(5 * C), np.zeros(6 * F), np.zeros(8 * NP)]
    rc = oracle.oracle_sedov_advance(ctypes.c_int32(T), i64p(nc), dptr(k("theta")), dptr(k("radii")), dptr(k("u")),
                                     dptr(np.ascontiguousarray(k("ghost_in")[:5 * T])),
                                     dptr(np.ascontiguousarray(k("ghost_out")[:5 * T])), ctypes.c_double(k("dt")[0]),
                                     ctypes.c_int32(int(k("use_plm")[0])), dptr(ro), dptr(uo), *[dptr(p) for p in parts])
    assert rc == 0
    assert np.array_equal(ro, k("euler/radii"))
    assert np.array_equal(uo, k("euler/u"))
    for nm, p in zip(("prim", "grad", "radial", "polar"), parts):
        assert np.array_equal(p, k(f"euler/{nm}")), nm


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("rk", [2, 3])
def test_rk_runs_match_reference(oracle, sedov_golden, name, rk):
    k, T, nc, C = case(sedov_golden, name)
    rad, u = k("radii").copy(), k("u").copy()
    for _ in range(3):
        assert oracle.oracle_sedov_advance_rk(ctypes.c_int32(T), i64p(nc), dptr(k("theta")), dptr(rad), dptr(u),
                                              dptr(k("ghost_in")), dptr(k("ghost_out")), ctypes.c_double(k("dt")[0]),
                                              ctypes.c_int32(rk), ctypes.c_int32(int(k("use_plm")[0]))) == 0
    assert np.array_equal(rad, k(f"rk{rk}_3/radii"))
    assert np.array_equal(u, k(f"rk{rk}_3/u"))


def test_geometry_matches_reference(oracle, sedov_golden):
    from oracle.oracle import load_reference
    r = load_reference()
    if r is None:
        pytest.skip("oracle/_ref is built only where the reference checkout is present")
    for f in ("cell_volume", "face_area"):
        getattr(oracle, f"oracle_sedov_{f}").restype = ctypes.c_double
        getattr(r, f"ref_sedov_{f}").restype = ctypes.c_double
    rng = np.random.default_rng(2)
    for _ in range(200):
        r0, r1 = np.sort(rng.uniform(0.5, 20.0, 2))
        t0, t1 = np.sort(rng.uniform(0.0, np.pi, 2))
        a = [ctypes.c_double(v) for v in (r0, r1, t0, t1)]
        assert oracle.oracle_sedov_cell_volume(*a) == r.ref_sedov_cell_volume(*a)
        assert oracle.oracle_sedov_face_area(*a) == r.ref_sedov_face_area(*a)


def remesh_cases(g):
    return sorted({k.split("/")[1] for k in g if k.startswith("remesh/")})


def test_remesh_matches_reference(oracle, sedov_golden):
    """sedov::remesh on tracks shaped for each branch (split, merges at the
    start, end and inside, inner-boundary drop, no change), bit for bit; the
    reference's recursion with exchanged aspect bounds included."""
    oracle.oracle_sedov_remesh.restype = ctypes.c_int64
    names = remesh_cases(sedov_golden)
    assert len(names) == 8
    for nm in names:
        k = lambda s: sedov_golden[f"remesh/{nm}/{s}"]  # noqa: E731
        rf, u = k("radii"), k("u")
        cells = len(rf) - 1
        amax, amin, inner, t0, t1 = k("bounds")
        ro = np.zeros(cells + 2)
        ro[:cells + 1] = rf
        uo = np.zeros(5 * (cells + 1))
        uo[:5 * cells] = u
        m = oracle.oracle_sedov_remesh(ctypes.c_int64(cells), ctypes.c_double(t0), ctypes.c_double(t1), dptr(ro),
                                       dptr(uo), ctypes.c_double(amax), ctypes.c_double(amin), ctypes.c_double(inner))
        assert m == int(k("cells_out")[0]), nm
        assert np.array_equal(ro[:m + 1], k("radii_out")), nm
        assert np.array_equal(uo[:5 * m], k("u_out")), nm
