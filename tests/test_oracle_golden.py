"""The oracle restatement against golden fixtures produced by the reference's
own compiled code (tests/golden/make_golden.py). CPU only; bit-exact."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle.oracle import MinidiskParams, dptr, iptr
from tests.golden.make_golden import MINIDISK_CASES
from tests.helpers import params_from_vector

CASES = list(MINIDISK_CASES)


@pytest.mark.parametrize("case", CASES)
def test_minidisk_substep_bitexact(oracle, golden, case):
    p = params_from_vector(golden[f"{case}/params"], float(golden[f"{case}/theta"][0]))
    u0 = golden[f"{case}/u0"]
    t, dt = golden[f"{case}/t"]
    out = np.zeros_like(u0)
    oracle.oracle_minidisk_substep(ctypes.byref(p), dptr(u0), dptr(out), ctypes.c_double(t), ctypes.c_double(dt), 2)
    assert np.array_equal(out, golden[f"{case}/substep"])


@pytest.mark.parametrize("case", CASES)
def test_minidisk_rk2_bitexact(oracle, golden, case):
    p = params_from_vector(golden[f"{case}/params"], float(golden[f"{case}/theta"][0]))
    u = golden[f"{case}/u0"].copy()
    t = oracle.oracle_minidisk_advance(ctypes.byref(p), dptr(u), ctypes.c_double(0.0), 5, 2, 0, 2)
    assert np.array_equal(u, golden[f"{case}/rk2_5"])
    assert t == golden[f"{case}/rk2_5_time"][0]


@pytest.mark.parametrize("case", CASES)
def test_minidisk_initial_state_matches_reference_formula(oracle, golden, case):
    p = params_from_vector(golden[f"{case}/params"])
    u = np.zeros_like(golden[f"{case}/u0"])
    oracle.oracle_minidisk_initial_conserved(ctypes.byref(p), ctypes.c_uint64(1234), ctypes.c_double(0.01), dptr(u))
    assert np.array_equal(u, golden[f"{case}/u0"])


def test_minidisk_block_update_bitexact(oracle, golden):
    p = params_from_vector(golden["block/params"])
    level, bi, bj = (int(x) for x in golden["block/index"])
    t, dt = golden["block/time_dt"]
    out = np.zeros_like(golden["block/uc"])
    oracle.oracle_minidisk_updated_conserved(ctypes.byref(p), dptr(golden["block/uc"]), dptr(golden["block/pe"]),
                                             ctypes.c_double(t), ctypes.c_double(dt), level, bi, bj, dptr(out))
    assert np.array_equal(out, golden["block/u1"])


@pytest.mark.parametrize("theta", [1.5, 2.0])
@pytest.mark.parametrize("axis", [0, 1])
def test_estimate_gradient_bitexact(oracle, golden, theta, axis):
    pe = golden["block/pe"]
    ref = golden[f"gradient/theta{theta}/axis{axis}"]
    out = np.zeros_like(ref)
    oracle.oracle_minidisk_estimate_gradient(dptr(pe), pe.shape[0], pe.shape[1], axis, ctypes.c_double(theta), dptr(out))
    assert np.array_equal(out, ref)


def test_plm_gradient_scalar_cases(oracle, golden):
    """plm_gradient on crafted triples (flat sides, zeros) at theta 1, 1.5, 2."""
    y = golden["plm/y"]
    for k, theta in enumerate(golden["plm/theta"]):
        pc = np.repeat(y.T[:, :, None], 3, axis=2).copy()      # (3, m, 3): the triple along axis 0
        out = np.zeros((1, y.shape[0], 3))
        oracle.oracle_minidisk_estimate_gradient(dptr(pc), 3, y.shape[0], 0, ctypes.c_double(theta), dptr(out))
        assert np.array_equal(out[0, :, 0], golden["plm/g"][k])


def test_binary_orbit_bitexact(oracle, golden):
    for i, (q, e, om) in enumerate(golden["binary/cases"]):
        p = MinidiskParams(block_size=8, depth=0, omega_frame=om, mach_number=10, nu=0, domain_radius=1,
                           softening_length=0.1, eccentricity=e, mass_ratio=q, sink_radius=0.1, sink_rate=1,
                           buffer_rate=1, buffer_scale=1, cfl=0.3, plm_theta=2.0)
        for j, t in enumerate(golden["binary/times"]):
            out = np.zeros(10)
            oracle.oracle_minidisk_binary(ctypes.byref(p), ctypes.c_double(t), dptr(out))
            assert np.array_equal(out, golden["binary/state"][i, j])


def test_srhd_conserved_and_recovery_bitexact(oracle, srhd_golden):
    g = 4.0 / 3.0
    prim = srhd_golden["srhd/prim"]
    n = prim.size // 5
    cons = np.zeros_like(prim)
    oracle.oracle_srhd_conserved_density(dptr(prim), ctypes.c_int64(n), ctypes.c_double(g), dptr(cons))
    assert np.array_equal(cons, srhd_golden["srhd/cons"])
    rec = np.zeros_like(prim)
    it = np.zeros(n, np.int32)
    st = np.zeros(n, np.int32)
    oracle.oracle_srhd_recover_primitive(dptr(cons), ctypes.c_int64(n), ctypes.c_double(g), ctypes.c_double(0.0),
                                         None, dptr(rec), iptr(it), iptr(st))
    assert np.array_equal(st, srhd_golden["srhd/status"])
    assert np.array_equal(rec, srhd_golden["srhd/recovered"])
    assert 4.0 < it.mean() < 6.0 and it.max() <= 51


def test_srhd_reference_known_answers(oracle, srhd_golden):
    """test_srhd's cons->prim round trips (src/physics_srhd.hpp:528-537): |p1 - p0| < 1e-10."""
    g = 4.0 / 3.0
    kat = srhd_golden["srhd_kat/prim"]
    cons = np.zeros_like(kat)
    oracle.oracle_srhd_conserved_density(dptr(kat), ctypes.c_int64(4), ctypes.c_double(g), dptr(cons))
    assert np.array_equal(cons, srhd_golden["srhd_kat/cons"])
    rec = np.zeros_like(kat)
    oracle.oracle_srhd_recover_primitive(dptr(cons), ctypes.c_int64(4), ctypes.c_double(g), ctypes.c_double(0.0),
                                         None, dptr(rec), None, None)
    assert np.array_equal(rec, srhd_golden["srhd_kat/recovered"])
    assert np.all(np.abs(rec - kat) < 1e-10)


@pytest.mark.parametrize("solver", ["hlle", "hllc"])
@pytest.mark.parametrize("axis", [1, 2, 3])
def test_srhd_riemann_bitexact(oracle, srhd_golden, solver, axis):
    pl, pr = srhd_golden["srhd_riemann/pl"], srhd_golden["srhd_riemann/pr"]
    n = pl.size // 5
    f = np.zeros_like(pl)
    bad = oracle.oracle_srhd_riemann(dptr(pl), dptr(pr), ctypes.c_int64(n), axis, ctypes.c_double(4.0 / 3.0),
                                     int(solver == "hllc"), dptr(f))
    assert bad == 0
    assert np.array_equal(f, srhd_golden[f"srhd_riemann/{solver}/axis{axis}"])


@pytest.fixture(scope="module")
def mhd_golden():
    from pathlib import Path
    return dict(np.load(Path(__file__).resolve().parent / "golden" / "mhd_golden.npz"))


def _mhd_oracle(oracle):
    for f in (oracle.oracle_mhd_advance_ct, oracle.oracle_mhd_rk2, oracle.oracle_mhd_max_div_b):
        f.restype = ctypes.c_double
    oracle.oracle_mhd_round_trip.restype = ctypes.c_int64
    return oracle


def test_mhd_initial_state_and_table(oracle, mhd_golden):
    """The oracle's mode table and construct_conserved discretisation
    reproduce the fixture's inputs; the library's host table agrees."""
    o = _mhd_oracle(oracle)
    N, g = int(mhd_golden["mhd/params"][0]), mhd_golden["mhd/params"][1]
    table = mhd_golden["mhd/table"]
    modes = table.size // 11
    t2 = np.zeros_like(table)
    assert o.oracle_mhd_mode_table(ctypes.c_uint64(3), modes, dptr(t2)) == 0
    assert np.array_equal(t2, table)
    from mara3p_gb300 import mhd
    assert np.array_equal(mhd.mode_table(3, modes), table)
    v_amp, a_amp = mhd_golden["mhd/amp"]
    assert np.allclose(mhd.amplitudes(modes), (v_amp, a_amp), rtol=1e-15)
    uc = np.zeros(N ** 3 * 5)
    bf = [np.zeros((N + 1) * N * N) for _ in range(3)]
    o.oracle_mhd_initial(N, dptr(table), modes, ctypes.c_double(v_amp), ctypes.c_double(a_amp), ctypes.c_double(g),
                         dptr(uc), *[dptr(b) for b in bf])
    assert np.array_equal(uc, mhd_golden["mhd/uc"])
    for k in range(3):
        assert np.array_equal(bf[k], mhd_golden[f"mhd/bf{k + 1}"])
    assert o.oracle_mhd_max_div_b(N, *[dptr(b) for b in bf]) < 1e-14


def test_mhd_advance_ct_bitexact(oracle, mhd_golden):
    o = _mhd_oracle(oracle)
    N, g, cfl, theta = mhd_golden["mhd/params"]
    N = int(N)
    outs = [np.zeros(N ** 3 * 5)] + [np.zeros((N + 1) * N * N) for _ in range(3)]
    dt = o.oracle_mhd_advance_ct(N, dptr(mhd_golden["mhd/uc"]), *[dptr(mhd_golden[f"mhd/bf{k}"]) for k in (1, 2, 3)],
                                 ctypes.c_double(1.0 / N), ctypes.c_double(cfl), ctypes.c_double(theta),
                                 ctypes.c_double(g), *[dptr(a) for a in outs])
    assert dt == mhd_golden["mhd/step_time"][0]
    assert np.array_equal(outs[0], mhd_golden["mhd/step_uc"])
    for k in range(3):
        assert np.array_equal(outs[k + 1], mhd_golden[f"mhd/step_bf{k + 1}"])


def test_mhd_rk2_bitexact(oracle, mhd_golden):
    o = _mhd_oracle(oracle)
    N, g, cfl, theta = mhd_golden["mhd/params"]
    N = int(N)
    uc = mhd_golden["mhd/uc"].copy()
    bf = [mhd_golden[f"mhd/bf{k}"].copy() for k in (1, 2, 3)]
    t = o.oracle_mhd_rk2(N, dptr(uc), *[dptr(b) for b in bf], ctypes.c_double(0.0), 2, ctypes.c_double(1.0 / N),
                         ctypes.c_double(cfl), ctypes.c_double(theta), ctypes.c_double(g))
    assert t == mhd_golden["mhd/rk2_time"][0]
    assert np.array_equal(uc, mhd_golden["mhd/rk2_uc"])
    for k in range(3):
        assert np.array_equal(bf[k], mhd_golden[f"mhd/rk2_bf{k + 1}"])


def test_mhd_rk2_threads_bitexact(oracle, mhd_golden):
    """The threaded oracle loop gives the reference's RK2 result bit for bit."""
    o = _mhd_oracle(oracle)
    o.oracle_mhd_rk2_threads.restype = ctypes.c_double
    N, g, cfl, theta = mhd_golden["mhd/params"]
    N = int(N)
    uc = mhd_golden["mhd/uc"].copy()
    bf = [mhd_golden[f"mhd/bf{k}"].copy() for k in (1, 2, 3)]
    t = o.oracle_mhd_rk2_threads(N, dptr(uc), *[dptr(b) for b in bf], ctypes.c_double(0.0), 2,
                                 ctypes.c_double(1.0 / N), ctypes.c_double(cfl), ctypes.c_double(theta),
                                 ctypes.c_double(g), 4)
    assert t == mhd_golden["mhd/rk2_time"][0]
    assert np.array_equal(uc, mhd_golden["mhd/rk2_uc"])
    for k in range(3):
        assert np.array_equal(bf[k], mhd_golden[f"mhd/rk2_bf{k + 1}"])


def test_mhd_reference_known_answers(oracle, mhd_golden):
    """test_mhd's round trips (src/physics_mhd.hpp:405-415): within 1e-10."""
    o = _mhd_oracle(oracle)
    kat = mhd_golden["mhd_kat/prim"]
    cons = np.zeros(25)
    back = np.zeros_like(kat)
    assert o.oracle_mhd_round_trip(dptr(kat), ctypes.c_int64(5), ctypes.c_double(5.0 / 3.0), dptr(cons), dptr(back)) == 0
    assert np.array_equal(cons, mhd_golden["mhd_kat/cons"])
    assert np.array_equal(back, mhd_golden["mhd_kat/back"])
    assert np.all(np.abs(back - kat) < 1e-10)


# ---- mhd_scheme_v2 block operations: the numpy restatement against the
# reference's own outputs (tests/golden/physics_golden.npz)

@pytest.fixture(scope="module")
def physics_golden():
    from pathlib import Path
    return dict(np.load(Path(__file__).resolve().parent / "golden" / "physics_golden.npz"))


def _v2_shapes(g):
    c = tuple(int(x) for x in g["v2/block"])
    m = tuple(int(x) for x in g["v2/extended"])
    stag = lambda s, a, grow, side: tuple(n + (grow if k == a else side) for k, n in enumerate(s))  # noqa: E731
    return c, m, stag


def test_mhd_v2_face_to_cell_matches_reference(physics_golden):
    """primitive_array's cell fields are face_to_cell of the faces."""
    from oracle import mhd_v2_oracle as v2
    g = physics_golden
    c, _, stag = _v2_shapes(g)
    b = [g[f"v2/prim/bf{a + 1}"].reshape(stag(c, a, 1, 0)) for a in range(3)]
    pc = g["v2/prim/pc"].reshape(*c, 8)
    assert np.array_equal(v2.face_to_cell(*b), pc[..., 5:8])


def test_mhd_v2_electromotive_forces_bitexact(physics_golden):
    from oracle import mhd_v2_oracle as v2
    g = physics_golden
    _, m, stag = _v2_shapes(g)
    gf = [g[f"v2/god/gf{a + 1}"].reshape(*stag(m, a, -1, 0), 8) for a in range(3)]
    for a, e in enumerate(v2.electromotive_forces(*gf)):
        assert e.shape == stag(m, a, 0, -1)
        assert np.array_equal(e.ravel(), g[f"v2/emf/ee{a + 1}"])


def test_mhd_v2_updated_conserved_density_bitexact(physics_golden):
    from oracle import mhd_v2_oracle as v2
    g = physics_golden
    c, _, stag = _v2_shapes(g)
    dt, dl = g["v2/ucd/dt_dl"]
    gf = [g[f"v2/ucd/gf{a + 1}"].reshape(*stag(c, a, 1, 2), 8) for a in range(3)]
    out = v2.updated_conserved_density(g["v2/ucd/uc"].reshape(*c, 5), *gf, dt, dl)
    assert np.array_equal(out.ravel(), g["v2/ucd/out"])


def test_mhd_v2_curl_and_flux_update_bitexact(physics_golden):
    from oracle import mhd_v2_oracle as v2
    g = physics_golden
    c, _, stag = _v2_shapes(g)
    dt, dl = g["v2/ucd/dt_dl"]
    ee = [g[f"v2/curl/ee{a + 1}"].reshape(stag(c, a, 0, 1)) for a in range(3)]
    for a, cf in enumerate(v2.curl(*ee, dl)):
        assert np.array_equal(cf.ravel(), g[f"v2/curl/cf{a + 1}"])
    bf = [g[f"v2/umfd/bf{a + 1}"].reshape(stag(c, a, 1, 0)) for a in range(3)]
    ex = [g[f"v2/umfd/ee{a + 1}"].reshape(stag(c, a, 2, 1)) for a in range(3)]
    for a, b in enumerate(v2.updated_magnetic_flux_density(*bf, *ex, dt, dl)):
        assert np.array_equal(b.ravel(), g[f"v2/umfd/out{a + 1}"])


def test_mhd_v2_curl_of_reference_is_divergence_free(physics_golden):
    """A property of the reference's own curl output: div(curl E) = 0 to rounding."""
    g = physics_golden
    c, _, stag = _v2_shapes(g)
    cf = [g[f"v2/curl/cf{a + 1}"].reshape(stag(c, a, 1, 0)) for a in range(3)]
    div = np.diff(cf[0], axis=0) + np.diff(cf[1], axis=1) + np.diff(cf[2], axis=2)
    assert np.abs(div).max() < 1e-13 * max(np.abs(x).max() for x in cf)
