"""Generate the golden fixtures in this directory from the reference itself.

Run where the reference checkout is present (it is not on the GPU hosts):

    make -C oracle ref && python tests/golden/make_golden.py [--physics-only]

oracle/_ref/libref.so is the reference's own scheme and physics code
(problems/minidisk_scheme.cpp, src/physics_*.hpp, src/scheme_*) compiled in
place with oracle/ref_harness.cpp. Every output below is produced by that
library; inputs are seeded. The fixtures pin the oracle restatement
(tests/test_oracle_golden.py) and, through it, the GPU kernels.
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle.oracle import (MinidiskParams, dptr, iptr, load_oracle, load_reference,  # noqa: E402
                           load_reference_v2, solver_vector)

MINIDISK_CASES = {
    # name: solver_data (block_size 16, depth 2 -> 64^2 mesh), seed, perturbation, time, dt scale
    "config1_like": dict(block_size=16, depth=2, omega_frame=1.0, mach_number=10.0, nu=1e-3, domain_radius=1.0,
                         softening_length=0.05, eccentricity=0.0, mass_ratio=1.0, sink_radius=0.05, sink_rate=10.0,
                         buffer_rate=100.0, buffer_scale=0.2, cfl=0.3, plm_theta=2.0),
    "eccentric_unequal": dict(block_size=16, depth=2, omega_frame=1.0, mach_number=20.0, nu=5e-4, domain_radius=1.0,
                              softening_length=0.05, eccentricity=0.1, mass_ratio=0.5, sink_radius=0.05,
                              sink_rate=10.0, buffer_rate=100.0, buffer_scale=0.2, cfl=0.3, plm_theta=2.0),
    "inviscid_defaults": dict(block_size=8, depth=3, omega_frame=1.0, mach_number=10.0, nu=0.0, domain_radius=1.5,
                              softening_length=0.01, eccentricity=0.0, mass_ratio=1.0, sink_radius=0.01,
                              sink_rate=1e3, buffer_rate=1e2, buffer_scale=0.2, cfl=0.3, plm_theta=2.0),
}


def minidisk_fixtures(o, r) -> dict[str, np.ndarray]:
    out = {}
    for name, kw in MINIDISK_CASES.items():
        p = MinidiskParams(**kw)
        N = p.block_size << p.depth
        u0 = np.zeros(3 * N * N)
        o.oracle_minidisk_initial_conserved(ctypes.byref(p), ctypes.c_uint64(1234), ctypes.c_double(0.01), dptr(u0))
        sdv = solver_vector(p)
        # one forward-Euler substep at t = 0.37 with the reference dt formula
        t = 0.37
        dt = o.oracle_minidisk_dt_formula(ctypes.byref(p), ctypes.c_double(t))
        u1 = np.zeros_like(u0)
        assert r.ref_minidisk_substep(dptr(sdv), dptr(u0), dptr(u1), ctypes.c_double(t), ctypes.c_double(dt), 4) == 0
        # 5 RK2 steps from t = 0, control::advance_runge_kutta semantics
        u = u0.copy()
        tt = 0.0
        a = np.zeros_like(u0)
        b = np.zeros_like(u0)
        for _ in range(5):
            dts = o.oracle_minidisk_dt_formula(ctypes.byref(p), ctypes.c_double(tt))
            r.ref_minidisk_substep(dptr(sdv), dptr(u), dptr(a), ctypes.c_double(tt), ctypes.c_double(dts), 4)
            r.ref_minidisk_substep(dptr(sdv), dptr(a), dptr(b), ctypes.c_double(tt + dts), ctypes.c_double(dts), 4)
            u = u * 0.5 + b * (1.0 - 0.5)
            tt = tt * 0.5 + ((tt + dts) + dts) * (1.0 - 0.5)
        out[f"{name}/u0"] = u0
        out[f"{name}/t"] = np.array([t, dt])
        out[f"{name}/substep"] = u1
        out[f"{name}/rk2_5"] = u
        out[f"{name}/rk2_5_time"] = np.array([tt])
        out[f"{name}/params"] = sdv
        out[f"{name}/theta"] = np.array([p.plm_theta])
    return out


def block_fixture(r) -> dict[str, np.ndarray]:
    """updated_conserved on one block (level 2, block (1, 3)) with seeded pe/uc."""
    kw = MINIDISK_CASES["config1_like"]
    p = MinidiskParams(**kw)
    n = p.block_size
    rng = np.random.default_rng(99)
    x = np.linspace(-1, 1, n + 4)
    base = np.stack(np.meshgrid(x, x, indexing="ij"), -1)
    pe = np.empty((n + 4, n + 4, 3))
    pe[..., 0] = 1.0 + 0.2 * np.sin(3 * base[..., 0]) * np.cos(2 * base[..., 1]) + 0.01 * rng.standard_normal((n + 4, n + 4))
    pe[..., 1] = 0.3 * np.cos(base[..., 1] * 4) + 0.02 * rng.standard_normal((n + 4, n + 4))
    pe[..., 2] = -0.2 * np.sin(base[..., 0] * 5) + 0.02 * rng.standard_normal((n + 4, n + 4))
    pc = pe[2:-2, 2:-2]
    uc = np.stack([pc[..., 0], pc[..., 0] * pc[..., 1], pc[..., 0] * pc[..., 2]], -1).copy()
    pe = np.ascontiguousarray(pe)
    out_u = np.zeros_like(uc)
    assert r.ref_minidisk_updated_conserved(dptr(solver_vector(p)), dptr(uc), dptr(pe), ctypes.c_double(0.81),
                                            ctypes.c_double(2e-3), 2, 1, 3, dptr(out_u)) == 0
    res = {"block/pe": pe, "block/uc": uc, "block/u1": out_u, "block/params": solver_vector(p),
           "block/index": np.array([2, 1, 3]), "block/time_dt": np.array([0.81, 2e-3])}
    for theta in (1.5, 2.0):
        for axis in (0, 1):
            g = np.zeros((n + 2, n + 4, 3) if axis == 0 else (n + 4, n + 2, 3))
            r.ref_minidisk_estimate_gradient(dptr(pe), n + 4, n + 4, axis, ctypes.c_double(theta), dptr(g))
            res[f"gradient/theta{theta}/axis{axis}"] = g
    return res


def plm_fixture(r) -> dict[str, np.ndarray]:
    rng = np.random.default_rng(5)
    y = rng.standard_normal((512, 3))
    y[::7, 1] = y[::7, 0]            # flat left
    y[::11, 2] = y[::11, 1]          # flat right
    y[::13] = 0.0                     # all zero
    thetas = np.array([1.0, 1.5, 2.0])
    g = np.array([[r.ref_plm_gradient(th, *row) for row in y] for th in thetas])
    return {"plm/y": y, "plm/theta": thetas, "plm/g": g}


def binary_fixture(r) -> dict[str, np.ndarray]:
    cases = np.array([[1.0, 0.0, 1.0], [0.5, 0.1, 1.0], [0.3, 0.5, 0.0], [1.0, 0.4, 0.7]])
    times = np.array([0.0, 0.37, 2.3, 31.4159, 100.0])
    res = np.zeros((len(cases), len(times), 10))
    for i, (q, e, om) in enumerate(cases):
        for j, t in enumerate(times):
            buf = np.zeros(10)
            r.ref_minidisk_binary(ctypes.c_double(q), ctypes.c_double(e), ctypes.c_double(om), ctypes.c_double(t), dptr(buf))
            res[i, j] = buf
    return {"binary/cases": cases, "binary/times": times, "binary/state": res}


def two_body_fixture(r) -> dict[str, np.ndarray]:
    """two_body::orbital_state and recover_orbital_elements of the reference on
    on-orbit states, states moved off the orbit (shifted, boosted, rescaled
    velocities) and unbound states."""
    rng = np.random.default_rng(17)
    elements = np.array([[1.0, 1.0, 1.0, 0.0], [1.0, 1.0, 1.0, 0.5], [1.0, 1.0, 0.5, 0.1], [2.0, 1.5, 0.3, 0.7]])
    times = np.array([0.0, 0.37, 2.3, 17.0])
    states, ts = [], []
    for el in elements:
        for t in times:
            buf = np.zeros(10)
            r.ref_two_body_state(*[ctypes.c_double(v) for v in el], ctypes.c_double(t), dptr(buf))
            states.append(buf.copy())
            ts.append(t)
            off = buf.copy()
            off[[1, 6]] += rng.uniform(-0.3, 0.3)
            off[[2, 7]] += rng.uniform(-0.3, 0.3)
            off[[3, 8]] += rng.uniform(-0.2, 0.2)
            off[[4, 9]] += rng.uniform(-0.2, 0.2)
            off[[3, 4, 8, 9]] *= rng.uniform(0.9, 1.1)
            states.append(off)
            ts.append(t)
    unbound = states[0].copy()
    unbound[[3, 4, 8, 9]] *= 2.0
    states.append(unbound)
    ts.append(0.0)
    states = np.array(states)
    out = np.zeros_like(states)
    status = np.zeros(len(states), np.int32)
    for i, (st, t) in enumerate(zip(states, ts)):
        status[i] = r.ref_two_body_elements(dptr(st), ctypes.c_double(t), dptr(out[i]))
    return {"two_body/elements": elements, "two_body/times": times, "two_body/state": states,
            "two_body/t": np.array(ts), "two_body/recovered": out, "two_body/status": status}


SEDOV_CASES = {
    # name: (track count, polar focus, radial aspect, outer radius, u3 amplitude, use_plm, seed)
    "uniform_plm": (6, 0.0, 0.5, 6.0, 0.0, 1, 31),
    "focused_swirl": (7, 0.5, 0.4, 5.0, 0.05, 1, 32),
    "focused_pcm": (5, 0.3, 0.6, 4.0, 0.0, 0, 33),
}


def sedov_case(o, r, name):
    """Tracks from the reference's generate_radial_track over polar bounds
    spaced as the driver's "focus" option spaces them, a seeded blast in a
    wind (primitives at the cell centres, conserved volume integrals), and
    ghost primitives for the boundary Riemann problems of three RK stages."""
    T, focus, aspect, r1, u3amp, use_plm, seed = SEDOV_CASES[name]
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, T + 1)
    theta = np.pi * (x + focus * (x - 1) * x) / (1 + 2 * focus * (x - 1) * x)
    r.ref_sedov_generate_track.restype = ctypes.c_int64
    r.ref_sedov_cell_volume.restype = ctypes.c_double
    radii, ncells = [], []
    for j in range(T):
        a = (ctypes.c_double(1.0), ctypes.c_double(r1), ctypes.c_double(theta[j]), ctypes.c_double(theta[j + 1]),
             ctypes.c_double(aspect))
        n = r.ref_sedov_generate_track(*a, None, ctypes.c_int64(0))
        buf = np.zeros(n)
        r.ref_sedov_generate_track(*a, dptr(buf), ctypes.c_int64(n))
        radii.append(buf)
        ncells.append(n - 1)
    cons = []
    for j in range(T):
        rf = radii[j]
        rc = 0.5 * (rf[:-1] + rf[1:])
        qc = 0.5 * (theta[j] + theta[j + 1])
        n = len(rc)
        pr = np.zeros((n, 5))
        pr[:, 0] = rc ** -2 * (1 + 0.05 * rng.uniform(-1, 1, n))
        pr[:, 1] = 0.5 + 0.3 * np.sin(3 * qc) + 0.05 * rng.uniform(-1, 1, n)
        pr[:, 2] = 0.02 * rng.uniform(-1, 1, n)
        pr[:, 3] = u3amp * rng.uniform(-1, 1, n)
        pr[:, 4] = 1e-3 * pr[:, 0] * (1 + 0.1 * rng.uniform(0, 1, n)) + np.where(rc < 2.0, 0.5, 0.0)
        uc = np.zeros(5 * n)
        o.oracle_srhd_conserved_density(dptr(np.ascontiguousarray(pr.ravel())), ctypes.c_int64(n),
                                        ctypes.c_double(4.0 / 3.0), dptr(uc))
        dv = np.array([r.ref_sedov_cell_volume(ctypes.c_double(rf[i]), ctypes.c_double(rf[i + 1]),
                                               ctypes.c_double(theta[j]), ctypes.c_double(theta[j + 1]))
                       for i in range(n)])
        cons.append((uc.reshape(n, 5) * dv[:, None]).ravel())
    stages = 3
    gin = np.zeros((stages, T, 5))
    gout = np.zeros((stages, T, 5))
    for s in range(stages):
        gin[s] = [2.0 + 0.1 * s, 1.0, 0.0, 0.0, 0.1]
        gout[s] = [0.01, 0.1 + 0.01 * s, 0.0, 0.0, 1e-4]
    return {"T": np.array([T]), "ncells": np.array(ncells, np.int64), "theta": np.repeat(theta, 2)[1:-1].copy(),
            "radii": np.concatenate(radii), "u": np.concatenate(cons), "ghost_in": gin.ravel(),
            "ghost_out": gout.ravel(), "use_plm": np.array([use_plm])}


def sedov_dt(c) -> float:
    """0.3 of the smallest radial spacing (the driver's cfl * min spacing / c)."""
    nc = c["ncells"]
    off = np.concatenate([[0], np.cumsum(nc + 1)])
    return 0.3 * min(np.diff(c["radii"][off[j]:off[j + 1]]).min() for j in range(len(nc)))


def sedov_fixtures(o, r) -> dict[str, np.ndarray]:
    """One forward-Euler advance of every case through the reference's sedov::
    functions (with its intermediate arrays), and RK2 / RK3 runs of three
    steps composed with the reference's weighted_sum semantics."""
    out = {}
    for name in SEDOV_CASES:
        c = sedov_case(o, r, name)
        T = int(c["T"][0])
        nc = c["ncells"]
        C = int(nc.sum())
        F = C + T
        NP = int(sum(nc[j] + nc[j + 1] + 1 for j in range(T - 1)))
        dt = sedov_dt(c)
        plm = ctypes.c_int32(int(c["use_plm"][0]))
        args = (ctypes.c_int32(T), nc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), dptr(c["theta"]))
        T5 = 5 * T

        def step(rad, u, s, parts=None):
            ro_, uo_ = np.zeros(F), np.zeros(5 * C)
            gi = np.ascontiguousarray(c["ghost_in"][T5 * s: T5 * (s + 1)])
            go = np.ascontiguousarray(c["ghost_out"][T5 * s: T5 * (s + 1)])
            extra = [dptr(x) for x in parts] if parts else [None] * 4
            assert r.ref_sedov_advance(*args, dptr(rad), dptr(u), dptr(gi), dptr(go), ctypes.c_double(dt), plm,
                                       dptr(ro_), dptr(uo_), *extra) == 0
            return ro_, uo_

        parts = [np.zeros(5 * C), np.zeros(5 * C), np.zeros(6 * F), np.zeros(8 * NP)]
        ro, uo = step(c["radii"], c["u"], 0, parts)
        for k, v in c.items():
            out[f"sedov/{name}/{k}"] = v
        out[f"sedov/{name}/dt"] = np.array([dt])
        out[f"sedov/{name}/euler/radii"] = ro
        out[f"sedov/{name}/euler/u"] = uo
        for k, v in zip(("prim", "grad", "radial", "polar"), parts):
            out[f"sedov/{name}/euler/{k}"] = v
        for rk in (2, 3):
            rad, u = c["radii"].copy(), c["u"].copy()
            for _ in range(3):
                r0, u0 = rad, u
                r1_, u1 = step(r0, u0, 0)
                r2_, u2 = step(r1_, u1, 1)
                if rk == 2:
                    rad, u = r0 * (1 / 2) + r2_ * (1 / 2), u0 * (1 / 2) + u2 * (1 / 2)
                else:
                    r2_, u2 = r0 * (3 / 4) + r2_ * (1 / 4), u0 * (3 / 4) + u2 * (1 / 4)
                    r3_, u3 = step(r2_, u2, 2)
                    rad, u = r0 * (1 / 3) + r3_ * (2 / 3), u0 * (1 / 3) + u3 * (2 / 3)
            out[f"sedov/{name}/rk{rk}_3/radii"] = rad
            out[f"sedov/{name}/rk{rk}_3/u"] = u
    return out


def sedov_remesh_cases(r):
    """Tracks shaped to take each branch of sedov::remesh: a split of the most
    elongated cell, merges at the start, the end and inside (either
    neighbour), the inner-boundary drop (after which the reference recurses
    with the aspect bounds exchanged), and a track left alone."""
    rng = np.random.default_rng(77)
    dth = np.pi / 24
    # geometric radii of aspect dr / (r_c dtheta) = 1 everywhere
    q = (2 + dth) / (2 - dth)
    base = 1.0 * q ** np.arange(30)
    cases = []
    def add(name, rf, inner=1.0, amax=2.0, amin=0.5):
        cells = len(rf) - 1
        u = rng.uniform(0.5, 2.0, (cells, 5))
        cases.append((name, rf, u.ravel(), inner, amax, amin))
    add("unchanged", base.copy())
    rf = base.copy(); rf[5] = 0.5 * (rf[4] + rf[6]) + 0.45 * (rf[6] - rf[4]); add("split", rf, amax=1.6)
    rf = base.copy(); rf[1] = rf[0] + 0.1 * (rf[2] - rf[0]); add("merge_first", rf)
    rf = base.copy(); rf[-2] = rf[-1] - 0.1 * (rf[-1] - rf[-3]); add("merge_last", rf)
    rf = base.copy(); rf[7] = rf[6] + 0.05 * (rf[8] - rf[6]); add("merge_inner_left", rf)
    rf = base.copy(); rf[7] = rf[8] - 0.05 * (rf[8] - rf[6]); add("merge_inner_right", rf)
    rf = base.copy(); add("inner_drop", rf, inner=0.5 * (rf[1] + rf[2]))
    rf = base.copy(); add("inner_drop_wide_bounds", rf, inner=0.5 * (rf[0] + rf[1]), amax=50.0, amin=0.01)
    return cases


def sedov_remesh_fixture(r) -> dict[str, np.ndarray]:
    out = {}
    for name, rf, u, inner, amax, amin in sedov_remesh_cases(r):
        cells = len(rf) - 1
        ro, uo = np.zeros(cells + 2), np.zeros(5 * (cells + 1))
        m = r.ref_sedov_remesh.restype = ctypes.c_int64
        m = r.ref_sedov_remesh(ctypes.c_int64(cells), ctypes.c_double(0.3), ctypes.c_double(0.3 + np.pi / 24),
                               dptr(rf), dptr(u), ctypes.c_double(amax), ctypes.c_double(amin), ctypes.c_double(inner),
                               dptr(ro), dptr(uo))
        out[f"remesh/{name}/radii"] = rf
        out[f"remesh/{name}/u"] = u
        out[f"remesh/{name}/bounds"] = np.array([amax, amin, inner, 0.3, 0.3 + np.pi / 24])
        out[f"remesh/{name}/cells_out"] = np.array([m])
        out[f"remesh/{name}/radii_out"] = ro[:m + 1]
        out[f"remesh/{name}/u_out"] = uo[:5 * m]
    return out


def srhd_fixtures(o, r) -> dict[str, np.ndarray]:
    g = 4.0 / 3.0
    n = 4096
    prim = np.zeros(5 * n)
    cons = np.zeros(5 * n)
    # the recovery batch's distribution: rho 1e-4..1, p 1e-6..10, Lorentz factor 1..50
    o.oracle_srhd_seeded_zones(ctypes.c_uint64(4242), ctypes.c_int64(n), ctypes.c_double(1e-4), ctypes.c_double(1.0),
                               ctypes.c_double(1e-6), ctypes.c_double(10.0), ctypes.c_double(50.0), ctypes.c_double(g),
                               dptr(prim), dptr(cons))
    cref = np.zeros(5 * n)
    r.ref_srhd_conserved_density(dptr(prim), ctypes.c_int64(n), ctypes.c_double(g), dptr(cref))
    rec = np.zeros(5 * n)
    st = np.zeros(n, np.int32)
    r.ref_srhd_recover_primitive(dptr(cref), ctypes.c_int64(n), ctypes.c_double(g), ctypes.c_double(0.0), dptr(rec), iptr(st))
    out = {"srhd/prim": prim, "srhd/cons": cref, "srhd/recovered": rec, "srhd/status": st}
    # the reference's own known-answer states (src/physics_srhd.hpp:534-537)
    kat = np.array([[1.0, 0, 0, 0, 1.0], [1.5, 0, 0, 0, 1e3], [1.0, 0, 0, 0, 1.0], [5.7, 1.0, 2.0, 3.0, 5.0]]).ravel()
    kc = np.zeros_like(kat)
    r.ref_srhd_conserved_density(dptr(kat), ctypes.c_int64(4), ctypes.c_double(g), dptr(kc))
    kr = np.zeros_like(kat)
    ks = np.zeros(4, np.int32)
    r.ref_srhd_recover_primitive(dptr(kc), ctypes.c_int64(4), ctypes.c_double(g), ctypes.c_double(0.0), dptr(kr), iptr(ks))
    out.update({"srhd_kat/prim": kat, "srhd_kat/cons": kc, "srhd_kat/recovered": kr})
    m = 1000
    pl = prim[: 5 * m].copy()
    pr = prim[5 * m: 10 * m].copy()
    out["srhd_riemann/pl"] = pl
    out["srhd_riemann/pr"] = pr
    for hllc in (0, 1):
        for axis in (1, 2, 3):
            f = np.zeros(5 * m)
            assert r.ref_srhd_riemann(dptr(pl), dptr(pr), ctypes.c_int64(m), axis, ctypes.c_double(g), hllc, dptr(f)) == 0
            out[f"srhd_riemann/{'hllc' if hllc else 'hlle'}/axis{axis}"] = f
    return out


MHD_CASE = dict(N=8, modes=12, seed=3, gamma=5.0 / 3.0, cfl=0.3, theta=1.5)


def mhd_fixtures(o, r) -> dict[str, np.ndarray]:
    """advance_mhd_ct and two mhd3d RK2 steps on a seeded 8^3 cube, from the reference."""
    c = MHD_CASE
    N, modes, g = c["N"], c["modes"], c["gamma"]
    o.oracle_mhd_round_trip.restype = ctypes.c_int64
    r.ref_mhd_advance_ct.restype = ctypes.c_double
    table = np.zeros(11 * modes)
    assert o.oracle_mhd_mode_table(ctypes.c_uint64(c["seed"]), modes, dptr(table)) == 0
    half = np.sqrt(modes / 2.0)
    v_amp, a_amp = 0.5 / half, np.sqrt(2.0 / 10.0) / (2.0 * np.pi * half)
    uc = np.zeros(N ** 3 * 5)
    bf = [np.zeros((N + 1) * N * N) for _ in range(3)]
    o.oracle_mhd_initial(N, dptr(table), modes, ctypes.c_double(v_amp), ctypes.c_double(a_amp), ctypes.c_double(g),
                         dptr(uc), *[dptr(b) for b in bf])
    dl = 1.0 / N
    out = {"mhd/table": table, "mhd/amp": np.array([v_amp, a_amp]), "mhd/uc": uc.copy(),
           "mhd/params": np.array([N, g, c["cfl"], c["theta"]])}
    for k in range(3):
        out[f"mhd/bf{k + 1}"] = bf[k].copy()

    def step(u, b, t):
        u1 = np.zeros_like(u)
        b1 = [np.zeros_like(x) for x in b]
        t1 = r.ref_mhd_advance_ct(N, ctypes.c_double(t), dptr(u), *[dptr(x) for x in b], ctypes.c_double(dl),
                                  ctypes.c_double(c["cfl"]), ctypes.c_double(c["theta"]), dptr(u1), *[dptr(x) for x in b1])
        assert t1 > t
        return u1, b1, t1

    u1, b1, t1 = step(uc, bf, 0.0)
    out["mhd/step_uc"] = u1
    for k in range(3):
        out[f"mhd/step_bf{k + 1}"] = b1[k]
    out["mhd/step_time"] = np.array([t1])
    # examples/mhd3d.cpp RK2: each stage its own dt, states and times averaged
    u, b, t = uc.copy(), [x.copy() for x in bf], 0.0
    for _ in range(2):
        ua, ba, ta = step(u, b, t)
        ub, bb, tb = step(ua, ba, ta)
        u = u * 0.5 + ub * (1 - 0.5)
        b = [x * 0.5 + y * (1 - 0.5) for x, y in zip(b, bb)]
        t = t * 0.5 + tb * (1 - 0.5)
    out["mhd/rk2_uc"] = u
    for k in range(3):
        out[f"mhd/rk2_bf{k + 1}"] = b[k]
    out["mhd/rk2_time"] = np.array([t])
    # the reference's test_mhd states (src/physics_mhd.hpp:409-413)
    kat = np.array([[1.0, 0, 0, 0, 1.0, 0, 0, 0], [1.5, 0, 0, 0, 1e3, 0, 0, 0], [1.0, 0, 0, 0, 1.0, 0, 0, 0],
                    [5.7, 1.0, 2.0, 3.0, 5.0, 0, 0, 0], [5.7, 1.0, 2.0, 3.0, 5.0, 3.0, 2.0, 1.0]]).ravel()
    cons = np.zeros(5 * 5)
    back = np.zeros_like(kat)
    assert r.ref_mhd_round_trip(dptr(kat), ctypes.c_int64(5), ctypes.c_double(g), dptr(cons), dptr(back)) == 0
    out.update({"mhd_kat/prim": kat, "mhd_kat/cons": cons, "mhd_kat/back": back})
    return out


# Block shapes of the mhd_scheme_v2 fixtures: a non-cubic block and the same
# block extended by one cell on every side (the shapes its calls take).
V2_BLOCK = (3, 4, 5)
V2_GAMMA = 5.0 / 3.0   # the reference's scheme_mhd_v2 fixes gamma_law_index


def staggered(shape, axis, grow, side):
    return tuple(n + (grow if a == axis else side) for a, n in enumerate(shape))


def mhd_prims(rng, n, b=None):
    """n valid MHD primitive 8-tuples (rho, v, p, B); B drawn unless given."""
    p = np.zeros((n, 8))
    p[:, 0] = rng.uniform(0.5, 2.0, n)
    p[:, 1:4] = rng.uniform(-1.0, 1.0, (n, 3))
    p[:, 4] = rng.uniform(0.1, 2.0, n)
    p[:, 5:8] = rng.uniform(-1.0, 1.0, (n, 3)) if b is None else b
    return p


def mhd_conserved(p, g):
    d, v, pg, b = p[:, 0], p[:, 1:4], p[:, 4], p[:, 5:8]
    u = np.zeros((p.shape[0], 5))
    u[:, 0] = d
    u[:, 1:4] = d[:, None] * v
    u[:, 4] = 0.5 * d * (v * v).sum(1) + pg / (g - 1.0) + 0.5 * (b * b).sum(1)
    return u


def physics_fixtures(r) -> dict[str, np.ndarray]:
    """Pointwise iso2d and mhd physics (src/physics_iso2d.hpp:99-173,
    src/physics_mhd.hpp:216-390) on seeded points, by the reference's own
    functions."""
    out = {}
    rng = np.random.default_rng(2024)
    n = 96
    pl = np.stack([rng.uniform(0.5, 2.0, n), rng.uniform(-3, 3, n), rng.uniform(-3, 3, n)], 1).ravel()
    pr = np.stack([rng.uniform(0.5, 2.0, n), rng.uniform(-3, 3, n), rng.uniform(-3, 3, n)], 1).ravel()
    cs2 = np.exp(rng.uniform(np.log(1e-4), np.log(4.0), n))
    out["iso2d/pl"], out["iso2d/pr"], out["iso2d/cs2"] = pl, pr, cs2
    for axis in (1, 2):
        flux, outer, fastest, hlle = np.zeros(3 * n), np.zeros(2 * n), np.zeros(n), np.zeros(3 * n)
        r.ref_iso2d_pointwise(dptr(pl), dptr(pr), dptr(cs2), ctypes.c_int64(n), ctypes.c_uint32(axis), dptr(flux),
                              dptr(outer), dptr(fastest), dptr(hlle))
        out[f"iso2d/axis{axis}/flux"], out[f"iso2d/axis{axis}/outer"] = flux, outer
        out[f"iso2d/fastest"], out[f"iso2d/axis{axis}/hlle"] = fastest, hlle
    for g in (5.0 / 3.0, 1.4):
        tag = f"mhd_g{g:.4f}"
        a = mhd_prims(rng, n).ravel()
        b = mhd_prims(rng, n).ravel()
        bl = rng.uniform(-1.0, 1.0, n)
        out[f"{tag}/pl"], out[f"{tag}/pr"], out[f"{tag}/bl"] = a, b, bl
        for axis in (1, 2, 3):
            flux, cf2, fastest, hlle = np.zeros(5 * n), np.zeros(n), np.zeros(n), np.zeros(8 * n)
            r.ref_mhd_pointwise(dptr(a), ctypes.c_int64(n), ctypes.c_uint32(axis), ctypes.c_double(g), dptr(flux),
                                dptr(cf2), dptr(fastest))
            r.ref_mhd_riemann_hlle(dptr(a), dptr(b), dptr(bl), ctypes.c_int64(n), ctypes.c_uint32(axis),
                                   ctypes.c_double(g), dptr(hlle))
            out[f"{tag}/axis{axis}/flux"], out[f"{tag}/axis{axis}/cf2"] = flux, cf2
            out[f"{tag}/fastest"], out[f"{tag}/axis{axis}/hlle"] = fastest, hlle
        # recovery from conserved densities, with a few states the reference
        # rejects: negative pressure (energy below kinetic + magnetic) and
        # negative density
        prim = mhd_prims(rng, n)
        u = mhd_conserved(prim, g)
        u[5, 4] = 0.4 * (0.5 * u[5, 0] * (prim[5, 1:4] ** 2).sum() + 0.5 * (prim[5, 5:8] ** 2).sum())
        u[17, 4] = 0.0
        u[40, 0] = -u[40, 0]
        bc = np.ascontiguousarray(prim[:, 5:8]).ravel()
        u = u.ravel()
        back, status = np.zeros(8 * n), np.zeros(n, dtype=np.int32)
        r.ref_mhd_recover_primitive(dptr(u), dptr(bc), ctypes.c_int64(n), ctypes.c_double(g), dptr(back), iptr(status))
        assert status.sum() == 3, status
        out[f"{tag}/recover_u"], out[f"{tag}/recover_b"] = u, bc
        out[f"{tag}/recover_p"], out[f"{tag}/recover_status"] = back, status
    return out


def mhd_v2_fixtures(rv) -> dict[str, np.ndarray]:
    """mhd_scheme_v2's block calls (src/scheme_mhd_v2.cpp:75-278) on seeded
    blocks, by the reference's own code (oracle/_ref/libref_v2.so)."""
    out = {}
    rng = np.random.default_rng(77)
    c = V2_BLOCK
    m = tuple(x + 2 for x in c)
    size = lambda s: int(np.prod(s))  # noqa: E731
    i32 = [ctypes.c_int32(x) for x in c]
    m32 = [ctypes.c_int32(x) for x in m]
    out["v2/block"], out["v2/extended"] = np.array(c), np.array(m)
    # primitive_array: faces drawn, conserved from primitives holding the cells' mean fields
    bf = [rng.uniform(-1, 1, size(staggered(c, a, 1, 0))) for a in range(3)]
    b3 = [x.reshape(staggered(c, a, 1, 0)) for a, x in enumerate(bf)]
    bc = np.stack([0.5 * (b3[0][:-1] + b3[0][1:]), 0.5 * (b3[1][:, :-1] + b3[1][:, 1:]),
                   0.5 * (b3[2][:, :, :-1] + b3[2][:, :, 1:])], -1).reshape(-1, 3)
    uc = mhd_conserved(mhd_prims(rng, size(c), bc), V2_GAMMA).ravel()
    pc = np.zeros(8 * size(c))
    assert rv.ref_mhd_v2_primitive_array(*i32, dptr(uc), *[dptr(x) for x in bf], dptr(pc)) == 0
    out.update({"v2/prim/uc": uc, "v2/prim/bf1": bf[0], "v2/prim/bf2": bf[1], "v2/prim/bf3": bf[2], "v2/prim/pc": pc})
    # godunov_fluxes on the extended block
    pe = mhd_prims(rng, size(m)).ravel()
    bfe = [rng.uniform(-1, 1, size(staggered(m, a, -1, 0))) for a in range(3)]
    gf = [np.zeros(8 * size(staggered(m, a, -1, 0))) for a in range(3)]
    assert rv.ref_mhd_v2_godunov_fluxes(*m32, dptr(pe), *[dptr(x) for x in bfe], *[dptr(x) for x in gf]) == 0
    out.update({"v2/god/pc": pe, **{f"v2/god/bf{a + 1}": bfe[a] for a in range(3)},
                **{f"v2/god/gf{a + 1}": gf[a] for a in range(3)}})
    # electromotive_forces of those godunov data
    ee = [np.zeros(size(staggered(m, a, 0, -1))) for a in range(3)]
    assert rv.ref_mhd_v2_electromotive_forces(*m32, *[dptr(x) for x in gf], *[dptr(x) for x in ee]) == 0
    out.update({f"v2/emf/ee{a + 1}": ee[a] for a in range(3)})
    # updated_conserved_density with drawn godunov data (extended transversely)
    uc2 = mhd_conserved(mhd_prims(rng, size(c)), V2_GAMMA).ravel()
    gx = [rng.uniform(-1, 1, 8 * size(staggered(c, a, 1, 2))) for a in range(3)]
    uo = np.zeros_like(uc2)
    assert rv.ref_mhd_v2_updated_conserved_density(*i32, dptr(uc2), *[dptr(x) for x in gx], ctypes.c_double(0.013),
                                                   ctypes.c_double(0.1), dptr(uo)) == 0
    out.update({"v2/ucd/uc": uc2, **{f"v2/ucd/gf{a + 1}": gx[a] for a in range(3)}, "v2/ucd/out": uo,
                "v2/ucd/dt_dl": np.array([0.013, 0.1])})
    # curl of the block's own edges
    ek = [rng.uniform(-1, 1, size(staggered(c, a, 0, 1))) for a in range(3)]
    cf = [np.zeros(size(staggered(c, a, 1, 0))) for a in range(3)]
    assert rv.ref_mhd_v2_curl(*i32, *[dptr(x) for x in ek], ctypes.c_double(0.1), *[dptr(x) for x in cf]) == 0
    out.update({**{f"v2/curl/ee{a + 1}": ek[a] for a in range(3)}, **{f"v2/curl/cf{a + 1}": cf[a] for a in range(3)}})
    # updated_magnetic_flux_density with the extended block's edge EMFs
    bb = [rng.uniform(-1, 1, size(staggered(c, a, 1, 0))) for a in range(3)]
    ex = [rng.uniform(-1, 1, size(staggered(c, a, 2, 1))) for a in range(3)]
    bo = [np.zeros_like(x) for x in bb]
    assert rv.ref_mhd_v2_updated_magnetic_flux_density(*i32, *[dptr(x) for x in bb], *[dptr(x) for x in ex],
                                                       ctypes.c_double(0.013), ctypes.c_double(0.1),
                                                       *[dptr(x) for x in bo]) == 0
    out.update({**{f"v2/umfd/bf{a + 1}": bb[a] for a in range(3)}, **{f"v2/umfd/ee{a + 1}": ex[a] for a in range(3)},
                **{f"v2/umfd/out{a + 1}": bo[a] for a in range(3)}})
    return out


def main() -> None:
    if "--physics-only" in sys.argv:
        r, rv = load_reference(), load_reference_v2()
        if r is None or rv is None:
            raise SystemExit("oracle/_ref is missing: run `make -C oracle ref` where the reference is present")
        np.savez_compressed(HERE / "physics_golden.npz", **physics_fixtures(r), **mhd_v2_fixtures(rv))
        return
    o = load_oracle()
    r = load_reference()
    if r is None:
        raise SystemExit("oracle/_ref/libref.so is missing: run `make -C oracle ref` where the reference is present")
    fixtures = {}
    fixtures.update(minidisk_fixtures(o, r))
    fixtures.update(block_fixture(r))
    fixtures.update(plm_fixture(r))
    fixtures.update(binary_fixture(r))
    np.savez_compressed(HERE / "minidisk_golden.npz", **fixtures)
    np.savez_compressed(HERE / "srhd_golden.npz", **srhd_fixtures(o, r))
    np.savez_compressed(HERE / "mhd_golden.npz", **mhd_fixtures(o, r))
    np.savez_compressed(HERE / "two_body_golden.npz", **two_body_fixture(r))
    np.savez_compressed(HERE / "sedov_golden.npz", **sedov_fixtures(o, r), **sedov_remesh_fixture(r))
    rv = load_reference_v2()
    if rv is None:
        raise SystemExit("oracle/_ref/libref_v2.so is missing: run `make -C oracle ref`")
    np.savez_compressed(HERE / "physics_golden.npz", **physics_fixtures(r), **mhd_v2_fixtures(rv))
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
