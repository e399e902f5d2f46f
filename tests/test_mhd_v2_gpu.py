"""GPU parity of the reference's split MHD block API (mhd_scheme_v2) and of
the pointwise iso2d / mhd physics, through the C ABI, against outputs of the
reference's own code (tests/golden/physics_golden.npz, made by
tests/golden/make_golden.py from oracle/_ref).

Tolerance: FP64, relative 1e-13 of each array's scale (FMA contraction is the
only difference); statuses and the pure averaging / differencing operations
(face_to_cell, edge EMFs, curl) exact to that bound as well."""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
RTOL = 1e-13


@pytest.fixture(scope="module")
def g():
    return dict(np.load(Path(__file__).resolve().parent / "golden" / "physics_golden.npz"))


@pytest.fixture(scope="module")
def capi():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mara3p_gb300 import _capi
    return _capi


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def zeros(n, dtype=torch.float64):
    return torch.zeros(int(n), dtype=dtype, device="cuda")


def close(got, ref, rtol=RTOL):
    got = got.cpu().numpy().ravel() if isinstance(got, torch.Tensor) else np.asarray(got).ravel()
    ref = np.asarray(ref).ravel()
    scale = max(np.abs(ref).max(), 1e-300)
    err = np.abs(got - ref).max() / scale
    assert err <= rtol, err


def stream():
    return torch.cuda.current_stream().cuda_stream


def shapes(g):
    c = tuple(int(x) for x in g["v2/block"])
    m = tuple(int(x) for x in g["v2/extended"])
    stag = lambda s, a, grow, side: tuple(n + (grow if k == a else side) for k, n in enumerate(s))  # noqa: E731
    return c, m, stag


def test_v2_primitive_array(capi, g):
    c, _, _ = shapes(g)
    pc = zeros(8 * np.prod(c))
    fails = torch.zeros(1, dtype=torch.int64, device="cuda")
    args = [dev(g[k]) for k in ("v2/prim/uc", "v2/prim/bf1", "v2/prim/bf2", "v2/prim/bf3")]
    capi.check(capi.lib.mara_mhd_v2_primitive_array(*c, *[a.data_ptr() for a in args], 5.0 / 3.0, pc.data_ptr(),
                                                    fails.data_ptr(), stream()))
    close(pc, g["v2/prim/pc"])
    assert int(fails.item()) == 0


def test_v2_godunov_fluxes_and_emfs(capi, g):
    _, m, stag = shapes(g)
    pe = dev(g["v2/god/pc"])
    bf = [dev(g[f"v2/god/bf{a + 1}"]) for a in range(3)]
    gf = [zeros(8 * np.prod(stag(m, a, -1, 0))) for a in range(3)]
    capi.check(capi.lib.mara_mhd_v2_godunov_fluxes(*m, pe.data_ptr(), *[b.data_ptr() for b in bf], 5.0 / 3.0,
                                                   *[x.data_ptr() for x in gf], stream()))
    for a in range(3):
        close(gf[a], g[f"v2/god/gf{a + 1}"])
    # the edge EMFs of the reference's godunov data
    gref = [dev(g[f"v2/god/gf{a + 1}"]) for a in range(3)]
    ee = [zeros(np.prod(stag(m, a, 0, -1))) for a in range(3)]
    capi.check(capi.lib.mara_mhd_v2_electromotive_forces(*m, *[x.data_ptr() for x in gref],
                                                         *[x.data_ptr() for x in ee], stream()))
    for a in range(3):
        close(ee[a], g[f"v2/emf/ee{a + 1}"])


def test_v2_updated_conserved_density(capi, g):
    c, _, _ = shapes(g)
    dt, dl = (float(x) for x in g["v2/ucd/dt_dl"])
    uc = dev(g["v2/ucd/uc"])
    gf = [dev(g[f"v2/ucd/gf{a + 1}"]) for a in range(3)]
    out = torch.empty_like(uc)
    capi.check(capi.lib.mara_mhd_v2_updated_conserved_density(*c, uc.data_ptr(), *[x.data_ptr() for x in gf], dt, dl,
                                                              out.data_ptr(), stream()))
    close(out, g["v2/ucd/out"])


def test_v2_curl_and_magnetic_flux_update(capi, g):
    c, _, stag = shapes(g)
    dt, dl = (float(x) for x in g["v2/ucd/dt_dl"])
    ee = [dev(g[f"v2/curl/ee{a + 1}"]) for a in range(3)]
    cf = [zeros(np.prod(stag(c, a, 1, 0))) for a in range(3)]
    capi.check(capi.lib.mara_mhd_v2_curl(*c, *[x.data_ptr() for x in ee], dl, *[x.data_ptr() for x in cf], stream()))
    for a in range(3):
        close(cf[a], g[f"v2/curl/cf{a + 1}"])
    bf = [dev(g[f"v2/umfd/bf{a + 1}"]) for a in range(3)]
    ex = [dev(g[f"v2/umfd/ee{a + 1}"]) for a in range(3)]
    bo = [torch.empty_like(b) for b in bf]
    capi.check(capi.lib.mara_mhd_v2_updated_magnetic_flux_density(*c, *[x.data_ptr() for x in bf],
                                                                  *[x.data_ptr() for x in ex], dt, dl,
                                                                  *[x.data_ptr() for x in bo], stream()))
    for a in range(3):
        close(bo[a], g[f"v2/umfd/out{a + 1}"])


def test_v2_rejects_bad_shapes(capi):
    assert capi.lib.mara_mhd_v2_godunov_fluxes(1, 4, 4, None, None, None, None, 5.0 / 3.0, None, None, None,
                                               None) == 1
    assert b"two cells per axis" in capi.lib.mara_last_error()
    assert capi.lib.mara_mhd_v2_curl(3, 0, 3, None, None, None, 0.1, None, None, None, None) == 1


@pytest.mark.parametrize("gamma", [5.0 / 3.0, 1.4])
def test_mhd_pointwise(capi, g, gamma):
    tag = f"mhd_g{gamma:.4f}"
    n = g[f"{tag}/bl"].size
    pl, pr, bl = dev(g[f"{tag}/pl"]), dev(g[f"{tag}/pr"]), dev(g[f"{tag}/bl"])
    fastest = zeros(n)
    capi.check(capi.lib.mara_mhd_fastest_speed(pl.data_ptr(), n, gamma, fastest.data_ptr(), stream()))
    close(fastest, g[f"{tag}/fastest"])
    for axis in (1, 2, 3):
        f, cf2, hlle = zeros(5 * n), zeros(n), zeros(8 * n)
        capi.check(capi.lib.mara_mhd_flux(pl.data_ptr(), n, axis, gamma, f.data_ptr(), stream()))
        capi.check(capi.lib.mara_mhd_fast_speed_squared(pl.data_ptr(), n, axis, gamma, cf2.data_ptr(), stream()))
        capi.check(capi.lib.mara_mhd_riemann_hlle(pl.data_ptr(), pr.data_ptr(), bl.data_ptr(), n, axis, gamma,
                                                  hlle.data_ptr(), stream()))
        close(f, g[f"{tag}/axis{axis}/flux"])
        close(cf2, g[f"{tag}/axis{axis}/cf2"])
        close(hlle, g[f"{tag}/axis{axis}/hlle"])
    # recovery, with the three states the reference rejects
    u, b = dev(g[f"{tag}/recover_u"]), dev(g[f"{tag}/recover_b"])
    p = zeros(8 * n)
    status = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    fails = torch.zeros(1, dtype=torch.int64, device="cuda")
    capi.check(capi.lib.mara_mhd_recover_primitive(u.data_ptr(), b.data_ptr(), n, gamma, p.data_ptr(),
                                                   status.data_ptr(), fails.data_ptr(), stream()))
    ref_status = g[f"{tag}/recover_status"]
    assert np.array_equal(status.cpu().numpy(), ref_status)
    assert int(fails.item()) == int(ref_status.sum())
    ok = np.repeat(ref_status == 0, 8)
    close(p.cpu().numpy()[ok], g[f"{tag}/recover_p"][ok])
    # conserved_density inverts the recovery of the accepted states
    uu = zeros(5 * n)
    capi.check(capi.lib.mara_mhd_conserved_density(p.data_ptr(), n, gamma, uu.data_ptr(), stream()))
    okc = np.repeat(ref_status == 0, 5)
    close(uu.cpu().numpy()[okc], g[f"{tag}/recover_u"][okc], rtol=1e-12)


def test_iso2d_pointwise(capi, g):
    pl, pr, cs2 = dev(g["iso2d/pl"]), dev(g["iso2d/pr"]), dev(g["iso2d/cs2"])
    n = g["iso2d/cs2"].size
    fastest = zeros(n)
    capi.check(capi.lib.mara_iso2d_fastest_wavespeed(pl.data_ptr(), cs2.data_ptr(), n, fastest.data_ptr(), stream()))
    close(fastest, g["iso2d/fastest"])
    for axis in (1, 2):
        f, outer, hlle = zeros(3 * n), zeros(2 * n), zeros(3 * n)
        capi.check(capi.lib.mara_iso2d_flux(pl.data_ptr(), cs2.data_ptr(), n, axis, f.data_ptr(), stream()))
        capi.check(capi.lib.mara_iso2d_outer_wavespeeds(pl.data_ptr(), cs2.data_ptr(), n, axis, outer.data_ptr(),
                                                        stream()))
        capi.check(capi.lib.mara_iso2d_riemann_hlle(pl.data_ptr(), pr.data_ptr(), cs2.data_ptr(), n, axis,
                                                    hlle.data_ptr(), stream()))
        close(f, g[f"iso2d/axis{axis}/flux"])
        close(outer, g[f"iso2d/axis{axis}/outer"])
        close(hlle, g[f"iso2d/axis{axis}/hlle"])
    assert capi.lib.mara_iso2d_flux(pl.data_ptr(), cs2.data_ptr(), n, 3, None, None) == 1


def test_pointwise_empty_batches(capi):
    assert capi.lib.mara_mhd_flux(None, 0, 1, 5.0 / 3.0, None, None) == 0
    assert capi.lib.mara_iso2d_riemann_hlle(None, None, None, 0, 1, None, None) == 0
    assert capi.lib.mara_mhd_recover_primitive(None, None, 0, 5.0 / 3.0, None, None, None, None) == 0
