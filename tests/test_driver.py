"""The C++17 minidisk driver (problems/minidisk.cpp's main loop over the C
ABI) and the checkpoint format. CPU tests cover the configuration and the
checkpoint reader/writer; GPU tests run the driver: its state against the
oracle, its checkpoints and a restart that continues bit for bit."""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mara3p_gb300 import checkpoint

ROOT = Path(__file__).resolve().parents[1]
DRIVER = ROOT / "mara3p_gb300" / "mara_minidisk"


def run_driver(*args, check=True):
    if not DRIVER.exists():
        pytest.fail("the driver is not built: run __graft_entry__.build()")
    res = subprocess.run([str(DRIVER), *args], capture_output=True, text=True, timeout=600)
    if check and res.returncode != 0:
        raise AssertionError(res.stdout + res.stderr)
    return res


def test_dry_run_prints_the_reference_template_with_overrides():
    out = run_driver("dry=1", "block_size=32", "depth=3", "fold=10", "mach_number=25").stdout
    cfg = dict(re.findall(r"^\t(\w+) \.+ ?(.*)$", out, flags=re.M))
    # the reference's template keys and defaults (problems/minidisk.hpp:99-122)
    assert cfg["block_size"] == "32" and cfg["depth"] == "3" and cfg["fold"] == "10" and cfg["mach_number"] == "25"
    assert cfg["domain_radius"] == "1.5" and cfg["sink_rate"] == "1e3" and cfg["cpi"] == "0.1"
    assert cfg["orbits"] == "100.0" and cfg["outdir"] == "."
    for key in ("omega_frame", "nu", "eccentricity", "mass_ratio", "softening_length", "sink_radius",
                "buffer_rate", "buffer_scale", "cfl", "threads", "restart"):
        assert key in cfg


@pytest.mark.parametrize("arg,msg", [("bogus=1", "unknown configuration key"), ("block_size=abc", "expects int"),
                                     ("cfl=", "expects double"), ("precision=fp16", "fp64 or mixed"),
                                     ("nothing", "key=value"), ("mach_number=-1", "mach_number")])
def test_bad_arguments_are_rejected(arg, msg):
    res = run_driver("dry=1", arg, check=False)
    assert res.returncode == 1
    assert msg in res.stderr


def test_block_names_follow_the_reference_format():
    assert checkpoint.block_name(0, 0, 0) == "0:0-0"
    assert checkpoint.block_name(2, 1, 3) == "2:1-3"
    assert checkpoint.block_name(4, 3, 15) == "4:03-15"
    assert checkpoint.block_name(6, 5, 63) == "6:05-63"
    assert checkpoint.block_name(10, 7, 1023) == "10:0007-1023"


def test_checkpoint_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    u = rng.standard_normal((3, 64, 64))
    cfg = {"block_size": 16, "depth": 2, "cfl": 0.3}
    sch = {"checkpoint": {"next_due": 1.25, "count": 3}, "time_series": {"next_due": 0.0, "count": 0}}
    checkpoint.write(tmp_path / "chkpt.0003", cfg, sch, 17, 0.75, u, "abc")
    got = checkpoint.read(tmp_path / "chkpt.0003")
    assert np.array_equal(got["conserved"], u)
    assert got["iteration"] == 17 and got["time"] == 0.75 and got["schedule"] == sch and got["git_commit"] == "abc"
    names = sorted(f.name for f in (tmp_path / "chkpt.0003" / "solution" / "conserved").iterdir())
    assert names == sorted(checkpoint.block_name(2, i, j) for i in range(4) for j in range(4))
    # one block holds the (n, n, 3) conserved tuples of its cells
    b = np.fromfile(tmp_path / "chkpt.0003" / "solution" / "conserved" / "2:1-2", "<f8").reshape(16, 16, 3)
    assert np.array_equal(b, u[:, 16:32, 32:48].transpose(1, 2, 0))


SMALL = ["block_size=32", "depth=1", "domain_radius=4.0", "softening_length=0.05", "sink_radius=0.05",
         "sink_rate=10", "nu=1e-3", "mach_number=10"]


@pytest.mark.gpu
def test_driver_matches_the_oracle_and_prints_the_reference_lines(tmp_path, oracle):
    from oracle.oracle import MinidiskParams, dptr
    orbits = 0.002
    # cpi = orbits: a checkpoint at t = 0 and one when the run ends (side_effects, minidisk.cpp:239-264)
    res = run_driver(*SMALL, f"orbits={orbits}", f"cpi={orbits}", f"outdir={tmp_path}")
    lines = re.findall(r"^\[(\d{6})\] orbit=(\S+) kzps=(\S+)$", res.stdout, flags=re.M)
    assert lines, res.stdout
    assert [int(l[0]) for l in lines] == list(range(1, len(lines) + 1))
    assert float(lines[-1][1]) >= orbits
    # checkpoints: at t = 0 (cpi due) and after the loop
    first = checkpoint.read(tmp_path / "chkpt.0000")
    last = checkpoint.read(tmp_path / "chkpt.0001")
    assert first["iteration"] == 0 and last["iteration"] == len(lines)
    # the same forward-Euler steps on the oracle (the reference's scheme, theta = 2)
    p = MinidiskParams(block_size=32, depth=1, omega_frame=1.0, mach_number=10.0, nu=1e-3, domain_radius=4.0,
                       softening_length=0.05, eccentricity=0.0, mass_ratio=1.0, sink_radius=0.05, sink_rate=10.0,
                       buffer_rate=1e2, buffer_scale=0.2, cfl=0.3, plm_theta=2.0)
    u = np.ascontiguousarray(first["conserved"])
    oracle.oracle_minidisk_advance.restype = ctypes.c_double
    t = oracle.oracle_minidisk_advance(ctypes.byref(p), dptr(u), ctypes.c_double(0.0), len(lines), 1, 0, 4)
    assert abs(t - last["time"]) <= 1e-14 * t
    err = np.abs(u - last["conserved"]).sum() / np.abs(u).sum()
    assert err < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restart_continues_bit_for_bit(tmp_path, precision):
    args = [*SMALL, "fold=4", "orbits=0.003", "cpi=0.0015", f"precision={precision}", "perturbation=0.01", "seed=7"]
    run_driver(*args, f"outdir={tmp_path / 'a'}")
    ckpts = sorted(p.name for p in (tmp_path / "a").iterdir())
    assert ckpts[0] == "chkpt.0000" and len(ckpts) >= 3
    mid = tmp_path / "a" / ckpts[1]
    run_driver(f"restart={mid}", f"outdir={tmp_path / 'b'}")
    a = checkpoint.read(tmp_path / "a" / ckpts[-1])
    b = checkpoint.read(tmp_path / "b" / ckpts[-1])
    assert a["iteration"] == b["iteration"] and a["time"] == b["time"]
    assert np.array_equal(a["conserved"], b["conserved"])
    assert b["run_config"]["precision"] == precision and b["run_config"]["fold"] == 4


@pytest.mark.gpu
def test_graph_replay_equals_direct_launches(tmp_path):
    args = [*SMALL, "fold=3", "orbits=0.002", "cpi=0.002", "precision=mixed", "dt=cfl", "rk=2"]
    run_driver(*args, "graph=1", f"outdir={tmp_path / 'g'}")
    run_driver(*args, "graph=0", f"outdir={tmp_path / 'd'}")
    g = checkpoint.read(tmp_path / "g" / "chkpt.0001")
    d = checkpoint.read(tmp_path / "d" / "chkpt.0001")
    assert np.array_equal(g["conserved"], d["conserved"]) and g["time"] == d["time"]


def read_time_series(path):
    rows = [list(map(float, line.split())) for line in open(path) if not line.startswith("#")]
    return np.array(rows)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_time_series_rows_and_mass_balance(tmp_path, precision):
    # tsi = cpi: a sample (and a checkpoint) at t = 0 and every 0.001 orbits
    args = [*SMALL, "fold=2", "orbits=0.003", "cpi=0.001", "tsi=0.001", f"precision={precision}", "rk=2",
            "perturbation=0.01", "seed=3", f"outdir={tmp_path}"]
    run_driver(*args)
    ts = read_time_series(tmp_path / "time_series.dat")
    assert ts.shape[1] == 2 + 16 + 16 + 2 + 4
    assert len(ts) >= 3 and np.all(np.diff(ts[:, 0]) > 0)
    assert np.all(ts[0, 2:34] == 0.0)                      # nothing integrated at t = 0
    # a = 1, e = 0 (e is a square root of a rounding-level difference, so ~1e-8)
    assert np.allclose(ts[:, 34], 1.0, rtol=1e-12) and np.allclose(ts[:, 35], 0.0, atol=1e-7)
    # the disk mass changes by the integrated buffer and sink rates
    ck = sorted(p.name for p in tmp_path.iterdir() if p.name.startswith("chkpt."))
    first, last = checkpoint.read(tmp_path / ck[0]), checkpoint.read(tmp_path / ck[-2])
    N = first["conserved"].shape[1]
    dl = 2 * 4.0 / N
    row = ts[np.argmin(np.abs(ts[:, 0] - last["time"]))]
    assert row[0] == last["time"]
    I = row[2:18]
    dm = (last["conserved"][0].sum() - first["conserved"][0].sum()) * dl * dl
    scale = abs(I[10]) + abs(I[0]) + abs(I[1])
    assert abs(dm - (I[10] - I[0] - I[1])) <= (1e-9 if precision == "fp64" else 1e-4) * scale


@pytest.mark.gpu
def test_time_series_continues_across_restart(tmp_path):
    args = [*SMALL, "fold=2", "orbits=0.003", "cpi=0.0015", "tsi=0.0005", "precision=mixed", "rk=2"]
    run_driver(*args, f"outdir={tmp_path / 'a'}")
    ckpts = sorted(p.name for p in (tmp_path / "a").iterdir() if p.name.startswith("chkpt."))
    run_driver(f"restart={tmp_path / 'a' / ckpts[1]}", f"outdir={tmp_path / 'b'}")
    a = read_time_series(tmp_path / "a" / "time_series.dat")
    b = read_time_series(tmp_path / "b" / "time_series.dat")
    # the restarted run writes the samples after its checkpoint: the same times and
    # iterations as the straight run's, and the same integrals up to the order of the
    # device's FP64 atomic sums
    assert len(b) >= 1
    tail = a[-len(b):]
    assert np.array_equal(tail[:, :2], b[:, :2])
    assert np.allclose(tail[:, 2:], b[:, 2:], rtol=1e-10, atol=1e-14)
