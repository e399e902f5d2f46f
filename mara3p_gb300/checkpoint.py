"""Minidisk checkpoints in the reference's group layout.

The reference driver writes chkpt.%04d.h5 with the groups git_commit,
run_config, schedule/{checkpoint,time_series}/{next_due,count} and
solution/{iteration,time,conserved/<level:i-j>} (problems/minidisk.cpp:239-264,
problems/minidisk_io.cpp:56-114), each block the (n, n, 3) array of its
conserved tuples. HDF5 is not available here, so the same tree is a directory
chkpt.%04d/ of JSON files and raw little-endian float64 blocks; the C++ driver
(mara_minidisk) and these functions read and write the same format.
"""
from __future__ import annotations

import json
import math
import os
import shutil
from pathlib import Path

import numpy as np


def block_name(level: int, i: int, j: int) -> str:
    """mesh::format_block_index (src/mesh_block_index.hpp:361-375): "level:i-j",
    coordinates zero-padded to 1 + log10(2^level) digits."""
    width = int(1 + math.log10(1 << level))
    return f"{level}:{i:0{width}d}-{j:0{width}d}"


def read(path: str | os.PathLike) -> dict:
    """A checkpoint as a dict: run_config, schedule, iteration, time, git_commit
    and conserved, the whole mesh as the SoA array (3, N, N)."""
    p = Path(path)
    run_config = json.loads((p / "run_config.json").read_text())
    schedule = json.loads((p / "schedule.json").read_text())
    sol = json.loads((p / "solution.json").read_text())
    n, depth = int(run_config["block_size"]), int(run_config["depth"])
    nb = 1 << depth
    N = n * nb
    u = np.empty((3, N, N))
    for bi in range(nb):
        for bj in range(nb):
            f = p / "solution" / "conserved" / block_name(depth, bi, bj)
            b = np.fromfile(f, dtype="<f8")
            if b.size != n * n * 3:
                raise ValueError(f"{f}: {b.size} values, expected {n * n * 3}")
            u[:, bi * n:(bi + 1) * n, bj * n:(bj + 1) * n] = b.reshape(n, n, 3).transpose(2, 0, 1)
    return {"run_config": run_config, "schedule": schedule, "iteration": int(sol["iteration"]),
            "time": float(sol["time"]), "git_commit": (p / "git_commit").read_text(), "conserved": u}


def write(path: str | os.PathLike, run_config: dict, schedule: dict, iteration: int, time: float,
          conserved: np.ndarray, git_commit: str = "") -> None:
    """Write a checkpoint of the SoA state (3, N, N); run_config must hold
    block_size and depth. Written to path.partial, then renamed."""
    p = Path(path)
    n, depth = int(run_config["block_size"]), int(run_config["depth"])
    nb = 1 << depth
    u = np.asarray(conserved, dtype=np.float64)
    if u.shape != (3, n * nb, n * nb):
        raise ValueError(f"conserved has shape {u.shape}, expected {(3, n * nb, n * nb)}")
    tmp = Path(str(p) + ".partial")
    shutil.rmtree(tmp, ignore_errors=True)
    (tmp / "solution" / "conserved").mkdir(parents=True)
    (tmp / "git_commit").write_text(git_commit)
    (tmp / "run_config.json").write_text(json.dumps(run_config, indent=2) + "\n")
    (tmp / "schedule.json").write_text(json.dumps(schedule, indent=2) + "\n")
    (tmp / "solution.json").write_text(json.dumps({"iteration": int(iteration), "time": float(time)}, indent=2) + "\n")
    for bi in range(nb):
        for bj in range(nb):
            block = u[:, bi * n:(bi + 1) * n, bj * n:(bj + 1) * n].transpose(1, 2, 0)
            np.ascontiguousarray(block, dtype="<f8").tofile(tmp / "solution" / "conserved" / block_name(depth, bi, bj))
    shutil.rmtree(p, ignore_errors=True)
    tmp.rename(p)
