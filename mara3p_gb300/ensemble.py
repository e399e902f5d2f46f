"""Batched minidisk ensembles: many independent meshes advanced on one GPU.

The reference advances one minidisk mesh per process and folds steps on the
host (problems/minidisk.cpp:174-213). An `Ensemble` advances many members,
each with its own `SolverData` (mesh size, binary, Mach number, viscosity),
through libmara_gb300's ensemble entry points: one persistent launch per RK
stage over a device work-list of strip segments of all members, and one
replayed CUDA graph per RK step. Each member's state and clock equal those of
`minidisk.Run` on that member alone.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from ._capi import EnsembleConfig, MinidiskClock, MinidiskParams, check, lib
from .minidisk import DT_CFL, MIXED, SolverData, _stream, initial_conserved

STRIP_COLUMNS = {1: 28, 2: 60}      # interior columns of a sweep strip, by columns per lane
MESH_SIZES = (128, 256, 512, 1024)
_i32p = ctypes.POINTER(ctypes.c_int32)


def plan(sizes, chunks: int, cols_per_lane: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """The work-list of meshes of the given sizes cut into `chunks` chunks:
    items (k, 4) = (member, strip, row begin, row end) and chunk offsets
    (chunks + 1), for the 1- or 2-column sweep. Host only."""
    s = np.ascontiguousarray(sizes, dtype=np.int32)
    width = STRIP_COLUMNS.get(cols_per_lane, 0)
    n = lib.mara_minidisk_ensemble_plan(s.ctypes.data_as(_i32p), len(s), chunks, width, None, 0, None)
    if n < 0:
        check(1, "mara_minidisk_ensemble_plan")
    items = np.zeros((n, 4), np.int32)
    first = np.zeros(chunks + 1, np.int32)
    got = lib.mara_minidisk_ensemble_plan(s.ctypes.data_as(_i32p), len(s), chunks, width,
                                          items.ctypes.data_as(_i32p), n, first.ctypes.data_as(_i32p))
    assert got == n
    return items, first


def seeded_members(seed: int, count: int, base: SolverData, sizes=MESH_SIZES) -> list[SolverData]:
    """Per-member solver data drawn by seed: mesh size from `sizes` (64^2
    blocks), mass ratio U(0.1, 1), eccentricity U(0, 0.5), Mach number
    U(10, 30) and viscosity U(1e-4, 1e-3); everything else from `base`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(sizes))
        block = 64 if n % 64 == 0 and n >= 64 else n
        depth = int(round(math.log2(n // block)))
        out.append(base.with_(block_size=block, depth=depth, mass_ratio=float(rng.uniform(0.1, 1.0)),
                              eccentricity=float(rng.uniform(0.0, 0.5)), mach_number=float(rng.uniform(10.0, 30.0)),
                              nu=float(rng.uniform(1e-4, 1e-3))))
    return out


class Ensemble:
    """`members` advanced together on the current CUDA device.

    states: one (3, N, N) float64 CUDA tensor per member (SoA, the layout of
    `minidisk.Run`); None creates the seeded initial states. The tensors are
    updated in place and must outlive the ensemble. autotune: 0 default launch
    shape, 1 tune once per set of mesh sizes in the process, 2 always tune."""

    def __init__(self, members: list[SolverData], states: list[torch.Tensor] | None = None, *, time: float = 0.0,
                 rk_order: int = 2, precision: int = MIXED, dt_mode: int = DT_CFL, autotune: int = 1,
                 seed: int = 0, amplitude: float = 0.01, device: str | torch.device = "cuda"):
        self.members = list(members)
        count = len(self.members)
        if states is None:
            states = [initial_conserved(sd, seed=seed + m, amplitude=amplitude, device=device)
                      for m, sd in enumerate(self.members)]
        self.states = list(states)
        for sd, u in zip(self.members, self.states):
            n = sd.cells_per_side
            if u.dtype != torch.float64 or not u.is_cuda or not u.is_contiguous() or u.numel() != 3 * n * n:
                raise ValueError("each state must be a contiguous float64 CUDA tensor of 3*N*N values")
        self.rk_order, self.precision, self.dt_mode = rk_order, precision, dt_mode
        dev = self.states[0].device if count else torch.device(device)
        self.clocks = torch.zeros(max(count, 1) * ctypes.sizeof(MinidiskClock), dtype=torch.uint8, device=dev)
        self._params = (MinidiskParams * max(count, 1))(*[sd.to_c() for sd in self.members])
        self._ptrs = (ctypes.c_void_p * max(count, 1))(*[u.data_ptr() for u in self.states])
        torch.cuda.synchronize(dev)
        self._handle = ctypes.c_void_p()
        check(lib.mara_minidisk_ensemble_create(self._params, count, self._ptrs, self.clocks.data_ptr(), rk_order,
                                                precision, dt_mode, autotune, ctypes.byref(self._handle)),
              "mara_minidisk_ensemble_create")
        check(lib.mara_minidisk_ensemble_clock_init(self._handle, time, _stream()), "mara_minidisk_ensemble_clock_init")

    # ------------------------------------------------------------------
    def advance(self, steps: int) -> None:
        check(lib.mara_minidisk_ensemble_advance(self._handle, steps, _stream()), "mara_minidisk_ensemble_advance")

    @property
    def config(self) -> dict:
        c = EnsembleConfig()
        check(lib.mara_minidisk_ensemble_get_config(self._handle, ctypes.byref(c)), "get_config")
        return {f: getattr(c, f) for f, _ in EnsembleConfig._fields_}

    def set_config(self, **kw) -> None:
        cfg = self.config
        cfg.update(kw)
        c = EnsembleConfig(**cfg)
        check(lib.mara_minidisk_ensemble_set_config(self._handle, ctypes.byref(c)), "set_config")

    def tune(self) -> dict:
        check(lib.mara_minidisk_ensemble_tune(self._handle), "tune")
        return self.config

    def stage_times(self, reps: int = 5) -> list[float]:
        """Median milliseconds of each stage launch over all members (mixed
        precision; the timing launches write only scratch)."""
        ms = (ctypes.c_double * self.rk_order)()
        check(lib.mara_minidisk_ensemble_stage_times(self._handle, reps, ms), "stage_times")
        return list(ms)

    def clock_states(self) -> list[MinidiskClock]:
        raw = self.clocks.cpu().numpy().tobytes()
        size = ctypes.sizeof(MinidiskClock)
        return [MinidiskClock.from_buffer_copy(raw[m * size:(m + 1) * size]) for m in range(len(self.members))]

    @property
    def cells(self) -> int:
        return sum(sd.cells_per_side ** 2 for sd in self.members)

    def close(self) -> None:
        if getattr(self, "_handle", None) and self._handle.value:
            check(lib.mara_minidisk_ensemble_destroy(self._handle), "mara_minidisk_ensemble_destroy")
            self._handle = ctypes.c_void_p()

    def __enter__(self) -> "Ensemble":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
