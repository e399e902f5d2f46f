"""Host-side mirror of the reference's spherical-track SRHD scheme
(src/scheme_sedov2d.hpp, driven by problems/sedov2d.cpp).

`Tracks` holds a set of radial tracks resident on one GPU in CSR form (see
include/mara_gb300.h): face radii, polar bounds and conserved volume
integrals. `advance` is the driver's RK step (control::advance_runge_kutta of
the forward-Euler advance); `stage` runs one forward-Euler advance and can
return the scheme's intermediate arrays (sedov::recover_primitive,
radial_gradient, radial_godunov_data, polar_godunov_data) for parity checks.
`generate_radial_track` is sedov::generate_radial_track. Every call goes
through libmara_gb300.so; errors raise MaraError.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from ._capi import MaraError, check, lib

GAMMA = 4.0 / 3.0


def generate_radial_track(r0: float, r1: float, theta0: float, theta1: float, aspect: float) -> np.ndarray:
    """Face radii of a log-spaced track (scheme_sedov2d.cpp:108-129):
    int(pi / (theta1 - theta0) / aspect) faces from r0 to r1."""
    n = int(math.pi / (theta1 - theta0) / aspect)
    a, b = math.log10(r0), math.log10(r1)
    return np.array([10.0 ** (a + (b - a) * float(i) / float(n - 1)) for i in range(n)])


def conserved_density(prim: np.ndarray, gamma: float = GAMMA) -> np.ndarray:
    """srhd::conserved_density (src/physics_srhd.hpp:291-304), c = 1, of
    (n, 5) primitives (rho, u1, u2, u3, p) with four-velocity components."""
    rho, uu, p = prim[:, 0], prim[:, 1:4], prim[:, 4]
    W = np.sqrt(1.0 + (uu ** 2).sum(1))
    D = rho * W
    h = (rho + p * (1.0 + 1.0 / (gamma - 1.0))) / rho
    out = np.empty_like(prim)
    out[:, 0] = D
    out[:, 1:4] = (D * h)[:, None] * uu
    out[:, 4] = D * (h * W - 1.0) - p
    return out


def cell_volumes(radii: np.ndarray, theta0: float, theta1: float) -> np.ndarray:
    """sedov::cell_volume of consecutive faces of one track."""
    dcost = -(math.cos(theta1) - math.cos(theta0))
    return 2.0 * math.pi * (radii[1:] ** 3 - radii[:-1] ** 3) / 3.0 * dcost


def seeded_tracks(track_count: int, aspect: float = 2.0, r0: float = 1.0, r1: float = 1.8, seed: int = 0,
                  focus: float = 0.0):
    """Tracks laid out as problems/sedov2d.cpp:528-561 lays them out (polar
    bounds from its "focus" spacing, each track from generate_radial_track
    between r0 and r1) holding a seeded relativistic wind with a hot core:
    rho ~ r^-2 (+-5%), radial four-velocity 0.4 (+-0.02), polar 0 (+-0.01),
    pressure 1e-3 rho plus 0.3 inside r < (r0 + r1) / 2.
    Returns (ncells, theta (T, 2), radii, u (cells, 5))."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, track_count + 1)
    theta = np.pi * (x + focus * (x - 1) * x) / (1 + 2 * focus * (x - 1) * x)
    ncells, radii, cons = [], [], []
    for j in range(track_count):
        rf = generate_radial_track(r0, r1, theta[j], theta[j + 1], aspect)
        rc = 0.5 * (rf[:-1] + rf[1:])
        n = len(rc)
        pr = np.zeros((n, 5))
        pr[:, 0] = rc ** -2 * (1 + 0.05 * rng.uniform(-1, 1, n))
        pr[:, 1] = 0.4 + 0.02 * rng.uniform(-1, 1, n)
        pr[:, 2] = 0.01 * rng.uniform(-1, 1, n)
        pr[:, 4] = 1e-3 * pr[:, 0] + np.where(rc < 0.5 * (r0 + r1), 0.3, 0.0)
        cons.append(conserved_density(pr) * cell_volumes(rf, theta[j], theta[j + 1])[:, None])
        ncells.append(n)
        radii.append(rf)
    return (np.array(ncells, np.int64), np.stack([theta[:-1], theta[1:]], 1), np.concatenate(radii),
            np.concatenate(cons))


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class Tracks:
    """Radial tracks on the GPU. ncells[j] cells on track j, theta (T, 2)
    polar bounds, radii the concatenated face radii, u the conserved volume
    integrals as (cells, 5) tuples (the reference's layout) or (5, cells)."""

    def __init__(self, ncells, theta, radii, u, device="cuda"):
        ncells = np.asarray(ncells, dtype=np.int64)
        self.T = len(ncells)
        self.cells = int(ncells.sum())
        if np.any(ncells < 2):
            raise ValueError("every track needs at least 2 cells")
        co = np.concatenate([[0], np.cumsum(ncells)]).astype(np.int64)
        self._ncells = ncells
        self.co = torch.from_numpy(co).to(device)
        self.theta = torch.from_numpy(np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(-1))).to(device)
        radii = np.asarray(radii, dtype=np.float64)
        if radii.size != self.cells + self.T:
            raise ValueError("radii must hold ncells[j] + 1 faces per track")
        self.radii = torch.from_numpy(radii.copy()).to(device)
        u = np.asarray(u, dtype=np.float64)
        soa = u.reshape(self.cells, 5).T if u.shape != (5, self.cells) else u
        self.u = torch.from_numpy(np.ascontiguousarray(soa)).to(device)
        nbytes = lib.mara_sedov_workspace_bytes(self.T, self.cells)
        if nbytes < 0:
            check(1, "mara_sedov_workspace_bytes")
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=device)
        self.failures = torch.zeros(1, dtype=torch.int32, device=device)

    @property
    def ncells(self) -> np.ndarray:
        """Cells per track (host copy, read from the device offsets after a
        remesh the first time it is asked for)."""
        if self._ncells is None:
            co = self.co.cpu().numpy()
            self._ncells = co[1:] - co[:-1]
        return self._ncells

    @property
    def polar_capacity(self) -> int:
        return 2 * self.cells + self.T

    def polar_offsets(self) -> list[int]:
        """First transverse face of each interface j | j+1, and the total."""
        co = self.co.cpu().numpy()
        return [int(co[j] + co[j + 1] - co[1] + j) for j in range(self.T)]

    def _ghosts(self, ghost, stages):
        g = torch.as_tensor(np.asarray(ghost, dtype=np.float64), device=self.u.device)
        g = g.reshape(-1, self.T, 5)
        if g.shape[0] < stages:
            raise ValueError(f"ghost states for {stages} stages are needed")
        return g.contiguous()

    def advance(self, dt: float, ghost_in, ghost_out, rk_order: int = 1, use_plm: bool = True) -> None:
        """control::advance_runge_kutta of the forward-Euler advance, in place;
        ghost_in / ghost_out: (stages, T, 5) boundary primitives."""
        gi, go = self._ghosts(ghost_in, rk_order), self._ghosts(ghost_out, rk_order)
        check(lib.mara_sedov_advance(self.T, self.cells, self.co.data_ptr(), self.theta.data_ptr(),
                                     self.radii.data_ptr(), self.u.data_ptr(), gi.data_ptr(), go.data_ptr(), dt,
                                     rk_order, int(use_plm), self.workspace.data_ptr(), self.failures.data_ptr(),
                                     _stream()), "mara_sedov_advance")

    def stage(self, dt: float, ghost_in, ghost_out, use_plm: bool = True) -> dict:
        """One forward-Euler advance into new arrays, with the intermediate
        arrays; the tracks themselves are unchanged."""
        dev = self.u.device
        C, F, NP = self.cells, self.cells + self.T, self.polar_capacity
        out = {"radii": torch.empty(F, dtype=torch.float64, device=dev),
               "u": torch.empty(5, C, dtype=torch.float64, device=dev),
               "prim": torch.empty(5, C, dtype=torch.float64, device=dev),
               "grad": torch.empty(5, C, dtype=torch.float64, device=dev),
               "radial": torch.empty(6, F, dtype=torch.float64, device=dev),
               "polar": torch.empty(6, NP, dtype=torch.float64, device=dev),
               "polar_index": torch.empty(2, NP, dtype=torch.int32, device=dev)}
        gi, go = self._ghosts(ghost_in, 1), self._ghosts(ghost_out, 1)
        check(lib.mara_sedov_stage(self.T, C, self.co.data_ptr(), self.theta.data_ptr(), self.radii.data_ptr(),
                                   self.u.data_ptr(), gi.data_ptr(), go.data_ptr(), dt, int(use_plm),
                                   out["radii"].data_ptr(), out["u"].data_ptr(), out["prim"].data_ptr(),
                                   out["grad"].data_ptr(), out["radial"].data_ptr(), out["polar"].data_ptr(),
                                   out["polar_index"].data_ptr(), self.workspace.data_ptr(),
                                   self.failures.data_ptr(), _stream()), "mara_sedov_stage")
        return out

    def remesh(self, max_aspect: float = 2.0, min_aspect: float = 0.5, inner_radius: float = 1.0) -> int:
        """sedov::remesh of every track (the driver's defaults: max_aspect 2,
        min_aspect 0.5, inner radius 1); the tracks move to new arrays.
        Returns the new cell count."""
        dev = self.u.device
        cap = self.cells + self.T
        co = torch.empty(self.T + 1, dtype=torch.int64, device=dev)
        radii = torch.empty(cap + self.T, dtype=torch.float64, device=dev)
        u = torch.empty(5 * cap, dtype=torch.float64, device=dev)
        nbytes = lib.mara_sedov_remesh_workspace_bytes(self.T, self.cells)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        cells = ctypes.c_int64()
        check(lib.mara_sedov_remesh(self.T, self.cells, self.co.data_ptr(), self.theta.data_ptr(),
                                    self.radii.data_ptr(), self.u.data_ptr(), max_aspect, min_aspect, inner_radius,
                                    co.data_ptr(), radii.data_ptr(), u.data_ptr(), ctypes.byref(cells),
                                    ws.data_ptr(), self.failures.data_ptr(), _stream()), "mara_sedov_remesh")
        self.cells = int(cells.value)
        self.co = co
        self.radii = radii[: self.cells + self.T]
        self.u = u[: 5 * self.cells].view(5, self.cells)
        self._ncells = None                      # read back from co on demand
        nbytes = lib.mara_sedov_workspace_bytes(self.T, self.cells)
        if self.workspace.numel() < nbytes:
            self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        return self.cells

    def min_spacing(self) -> float:
        """sedov::minimum_spacing over every track."""
        out = torch.empty(1, dtype=torch.float64, device=self.u.device)
        check(lib.mara_sedov_min_spacing(self.T, self.cells, self.co.data_ptr(), self.radii.data_ptr(),
                                         out.data_ptr(), _stream()), "mara_sedov_min_spacing")
        return float(out.item())

    def failure_count(self) -> int:
        return int(self.failures.item())

    def reset_failures(self) -> None:
        self.failures.zero_()

    def snapshot(self) -> dict:
        """A device copy of the tracks' state (offsets, radii, conserved)."""
        return {"co": self.co.clone(), "radii": self.radii.clone(), "u": self.u.clone(), "cells": self.cells,
                "ncells": None if self._ncells is None else self._ncells.copy()}

    def restore(self, snap: dict) -> None:
        """Put back a snapshot's state (copied, so the snapshot stays usable)."""
        self.co, self.radii, self.u = snap["co"].clone(), snap["radii"].clone(), snap["u"].clone()
        self.cells = snap["cells"]
        self._ncells = None if snap["ncells"] is None else snap["ncells"].copy()
        nbytes = lib.mara_sedov_workspace_bytes(self.T, self.cells)
        if self.workspace.numel() < nbytes:
            self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.u.device)

    def host_state(self) -> tuple[np.ndarray, np.ndarray]:
        """(radii, u as (cells, 5) tuples) on the host."""
        return self.radii.cpu().numpy(), self.u.cpu().numpy().T.copy()


class Driver:
    """The time loop of problems/sedov2d.cpp:697-741 around `Tracks`, with its
    safety mode: each step is the RK advance with dt = cfl * min spacing / c
    (c = 1) followed by the remesh of every track. Where the reference
    catches an exception (a failed primitive recovery, an HLLC contact speed
    it rejects), the GPU counts failures; a step whose count is not zero is
    handled as the reference handles the exception:
      - at the iteration that failed last, the failure is final: the state
        before the step is put back and MaraError is raised;
      - otherwise the state before the last successful step is restored
        (the reference's backup) and the next step runs in safety mode,
        dt x 1e-3 and PLM off; a successful step leaves safety mode.
    As in the reference, a failure at iteration 0 is final (its backup is
    empty and the iteration of the last failure starts at 0). The failure
    count is read after the advance and again after the remesh (one host
    synchronisation each); a failed advance skips the remesh, as the
    reference's exception does.

    tracks: a Tracks (or anything with its advance / remesh / min_spacing /
    snapshot / restore / reset_failures / failure_count methods);
    ghosts(time) -> (ghost_in, ghost_out), each (rk_order, T, 5) boundary
    primitives for the step starting at `time`."""

    def __init__(self, tracks, ghosts, cfl: float = 0.5, rk_order: int = 1, max_aspect: float = 2.0,
                 min_aspect: float = 0.5, inner_radius: float = 1.0, time: float = 0.0, iteration: int = 0):
        self.tracks = tracks
        self.ghosts = ghosts
        self.cfl, self.rk_order = cfl, rk_order
        self.max_aspect, self.min_aspect, self.inner_radius = max_aspect, min_aspect, inner_radius
        self.time, self.iteration = time, iteration
        self.backup = None           # (snapshot, time, iteration) before the last successful step
        self.safety = False
        self.failed_iter = 0

    def step(self) -> dict:
        """One step of the loop; returns what it did (dt, whether it was a
        safety-mode step, whether it rolled back)."""
        t = self.tracks
        safety = self.safety
        dt = self.cfl * (1e-3 if safety else 1.0) * t.min_spacing()
        ghost_in, ghost_out = self.ghosts(self.time)
        pre = (t.snapshot(), self.time, self.iteration)
        t.reset_failures()
        t.advance(dt, ghost_in, ghost_out, rk_order=self.rk_order, use_plm=not safety)
        failures = t.failure_count()
        if failures == 0:
            # the reference's exception would skip the remesh: so does a failed advance
            t.remesh(self.max_aspect, self.min_aspect, self.inner_radius)
            failures = t.failure_count()
        if failures == 0:
            self.time += dt
            self.iteration += 1
            self.backup = pre
            self.safety = False
            return {"dt": dt, "safety": safety, "rolled_back": False, "iteration": self.iteration}
        if self.iteration == self.failed_iter:
            t.restore(pre[0])
            raise MaraError(f"sedov step {self.iteration} failed ({failures} failed zones, faces or tracks) and "
                            "cannot be retried: it is the first step, or the step that failed last")
        self.failed_iter = self.iteration
        snap, self.time, self.iteration = self.backup
        t.restore(snap)
        self.safety = True
        return {"dt": dt, "safety": safety, "rolled_back": True, "iteration": self.iteration, "failures": failures}
