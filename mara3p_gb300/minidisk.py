"""Host-side mirror of the reference's minidisk interface (problems/minidisk.hpp).

Names and argument meanings follow the reference: `SolverData` is
minidisk::solver_data_t, `updated_conserved(uc, pe, time, dt, block, sd)` is
minidisk::updated_conserved, and so on. Arrays are torch CUDA float64 tensors:
per-block calls use the reference's AoS tuple layout ((n, n, 3) conserved,
(n+4, n+4, 3) primitives with halo); whole-mesh calls use the GPU layout,
SoA (3, N, N). Every call goes through libmara_gb300.so; errors raise
MaraError (the reference throws C++ exceptions).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, fields, replace

import torch

from ._capi import DIAG_COUNT, MinidiskClock, MinidiskDiagnostics, MinidiskParams, check, lib

FP64, MIXED = 0, 1
DT_FORMULA, DT_CFL, DT_FORMULA_HELD = 0, 1, 2


@dataclass(frozen=True)
class SolverData:
    """minidisk::solver_data_t (problems/minidisk.hpp:77-93); defaults are the
    reference's config_template (problems/minidisk.hpp:99-122). plm_theta is
    the PLM parameter the reference hard-codes to 2.0."""

    block_size: int = 64
    depth: int = 1
    omega_frame: float = 1.0
    mach_number: float = 10.0
    nu: float = 0.0
    domain_radius: float = 1.5
    softening_length: float = 0.01
    eccentricity: float = 0.0
    mass_ratio: float = 1.0
    sink_radius: float = 0.01
    sink_rate: float = 1e3
    buffer_rate: float = 1e2
    buffer_scale: float = 0.2
    cfl: float = 0.3
    plm_theta: float = 2.0

    @property
    def cells_per_side(self) -> int:
        return self.block_size << self.depth

    def to_c(self) -> MinidiskParams:
        return MinidiskParams(**{f.name: getattr(self, f.name) for f in fields(self)})

    def with_(self, **kw) -> "SolverData":
        return replace(self, **kw)


def make_solver_data(cfg: dict) -> SolverData:
    """make_solver_data (problems/minidisk.hpp:124-142) from a key=value map."""
    known = {f.name for f in fields(SolverData)}
    unknown = set(cfg) - known
    if unknown:
        raise ValueError(f"unknown minidisk config keys: {sorted(unknown)}")
    return SolverData(**cfg)


def smallest_cell_size(sd: SolverData) -> float:
    """minidisk::smallest_cell_size (problems/minidisk_scheme.cpp:122-125)."""
    return 2.0 * sd.domain_radius / float(sd.block_size) / float(1 << sd.depth)


def _ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError("expected a contiguous CUDA float64 tensor")
    return t.data_ptr()


def _any_ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise TypeError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _mesh_values(sd: "SolverData", t: torch.Tensor | None, what: str, dtype=torch.float64) -> None:
    """Reject a tensor that does not hold the SoA mesh (3, N, N) in `dtype`:
    the C ABI takes bare pointers, so a short buffer would be read or
    written past its end on the device."""
    if t is None:
        return
    N = sd.cells_per_side
    if t.numel() != 3 * N * N or t.dtype != dtype:
        raise ValueError(f"{what}: expected {3 * N * N} {dtype} values, (3, {N}, {N}); got {tuple(t.shape)} {t.dtype}")


def binary_state(sd: SolverData, time: float) -> list[float]:
    """Binary (m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2) in the rotating frame."""
    out = (ctypes.c_double * 10)()
    check(lib.mara_minidisk_binary(ctypes.byref(sd.to_c()), time, out), "mara_minidisk_binary")
    return list(out)


def dt_formula(sd: SolverData, time: float) -> float:
    """The fixed time step of problems/minidisk.cpp:204-206."""
    dt = ctypes.c_double()
    check(lib.mara_minidisk_dt_formula(ctypes.byref(sd.to_c()), time, ctypes.byref(dt)), "mara_minidisk_dt_formula")
    return dt.value


def updated_conserved(uc: torch.Tensor, pe: torch.Tensor, time: float, dt: float,
                      block: tuple[int, int, int], sd: SolverData) -> torch.Tensor:
    """minidisk::updated_conserved (problems/minidisk.hpp:164-170) on one block.
    block = (level, i, j); uc (n, n, 3); pe (n+4, n+4, 3) primitives."""
    n = sd.block_size
    if tuple(uc.shape) != (n, n, 3) or tuple(pe.shape) != (n + 4, n + 4, 3):
        raise ValueError("updated_conserved: uc must be (n, n, 3) and pe (n+4, n+4, 3)")
    level, bi, bj = block
    u1 = torch.empty_like(uc)
    check(lib.mara_minidisk_updated_conserved(ctypes.byref(sd.to_c()), _ptr(uc), _ptr(pe), time, dt,
                                              level, bi, bj, _ptr(u1), _stream()), "updated_conserved")
    return u1


def recover_primitive_array(uc: torch.Tensor) -> torch.Tensor:
    """minidisk::recover_primitive_array (problems/minidisk_scheme.cpp:208-211)."""
    if uc.shape[-1] != 3:
        raise ValueError("recover_primitive_array: last axis must hold (Σ, Σvx, Σvy)")
    pc = torch.empty_like(uc)
    check(lib.mara_minidisk_recover_primitive(_ptr(uc), uc.numel() // 3, _ptr(pc), _stream()), "recover_primitive_array")
    return pc


def estimate_gradient(pc: torch.Tensor, axis: int, theta: float) -> torch.Tensor:
    """minidisk::estimate_gradient (problems/minidisk_scheme.cpp:213-216)."""
    if pc.dim() != 3 or pc.shape[2] != 3 or axis not in (0, 1) or pc.shape[axis] < 3:
        raise ValueError("estimate_gradient: pc must be (n0, n1, 3) with at least 3 cells along axis 0 or 1")
    n0, n1 = pc.shape[0], pc.shape[1]
    shape = (n0 - 2, n1, 3) if axis == 0 else (n0, n1 - 2, 3)
    out = torch.empty(shape, dtype=torch.float64, device=pc.device)
    check(lib.mara_minidisk_estimate_gradient(_ptr(pc), n0, n1, axis, theta, _ptr(out), _stream()), "estimate_gradient")
    return out


def initial_conserved(sd: SolverData, seed: int = 0, amplitude: float = 0.0, device="cuda") -> torch.Tensor:
    """Initial SoA state (3, N, N): minidisk::initial_conserved_array over the
    whole mesh, with an optional seeded density perturbation."""
    N = sd.cells_per_side
    u = torch.empty((3, N, N), dtype=torch.float64, device=device)
    check(lib.mara_minidisk_initial_conserved(ctypes.byref(sd.to_c()), seed, amplitude, _ptr(u), _stream()),
          "initial_conserved")
    return u


def substep(sd: SolverData, u: torch.Tensor, time: float, dt: float, u_avg: torch.Tensor | None = None) -> torch.Tensor:
    """One whole-mesh forward-Euler substep (plain FP64); with u_avg, the RK2
    second stage u_avg/2 + L(u)/2."""
    _mesh_values(sd, u, "substep u")
    _mesh_values(sd, u_avg, "substep u_avg")
    out = torch.empty_like(u)
    check(lib.mara_minidisk_substep(ctypes.byref(sd.to_c()), _ptr(u), _ptr(u_avg), _ptr(out), time, dt, _stream()),
          "substep")
    return out


# Names of the rate-vector entries (mara_minidisk_diagnostics).
DIAG_NAMES = ("sink_mass_1", "sink_mass_2", "sink_px_1", "sink_py_1", "sink_px_2", "sink_py_2",
              "force_x_1", "force_y_1", "force_x_2", "force_y_2", "buffer_mass", "disk_mass",
              "disk_angular_momentum", "torque_1", "torque_2", "power")
assert len(DIAG_NAMES) == DIAG_COUNT


def rates(sd: SolverData, u: torch.Tensor, time: float, d1: torch.Tensor | None = None) -> dict[str, float]:
    """The time-series rate vector of the SoA state u (+ FP32 increment d1)
    at `time`, reduced on the GPU in FP64."""
    _mesh_values(sd, u, "rates u")
    _mesh_values(sd, d1, "rates d1", torch.float32)
    out = torch.zeros(DIAG_COUNT, dtype=torch.float64, device=u.device)
    check(lib.mara_minidisk_rates(ctypes.byref(sd.to_c()), _ptr(u), _any_ptr(d1), time, _ptr(out), _stream()),
          "mara_minidisk_rates")
    return dict(zip(DIAG_NAMES, out.tolist()))


def two_body_elements(state: list[float], time: float) -> dict[str, float]:
    """two_body::recover_orbital_elements (src/physics_two_body.hpp:284-379) of
    {m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2}; raises MaraError if unbound."""
    s = (ctypes.c_double * 10)(*state)
    out = (ctypes.c_double * 10)()
    check(lib.mara_two_body_elements(s, time, out), "mara_two_body_elements")
    return dict(zip(("a", "M", "q", "e", "x_cm", "y_cm", "vx_cm", "vy_cm", "pomega", "tau"), out))


def element_rates(state: list[float], time: float, rate: list[float] | dict[str, float]) -> dict[str, float]:
    """d(a, M, q, e)/dt implied by a rate vector acting on the binary state."""
    r = [rate[k] for k in DIAG_NAMES] if isinstance(rate, dict) else list(rate)
    s = (ctypes.c_double * 10)(*state)
    rv = (ctypes.c_double * DIAG_COUNT)(*r)
    out = (ctypes.c_double * 4)()
    check(lib.mara_two_body_element_rates(s, time, rv, out), "mara_two_body_element_rates")
    return dict(zip(("a", "M", "q", "e"), out))


class Run:
    """A minidisk run resident on one GPU: SoA state, device clock and workspace.

    advance() enqueues whole RK steps; time, dt and the binary position are
    computed on the device, so steps need no host round trip. With
    diagnostics=True every step also accumulates the time-series rates
    (mara_minidisk_diagnostics), read back by diagnostics()."""

    def __init__(self, sd: SolverData, u: torch.Tensor, time: float = 0.0, rk_order: int = 2,
                 precision: int = FP64, dt_mode: int = DT_FORMULA, diagnostics: bool = False):
        _mesh_values(sd, u, "Run state u")
        self.sd = sd
        self.c = sd.to_c()
        self.u = u
        self.rk_order = rk_order
        self.precision = precision
        self.dt_mode = dt_mode
        nbytes = lib.mara_minidisk_workspace_bytes(ctypes.byref(self.c), rk_order, precision)
        if nbytes < 0:
            check(1, "mara_minidisk_workspace_bytes")
        self.workspace = torch.empty(max(nbytes, 8), dtype=torch.uint8, device=u.device)
        self.clock = torch.zeros(ctypes.sizeof(MinidiskClock), dtype=torch.uint8, device=u.device)
        check(lib.mara_minidisk_clock_init(ctypes.byref(self.c), _ptr(u), time, self.clock.data_ptr(), _stream()),
              "clock_init")
        self.diag = None
        if diagnostics:
            self.diag = torch.zeros(ctypes.sizeof(MinidiskDiagnostics), dtype=torch.uint8, device=u.device)

    def _advance_call(self, steps: int) -> None:
        check(lib.mara_minidisk_advance_diag(ctypes.byref(self.c), _ptr(self.u), self.clock.data_ptr(), steps,
                                             self.rk_order, self.precision, self.dt_mode,
                                             self.workspace.data_ptr(), _any_ptr(self.diag), _stream()), "advance")

    def use_graph(self, steps_per_replay: int = 10) -> None:
        """Replay `steps_per_replay` steps from one captured CUDA graph
        (the reference driver's `fold` batch): small meshes, whose kernels
        take less time than their launches, stop waiting on the host. The
        same kernels run on the same buffers, so results do not change; a
        held formula dt is re-chosen at the start of each replay, as at the
        start of each advance call. Preparing the graph advances the run by
        steps_per_replay steps: one direct call (which also loads the
        kernels) before the capture, which itself runs nothing."""
        if steps_per_replay < 1:
            raise ValueError("steps_per_replay must be at least 1")
        self._advance_call(steps_per_replay)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self._advance_call(steps_per_replay)
        # uploaded to the device now: the first replay would otherwise pay for
        # it (about 60 us at 256^2, a fifth of a 10-step replay)
        if hasattr(graph, "raw_cuda_graph_exec"):
            check(lib.mara_graph_upload(graph.raw_cuda_graph_exec(), _stream()), "graph_upload")
        self._graph, self._graph_steps = graph, steps_per_replay

    def advance(self, steps: int) -> None:
        graph = getattr(self, "_graph", None)
        if graph is not None:
            while steps >= self._graph_steps:
                graph.replay()
                steps -= self._graph_steps
        if steps > 0:
            self._advance_call(steps)

    def diagnostics(self) -> dict:
        """rate (per stage of the last step), integral and steps of the
        run's diagnostics, entries named by DIAG_NAMES."""
        if self.diag is None:
            raise ValueError("this Run was made without diagnostics")
        d = MinidiskDiagnostics.from_buffer_copy(self.diag.cpu().numpy().tobytes())
        return {"rate": [dict(zip(DIAG_NAMES, list(d.rate[s]))) for s in range(2)],
                "integral": dict(zip(DIAG_NAMES, list(d.integral))), "steps": d.steps}

    def reset_diagnostics(self) -> None:
        if self.diag is not None:
            check(lib.mara_minidisk_diagnostics_reset(self.diag.data_ptr(), _stream()), "diagnostics_reset")

    def clock_state(self) -> MinidiskClock:
        raw = self.clock.cpu().numpy().tobytes()
        return MinidiskClock.from_buffer_copy(raw)

    @property
    def time(self) -> float:
        return self.clock_state().time


def kzps(cells: int, fold: int, seconds: float) -> float:
    """The reference's throughput figure, 1e6*fold*ncells/ns (problems/minidisk.cpp:298-299)."""
    return 1e-3 * fold * cells / seconds if seconds > 0 else math.inf
