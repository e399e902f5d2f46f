"""Host-side mirror of the reference's constrained-transport MHD scheme
(src/scheme_mhd_v1.hpp:102-134: advance_mhd_ct, construct_conserved) and of
the RK2 driver of examples/mhd3d.cpp, on torch CUDA tensors.

State: uc (5, N, N, N) SoA float64; bf1 (N+1, N, N), bf2 (N, N+1, N),
bf3 (N, N, N+1) face B as the reference holds them.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from ._capi import MaraError, MhdParams, check, lib

FP64, MIXED = 0, 1


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _p(t):
    if t is None:
        return None
    if not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError("expected a contiguous CUDA float64 tensor")
    return t.data_ptr()


@dataclass(frozen=True)
class MhdConfig:
    N: int = 128
    gamma_law_index: float = 5.0 / 3.0
    cfl: float = 0.3
    plm_theta: float = 1.5

    def to_c(self) -> MhdParams:
        return MhdParams(self.N, self.gamma_law_index, self.cfl, self.plm_theta)


def mode_table(seed: int, modes: int) -> np.ndarray:
    t = np.zeros(11 * modes)
    check(lib.mara_mhd_mode_table(seed, modes, t.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "mode_table")
    return t


def amplitudes(modes: int, v_rms: float = 0.5, beta: float = 10.0, pressure: float = 1.0) -> tuple[float, float]:
    """Velocity and vector-potential amplitudes for rms |v| = v_rms and plasma
    beta = 2p/<B^2> (each mode contributes 1/2 to the mean square; B modes
    have amplitude 2*pi*a_amp)."""
    half = math.sqrt(modes / 2.0)
    b_rms = math.sqrt(2.0 * pressure / beta)
    return v_rms / half, b_rms / (2.0 * math.pi * half)


@dataclass
class State:
    cfg: MhdConfig
    uc: torch.Tensor
    bf: list = field(default_factory=list)


def check_state(state: State, uc_in: torch.Tensor | None = None) -> None:
    """Reject a state whose arrays do not have the sizes of its mesh (cells
    (5, N, N, N); faces (N+1, N, N), (N, N+1, N), (N, N, N+1)): the C ABI
    takes bare pointers, so a short array would be read past its end."""
    N = state.cfg.N
    want = [5 * N ** 3] + [(N + 1) * N * N] * 3
    got = [state.uc.numel()] + [b.numel() for b in state.bf]
    if len(state.bf) != 3 or got != want:
        raise ValueError(f"MHD state of N = {N}: expected {want} values (uc, b1, b2, b3), got {got}")
    if uc_in is not None and uc_in.numel() != 5 * N ** 3:
        raise ValueError(f"advance_ct: uc_in must hold 5 N^3 = {5 * N ** 3} values, got {uc_in.numel()}")


def empty_state(cfg: MhdConfig, device="cuda") -> State:
    N = cfg.N
    f64 = dict(dtype=torch.float64, device=device)
    return State(cfg, torch.empty((5, N, N, N), **f64),
                 [torch.empty((N + 1, N, N), **f64), torch.empty((N, N + 1, N), **f64), torch.empty((N, N, N + 1), **f64)])


def initial_state(cfg: MhdConfig, seed: int = 0, modes: int = 24, v_rms: float = 0.5, beta: float = 10.0) -> State:
    s = empty_state(cfg)
    t = mode_table(seed, modes)
    v_amp, a_amp = amplitudes(modes, v_rms, beta)
    ws = torch.empty(88 * modes + 256, dtype=torch.uint8, device="cuda")
    check(lib.mara_mhd_initial_state(ctypes.byref(cfg.to_c()), t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), modes,
                                     v_amp, a_amp, _p(s.uc), _p(s.bf[0]), _p(s.bf[1]), _p(s.bf[2]), ws.data_ptr(),
                                     _stream()), "initial_state")
    torch.cuda.current_stream().synchronize()
    return s


class Clock:
    def __init__(self, time: float = 0.0, device="cuda"):
        self.buf = torch.zeros(lib.mara_mhd_clock_bytes(), dtype=torch.uint8, device=device)
        check(lib.mara_mhd_clock_init(self.buf.data_ptr(), time, _stream()), "clock_init")

    def read(self) -> dict:
        raw = self.buf.cpu().numpy()
        d = raw.view(np.float64)
        q = raw.view(np.uint64)
        return {"time": float(d[0]), "dt": (float(d[1]), float(d[2])), "iteration": int(raw[40:48].view(np.int64)[0]),
                "failures": int(q[6])}


def advance_ct(state: State, uc_in: torch.Tensor | None = None, layout: str = "soa", precision: int = FP64,
               clock: Clock | None = None) -> tuple[State, Clock]:
    """mara::advance_mhd_ct: one CFL step. uc_in (optional) in the reference's
    AoS layout (N, N, N, 5) when layout='aos'."""
    check_state(state, uc_in)
    cfg = state.cfg
    N = cfg.N
    clock = clock or Clock()
    out = empty_state(cfg)
    ws = torch.empty(lib.mara_mhd_workspace_bytes(ctypes.byref(cfg.to_c()), 1, precision), dtype=torch.uint8,
                     device="cuda")
    u = state.uc if uc_in is None else uc_in
    cs, zs = (N ** 3, 1) if layout == "soa" else (1, 5)
    check(lib.mara_mhd_advance_ct(ctypes.byref(cfg.to_c()), _p(u), cs, zs, _p(state.bf[0]), _p(state.bf[1]),
                                  _p(state.bf[2]), _p(out.uc), _p(out.bf[0]), _p(out.bf[1]), _p(out.bf[2]),
                                  clock.buf.data_ptr(), precision, ws.data_ptr(), _stream()), "advance_ct")
    return out, clock


class Run:
    """RK2 MHD run (examples/mhd3d.cpp semantics) resident on the GPU."""

    def __init__(self, state: State, time: float = 0.0, precision: int = FP64):
        check_state(state)
        self.state = state
        self.precision = precision
        self.clock = Clock(time)
        self.ws = torch.empty(lib.mara_mhd_workspace_bytes(ctypes.byref(state.cfg.to_c()), 2, precision),
                              dtype=torch.uint8, device="cuda")

    def advance(self, steps: int) -> None:
        s = self.state
        check(lib.mara_mhd_advance(ctypes.byref(s.cfg.to_c()), _p(s.uc), _p(s.bf[0]), _p(s.bf[1]), _p(s.bf[2]),
                                   self.clock.buf.data_ptr(), steps, 2, self.precision, self.ws.data_ptr(), _stream()),
              "mhd advance")

    def advance_checked(self, steps: int) -> None:
        """advance(steps), failing where the reference throws: its
        mhd::recover_primitive throws on a negative density or pressure
        (src/physics_mhd.hpp:290-303), which ends examples/mhd3d. If any zone
        failed during the call, the state and clock from before it are put
        back and MaraError is raised."""
        s = self.state
        before = self.clock.read()["failures"]
        snap = (s.uc.clone(), [b.clone() for b in s.bf], self.clock.buf.clone())
        self.advance(steps)
        failed = self.clock.read()["failures"] - before
        if failed:
            s.uc.copy_(snap[0])
            for b, b0 in zip(s.bf, snap[1]):
                b.copy_(b0)
            self.clock.buf.copy_(snap[2])
            raise MaraError(f"mhd advance: {failed} zone recoveries failed (negative density or pressure); "
                            "the state before the call is restored")

    def max_div_b(self) -> float:
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        s = self.state
        check(lib.mara_mhd_max_div_b(ctypes.byref(s.cfg.to_c()), _p(s.bf[0]), _p(s.bf[1]), _p(s.bf[2]), _p(out),
                                     _stream()), "max_div_b")
        return float(out.item())
