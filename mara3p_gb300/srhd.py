"""Host-side mirror of the reference's SRHD primitive recovery
(src/physics_srhd.hpp:231-285, srhd::recover_primitive) plus the learned
pressure guess. Arrays are torch CUDA tensors; zones are SoA (5, n) unless a
stride pair says otherwise."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from ._capi import check, lib

STATUS_OK, STATUS_NOT_CONVERGED, STATUS_NEGATIVE_PRESSURE = 0, 1, 2


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _f64(t: torch.Tensor) -> int:
    if not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError("expected a contiguous CUDA float64 tensor")
    return t.data_ptr()


@dataclass
class Recovery:
    prim: torch.Tensor          # (5, n): rho, u1, u2, u3, p
    iterations: torch.Tensor    # (n,) int32, FP64 Newton iterations
    status: torch.Tensor        # (n,) int32


def recover_primitive(cons: torch.Tensor, gamma_law_index: float = 4.0 / 3.0, temperature_floor: float = 0.0,
                      mlp: "PressureGuess | None" = None, refine32: int = 0, seeded_budget: int = 12,
                      layout: str = "soa") -> Recovery:
    """srhd::recover_primitive over many zones. cons is (5, n) for layout 'soa'
    or (n, 5) for 'aos' (the reference's tuple layout)."""
    if layout not in ("soa", "aos"):
        raise ValueError("layout must be 'soa' or 'aos'")
    if cons.dim() != 2 or cons.shape[0 if layout == "soa" else 1] != 5:
        raise ValueError(f"recover_primitive: cons must be {'(5, n)' if layout == 'soa' else '(n, 5)'}, "
                         f"got {tuple(cons.shape)}")
    if layout == "soa":
        n = cons.shape[1]
        cs, zs = n, 1
    else:
        n = cons.shape[0]
        cs, zs = 1, 5
    prim = torch.empty_like(cons)
    it = torch.empty(n, dtype=torch.int32, device=cons.device)
    st = torch.empty(n, dtype=torch.int32, device=cons.device)
    check(lib.mara_srhd_recover_primitive(_f64(cons), n, cs, zs, gamma_law_index, temperature_floor,
                                          mlp.weights.data_ptr() if mlp else None, refine32, seeded_budget,
                                          prim.data_ptr(), it.data_ptr(), st.data_ptr(), None, _stream()),
          "srhd recover_primitive")
    return Recovery(prim, it, st)


class HostRecovery:
    """srhd::recover_primitive for zones held in (pinned) host memory:
    `recover(cons)` takes a (5, n) float64 CPU tensor and returns the (5, n)
    primitives in a pinned CPU tensor of this object, pipelined through the
    GPU in `chunks` pieces (transfers of some pieces overlap the recovery of
    others). The device workspace and the output are kept between calls of
    the same n. `failures` holds the failed-zone count of the last call."""

    def __init__(self, mlp: "PressureGuess | None" = None, refine32: int = 0, seeded_budget: int = 12,
                 gamma_law_index: float = 4.0 / 3.0, temperature_floor: float = 0.0, chunks: int = 8):
        self.mlp, self.refine32, self.seeded_budget, self.chunks = mlp, refine32, seeded_budget, chunks
        self.gamma, self.floor = gamma_law_index, temperature_floor
        self.n = -1
        self.failures = 0

    def recover(self, cons: torch.Tensor) -> torch.Tensor:
        if cons.device.type != "cpu" or cons.dtype != torch.float64 or cons.dim() != 2 or cons.shape[0] != 5:
            raise ValueError("cons must be a (5, n) float64 CPU tensor")
        cons = cons.contiguous()
        n = cons.shape[1]
        if n != self.n:
            nbytes = lib.mara_srhd_host_workspace_bytes(n, self.chunks)
            if nbytes < 0:
                check(1, "mara_srhd_host_workspace_bytes")
            self.workspace = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
            self.prim = torch.empty((5, n), dtype=torch.float64).pin_memory()
            self.n = n
        failed = ctypes.c_ulonglong()
        check(lib.mara_srhd_recover_primitive_host(cons.data_ptr(), n, self.gamma, self.floor,
                                                   self.mlp.weights.data_ptr() if self.mlp else None,
                                                   self.refine32, self.seeded_budget, self.prim.data_ptr(),
                                                   self.chunks, self.workspace.data_ptr(), ctypes.byref(failed),
                                                   _stream()), "srhd recover_primitive_host")
        self.failures = int(failed.value)
        return self.prim


class PressureGuess:
    """The 4-64-64-1 MLP that seeds the recovery, trained on the GPU by the
    library's own kernels on (conserved, primitive) pairs."""

    def __init__(self, device="cuda"):
        self.weights = torch.zeros(lib.mara_srhd_mlp_weights_bytes(), dtype=torch.uint8, device=device)
        self.workspace = None
        self.n = 0

    def prepare(self, cons: torch.Tensor, prim: torch.Tensor, seed: int = 0) -> None:
        n = cons.shape[1]
        self.n = n
        self.workspace = torch.empty(lib.mara_srhd_mlp_workspace_bytes(n), dtype=torch.uint8, device=cons.device)
        check(lib.mara_srhd_mlp_prepare(_f64(cons), _f64(prim), n, self.weights.data_ptr(), seed,
                                        self.workspace.data_ptr(), _stream()), "mlp prepare")

    def gradient(self) -> tuple[torch.Tensor, float]:
        grad = torch.empty(lib.mara_srhd_mlp_param_count(), dtype=torch.float32, device=self.weights.device)
        loss = torch.empty(1, dtype=torch.float32, device=self.weights.device)
        check(lib.mara_srhd_mlp_gradient(self.weights.data_ptr(), self.workspace.data_ptr(), self.n,
                                         grad.data_ptr(), loss.data_ptr(), _stream()), "mlp gradient")
        return grad, float(loss.item())

    def train(self, steps: int, batch: int = 8192, lr: float = 2e-3, seed: int = 0) -> torch.Tensor:
        g = torch.Generator(device="cpu").manual_seed(seed)
        order = torch.randperm(self.n, generator=g).to(self.weights.device, torch.int64)
        hist = torch.empty(max(steps, 1), dtype=torch.float32, device=self.weights.device)
        check(lib.mara_srhd_mlp_train(self.weights.data_ptr(), self.workspace.data_ptr(), self.n,
                                      order.data_ptr(), steps, batch, lr, hist.data_ptr(), _stream()),
              "mlp train")
        return hist[:steps]

    def infer(self, features: torch.Tensor) -> torch.Tensor:
        y = torch.empty(features.shape[0], dtype=torch.float32, device=features.device)
        check(lib.mara_srhd_mlp_infer(self.weights.data_ptr(), features.data_ptr(), features.shape[0],
                                      y.data_ptr(), _stream()), "mlp infer")
        return y

    def parameters_f32(self) -> dict:
        """Host copy of the FP32 parameters (for checks against the CPU oracle)."""
        raw = self.weights.cpu().numpy()
        f = raw[: (len(raw) // 4) * 4].view("float32")
        o = {"norm_shift": f[0:4], "norm_scale": f[4:8], "w1": f[8:264].reshape(64, 4), "b1": f[264:328],
             "w2": f[328:4424].reshape(64, 64), "b2": f[4424:4488], "w3": f[4488:4552], "b3": f[4552],
             "out_shift": f[4553], "out_scale": f[4554]}
        return o


GUESS_ZERO, GUESS_MLP, GUESS_PREVIOUS = 0, 1, 2


class ShockTube:
    """2D SRHD on the unit square with the reference's recovery, PLM and HLLE
    (the relativistic shock-tube benchmark): u is (4, N, N) = (D, S1, S2, tau)."""

    def __init__(self, N: int = 1024, angle: float = 3.141592653589793 / 6, left=(10.0, 13.33), right=(1.0, 1e-6),
                 gamma_law_index: float = 4.0 / 3.0, cfl: float = 0.3, plm_theta: float = 1.5,
                 temperature_floor: float = 1e-10, device="cuda"):
        self.N, self.gamma, self.cfl, self.theta, self.floor = N, gamma_law_index, cfl, plm_theta, temperature_floor
        self.u = torch.empty((4, N, N), dtype=torch.float64, device=device)
        self.clock = torch.zeros(lib.mara_srhd_tube_clock_bytes(), dtype=torch.uint8, device=device)
        self.workspace = torch.empty(lib.mara_srhd_tube_workspace_bytes(N), dtype=torch.uint8, device=device)
        check(lib.mara_srhd_tube_initial(N, angle, left[0], left[1], right[0], right[1], gamma_law_index,
                                         self.u.data_ptr(), self.clock.data_ptr(), _stream()), "tube initial")

    def advance(self, steps: int, precision: int = 0, guess: int = GUESS_ZERO, mlp: "PressureGuess | None" = None,
                refine32: int = 0, riemann: str = "hlle") -> None:
        """`steps` RK2 steps; riemann is "hlle" or "hllc" (riemann_solver, physics_srhd.hpp:377-487)."""
        solver = {"hlle": 0, "hllc": 1}[riemann]
        check(lib.mara_srhd_tube_advance(self.N, self.u.data_ptr(), self.clock.data_ptr(), steps, self.cfl, self.theta,
                                         self.gamma, self.floor, precision, guess, mlp.weights.data_ptr() if mlp else None,
                                         refine32, solver, self.workspace.data_ptr(), _stream()), "tube advance")

    def clock_state(self) -> dict:
        raw = self.clock.cpu().numpy()
        d = raw.view("float64")
        q = raw.view("uint64")
        return {"time": float(d[0]), "dt": float(d[1]), "iteration": int(q[3]), "failures": int(q[4]),
                "newton": int(q[5]), "riemann_rejected": int(q[6])}


def riemann(pl: torch.Tensor, pr: torch.Tensor, axis: int, gamma_law_index: float = 4.0 / 3.0,
            solver: str = "hlle") -> tuple[torch.Tensor, torch.Tensor]:
    """srhd::riemann_solver at fixed faces (physics_srhd.hpp:377-487): left/right
    primitives (n, 5) float64 CUDA, axis 1..3; returns fluxes (n, 5) and the
    per-face status (1 where the reference throws)."""
    if pl.dim() != 2 or pl.shape[1] != 5 or pr.shape != pl.shape:
        raise ValueError(f"riemann: pl and pr must both be (n, 5), got {tuple(pl.shape)} and {tuple(pr.shape)}")
    pl, pr = pl.contiguous(), pr.contiguous()
    _f64(pl), _f64(pr)
    n = pl.shape[0]
    f = torch.empty_like(pl)
    status = torch.empty(n, dtype=torch.int32, device=pl.device)
    check(lib.mara_srhd_riemann(pl.data_ptr(), pr.data_ptr(), n, axis, gamma_law_index,
                                {"hlle": 0, "hllc": 1}[solver], f.data_ptr(), status.data_ptr(), _stream()), "riemann")
    return f, status
