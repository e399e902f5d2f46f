"""Shared test helpers (not collected as tests)."""
from __future__ import annotations

import numpy as np

from oracle.oracle import MinidiskParams

# The reference-sized minidisk: [-4,4]^2 on 256^2 cells (4x4 blocks of 64^2),
# an equal-mass circular binary, Mach 10, nu 1e-3 (the reference's PLM theta 2)
REFERENCE_DISK = dict(block_size=64, depth=2, omega_frame=1.0, mach_number=10.0, nu=1e-3, domain_radius=4.0,
                      softening_length=0.05, eccentricity=0.0, mass_ratio=1.0, sink_radius=0.05, sink_rate=10.0,
                      buffer_rate=100.0, buffer_scale=0.2, cfl=0.3, plm_theta=2.0)

SMALL_PARAMS = dict(REFERENCE_DISK, block_size=16, depth=2, domain_radius=1.0)

# The large-minidisk configuration: [-8,8]^2 on 4096^2 cells (64x64 blocks of
# 64^2), q 0.5, e 0.1, Mach 20, nu 5e-4, PLM theta 1.5 (CFL dt in its runs)
LARGE_DISK = dict(block_size=64, depth=6, omega_frame=1.0, mach_number=20.0, nu=5e-4, domain_radius=8.0,
                  softening_length=0.05, eccentricity=0.1, mass_ratio=0.5, sink_radius=0.05, sink_rate=10.0,
                  buffer_rate=100.0, buffer_scale=0.2, cfl=0.3, plm_theta=1.5)


def params_from_vector(v: np.ndarray, theta: float = 2.0) -> MinidiskParams:
    keys = ("block_size depth omega_frame mach_number nu domain_radius softening_length eccentricity "
            "mass_ratio sink_radius sink_rate buffer_rate buffer_scale cfl").split()
    kw = {k: (int(x) if k in ("block_size", "depth") else float(x)) for k, x in zip(keys, v)}
    return MinidiskParams(**kw, plm_theta=theta)


def rel_l1_components(a: np.ndarray, b: np.ndarray, ncomp: int = 3) -> float:
    """Largest per-component relative L1 difference, sum|a-b| / sum|b|."""
    a = np.asarray(a, dtype=np.float64).reshape(ncomp, -1)
    b = np.asarray(b, dtype=np.float64).reshape(ncomp, -1)
    num = np.abs(a - b).sum(axis=1)
    den = np.abs(b).sum(axis=1)
    return float(np.max(num / np.where(den > 0, den, 1.0)))
