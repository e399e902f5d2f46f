"""ORACLE — test infrastructure only.

ctypes access to oracle/liboracle.so (the CPU restatement) and, where it was
built, oracle/_ref/libref.so (the reference's own scheme code). Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


class MinidiskParams(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_int32), ("depth", ctypes.c_int32)] + [
        (k, ctypes.c_double) for k in (
            "omega_frame mach_number nu domain_radius softening_length eccentricity mass_ratio "
            "sink_radius sink_rate buffer_rate buffer_scale cfl plm_theta").split()]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def load_oracle() -> ctypes.CDLL:
    lib = ctypes.CDLL(str(HERE / "liboracle.so"))
    lib.oracle_minidisk_dt_formula.restype = ctypes.c_double
    lib.oracle_minidisk_dt_cfl.restype = ctypes.c_double
    lib.oracle_minidisk_advance.restype = ctypes.c_double
    lib.oracle_srhd_riemann.restype = ctypes.c_int64
    return lib


def load_reference() -> ctypes.CDLL | None:
    path = HERE / "_ref" / "libref.so"
    if not path.exists():
        return None
    lib = ctypes.CDLL(str(path))
    lib.ref_plm_gradient.restype = ctypes.c_double
    lib.ref_plm_gradient.argtypes = [ctypes.c_double] * 4
    return lib


def load_reference_v2() -> ctypes.CDLL | None:
    """oracle/_ref/libref_v2.so: the reference's mhd_scheme_v2 block API."""
    path = HERE / "_ref" / "libref_v2.so"
    return ctypes.CDLL(str(path)) if path.exists() else None


def params(sd) -> MinidiskParams:
    """Oracle params from any object with the solver_data_t field names."""
    return MinidiskParams(**{name: getattr(sd, name) for name, _ in MinidiskParams._fields_})


def solver_vector(p: MinidiskParams) -> np.ndarray:
    """The 14-double solver_data_t vector that the reference harness takes."""
    return np.array([p.block_size, p.depth, p.omega_frame, p.mach_number, p.nu, p.domain_radius,
                     p.softening_length, p.eccentricity, p.mass_ratio, p.sink_radius, p.sink_rate,
                     p.buffer_rate, p.buffer_scale, p.cfl], dtype=np.float64)
