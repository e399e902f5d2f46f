"""ORACLE — test infrastructure only.

numpy restatement of the array operations of the reference's mhd_scheme_v2
block API (src/scheme_mhd_v2.cpp:75-278) and of the staggered operators it
uses (src/mesh_cartesian_3d.hpp:236-305): face_to_cell, the edge EMFs of
electromotive_forces, updated_conserved_density, curl and
updated_magnetic_flux_density. Arrays are the reference's row-major blocks
(last axis contiguous); tuple-valued arrays carry the tuple as a trailing
axis. Each expression keeps the reference's evaluation order, so the results
are bit-identical to the reference's own (tests/test_oracle_golden.py pins
them against fixtures made by the reference). The Riemann solver and the
primitive recovery are not restated here: the GPU path is checked against
the reference's own outputs for those.
"""
from __future__ import annotations

import numpy as np


def _mean(x, axis):
    """nd::adjacent_mean (src/core_ndarray_ops.hpp:84-90): 0.5 * (x[i] + x[i+1])."""
    a = np.take(x, np.arange(x.shape[axis] - 1), axis=axis)
    b = np.take(x, np.arange(1, x.shape[axis]), axis=axis)
    return 0.5 * (a + b)


def _diff(x, axis):
    """nd::adjacent_diff (src/core_ndarray_ops.hpp:92-98): x[i+1] - x[i]."""
    a = np.take(x, np.arange(x.shape[axis] - 1), axis=axis)
    b = np.take(x, np.arange(1, x.shape[axis]), axis=axis)
    return b - a


def face_to_cell(b1, b2, b3):
    """mesh::face_to_cell (src/mesh_cartesian_3d.hpp:236-242): (n, n, n, 3)."""
    return np.stack([_mean(b1, 0), _mean(b2, 1), _mean(b3, 2)], axis=-1)


def electromotive_forces(gf1, gf2, gf3):
    """electromotive_forces (src/scheme_mhd_v2.cpp:168-192) of godunov data
    arrays (..., 8): E components are entries 5, 6, 7."""
    ee1 = 0.5 * (_mean(gf2[..., 5], 2) + _mean(gf3[..., 5], 1))
    ee2 = 0.5 * (_mean(gf3[..., 6], 0) + _mean(gf1[..., 6], 2))
    ee3 = 0.5 * (_mean(gf1[..., 7], 1) + _mean(gf2[..., 7], 0))
    return ee1, ee2, ee3


def updated_conserved_density(uc, gf1, gf2, gf3, dt, dl):
    """updated_conserved_density (src/scheme_mhd_v2.cpp:197-219): uc
    (n0, n1, n2, 5); godunov data extended by one zone on their transverse
    axes (remove_transverse(1), src/mesh_cartesian_3d.hpp:421-452)."""
    ff1 = gf1[:, 1:-1, 1:-1, :5]
    ff2 = gf2[1:-1, :, 1:-1, :5]
    ff3 = gf3[1:-1, 1:-1, :, :5]
    div = _diff(ff1, 0) + _diff(ff2, 1) + _diff(ff3, 2)
    return uc - div * dt / dl


def solenoidal_difference(e1, e2, e3):
    """mesh::solenoidal_difference (src/mesh_cartesian_3d.hpp:266-273)."""
    return _diff(e3, 1) - _diff(e2, 2), _diff(e1, 2) - _diff(e3, 0), _diff(e2, 0) - _diff(e1, 1)


def curl(ee1, ee2, ee3, dl):
    """curl (src/scheme_mhd_v2.cpp:224-237), with the reference's unit time."""
    return tuple(c * 1.0 / dl for c in solenoidal_difference(ee1, ee2, ee3))


def updated_magnetic_flux_density(bf1, bf2, bf3, ee1, ee2, ee3, dt, dl):
    """updated_magnetic_flux_density (src/scheme_mhd_v2.cpp:242-257): the
    edge EMFs of the extended block lose their longitudinal end layers (rl1..3)."""
    c1, c2, c3 = solenoidal_difference(ee1[1:-1], ee2[:, 1:-1], ee3[:, :, 1:-1])
    return bf1 - c1 * dt / dl, bf2 - c2 * dt / dl, bf3 - c3 * dt / dl
