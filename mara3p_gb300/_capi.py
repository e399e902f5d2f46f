"""ctypes binding of include/mara_gb300.h.

The library is loaded from this package directory. There is no fallback: if
libmara_gb300.so is missing or fails to load, importing raises, so nothing can
silently run on the CPU instead.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmara_gb300.so"

c_double_p = ctypes.POINTER(ctypes.c_double)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_int32_p = ctypes.POINTER(ctypes.c_int32)


class MinidiskParams(ctypes.Structure):
    """mara_minidisk_params: field-for-field minidisk::solver_data_t
    (problems/minidisk.hpp:77-93) plus plm_theta."""

    _fields_ = [
        ("block_size", ctypes.c_int32),
        ("depth", ctypes.c_int32),
        ("omega_frame", ctypes.c_double),
        ("mach_number", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("domain_radius", ctypes.c_double),
        ("softening_length", ctypes.c_double),
        ("eccentricity", ctypes.c_double),
        ("mass_ratio", ctypes.c_double),
        ("sink_radius", ctypes.c_double),
        ("sink_rate", ctypes.c_double),
        ("buffer_rate", ctypes.c_double),
        ("buffer_scale", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("plm_theta", ctypes.c_double),
    ]


class MinidiskClock(ctypes.Structure):
    _fields_ = [
        ("time", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("max_wavespeed", ctypes.c_double),
        ("iteration", ctypes.c_int64),
        ("binary", ctypes.c_double * 12),
    ]


DIAG_COUNT = 16


class MinidiskDiagnostics(ctypes.Structure):
    """mara_minidisk_diagnostics: per-stage rate vectors of the last step,
    their time integrals over the completed steps, and the step count."""

    _fields_ = [
        ("rate", (ctypes.c_double * DIAG_COUNT) * 2),
        ("integral", ctypes.c_double * DIAG_COUNT),
        ("steps", ctypes.c_int64),
    ]


# (name, restype, argtypes) for every exported entry point of include/mara_gb300.h.
_vp = ctypes.c_void_p
_MP = ctypes.POINTER(MinidiskParams)
SIGNATURES = {
    "mara_last_error": (ctypes.c_char_p, []),
    "mara_version": (ctypes.c_char_p, []),
    "mara_graph_upload": (ctypes.c_int, [_vp, _vp]),
    "mara_minidisk_binary": (ctypes.c_int, [_MP, ctypes.c_double, c_double_p]),
    "mara_minidisk_dt_formula": (ctypes.c_int, [_MP, ctypes.c_double, c_double_p]),
    "mara_minidisk_updated_conserved": (ctypes.c_int, [_MP, _vp, _vp, ctypes.c_double, ctypes.c_double,
                                                       ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, _vp, _vp]),
    "mara_minidisk_recover_primitive": (ctypes.c_int, [_vp, ctypes.c_int64, _vp, _vp]),
    "mara_minidisk_estimate_gradient": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                                       ctypes.c_double, _vp, _vp]),
    "mara_minidisk_substep": (ctypes.c_int, [_MP, _vp, _vp, _vp, ctypes.c_double, ctypes.c_double, _vp]),
    "mara_minidisk_initial_conserved": (ctypes.c_int, [_MP, ctypes.c_uint64, ctypes.c_double, _vp, _vp]),
    "mara_minidisk_workspace_bytes": (ctypes.c_int64, [_MP, ctypes.c_int32, ctypes.c_int32]),
    "mara_minidisk_clock_init": (ctypes.c_int, [_MP, _vp, ctypes.c_double, _vp, _vp]),
    "mara_minidisk_advance": (ctypes.c_int, [_MP, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_int32, _vp, _vp]),
    "mara_minidisk_host_workspace_bytes": (ctypes.c_int64, [_MP, ctypes.c_int32, ctypes.c_int32]),
    "mara_minidisk_advance_host": (ctypes.c_int, [_MP, _vp, _vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.c_int32, ctypes.c_int32, c_double_p, _vp, _vp]),
    "mara_minidisk_stage": (ctypes.c_int, [_MP, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int32,
                                           ctypes.c_int32, _vp]),
    "mara_minidisk_clock_update": (ctypes.c_int, [_MP, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.c_int32, _vp]),
    "mara_minidisk_sweep_columns": (ctypes.c_int, [ctypes.c_int32]),
    "mara_minidisk_sweep_shape": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32]),
    "mara_sedov_workspace_bytes": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int64]),
    "mara_sedov_stage": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_double,
                                        ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "mara_sedov_advance": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp,
                                          ctypes.c_double, ctypes.c_int32, ctypes.c_int32, _vp, _vp, _vp]),
    "mara_sedov_min_spacing": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, _vp, _vp, _vp, _vp]),
    "mara_sedov_remesh_workspace_bytes": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int64]),
    "mara_sedov_remesh": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, _vp, _vp, _vp,
                                         ctypes.POINTER(ctypes.c_int64), _vp, _vp, _vp]),
    "mara_minidisk_diagnostics_reset": (ctypes.c_int, [_vp, _vp]),
    "mara_minidisk_advance_diag": (ctypes.c_int, [_MP, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.c_int32, _vp, _vp, _vp]),
    "mara_minidisk_rates": (ctypes.c_int, [_MP, _vp, _vp, ctypes.c_double, _vp, _vp]),
    "mara_two_body_elements": (ctypes.c_int, [c_double_p, ctypes.c_double, c_double_p]),
    "mara_two_body_element_rates": (ctypes.c_int, [c_double_p, ctypes.c_double, c_double_p, c_double_p]),
    "mara_minidisk_advance_noalloc": (ctypes.c_int, [_MP, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                     ctypes.c_int32, _vp]),
    "mara_srhd_recover_primitive": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                                   ctypes.c_double, ctypes.c_double, _vp, ctypes.c_int32,
                                                   ctypes.c_int32, _vp, _vp, _vp, _vp, _vp]),
    "mara_srhd_host_workspace_bytes": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_int32]),
    "mara_srhd_recover_primitive_host": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_double, ctypes.c_double, _vp,
                                                        ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_int32, _vp, _vp,
                                                        _vp]),
    "mara_srhd_seeded_zones": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _vp,
                                              _vp, _vp]),
    "mara_srhd_mlp_weights_bytes": (ctypes.c_int64, []),
    "mara_srhd_mlp_param_count": (ctypes.c_int32, []),
    "mara_srhd_mlp_workspace_bytes": (ctypes.c_int64, [ctypes.c_int64]),
    "mara_srhd_mlp_prepare": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, ctypes.c_uint64, _vp, _vp]),
    "mara_srhd_mlp_gradient": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp]),
    "mara_srhd_mlp_train": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_float, _vp, _vp]),
    "mara_srhd_mlp_infer": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp]),
}


class MhdParams(ctypes.Structure):
    """mara_mhd_params."""

    _fields_ = [("N", ctypes.c_int32), ("gamma_law_index", ctypes.c_double), ("cfl", ctypes.c_double),
                ("plm_theta", ctypes.c_double)]


_HP = ctypes.POINTER(MhdParams)
SIGNATURES.update({
    "mara_mhd_clock_bytes": (ctypes.c_int64, []),
    "mara_mhd_fused_stage": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32]),
    "mara_mhd_clock_init": (ctypes.c_int, [_vp, ctypes.c_double, _vp]),
    "mara_mhd_workspace_bytes": (ctypes.c_int64, [_HP, ctypes.c_int32, ctypes.c_int32]),
    "mara_mhd_advance_ct": (ctypes.c_int, [_HP, _vp, ctypes.c_int64, ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                           _vp, ctypes.c_int32, _vp, _vp]),
    "mara_mhd_advance": (ctypes.c_int, [_HP, _vp, _vp, _vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        _vp, _vp]),
    "mara_mhd_mode_table": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int32, c_double_p]),
    "mara_mhd_initial_state": (ctypes.c_int, [_HP, c_double_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double, _vp,
                                              _vp, _vp, _vp, _vp, _vp]),
    "mara_mhd_max_div_b": (ctypes.c_int, [_HP, _vp, _vp, _vp, _vp, _vp]),
})


class EnsembleConfig(ctypes.Structure):
    """mara_ensemble_config."""

    _fields_ = [("blocks_per_sm", ctypes.c_int32), ("chunks_per_warp", ctypes.c_int32),
                ("cols_per_lane", ctypes.c_int32), ("register_variant", ctypes.c_int32),
                ("stage_ms", ctypes.c_double)]


_EC = ctypes.POINTER(EnsembleConfig)
_i32p = ctypes.POINTER(ctypes.c_int32)
SIGNATURES.update({
    "mara_minidisk_ensemble_plan": (ctypes.c_int64, [_i32p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _i32p,
                                                     ctypes.c_int64, _i32p]),
    "mara_minidisk_ensemble_create": (ctypes.c_int, [_MP, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p), _vp,
                                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                     ctypes.POINTER(ctypes.c_void_p)]),
    "mara_minidisk_ensemble_clock_init": (ctypes.c_int, [_vp, ctypes.c_double, _vp]),
    "mara_minidisk_ensemble_advance": (ctypes.c_int, [_vp, ctypes.c_int32, _vp]),
    "mara_minidisk_ensemble_get_config": (ctypes.c_int, [_vp, _EC]),
    "mara_minidisk_ensemble_set_config": (ctypes.c_int, [_vp, _EC]),
    "mara_minidisk_ensemble_tune": (ctypes.c_int, [_vp]),
    "mara_minidisk_ensemble_stage_times": (ctypes.c_int, [_vp, ctypes.c_int32, c_double_p]),
    "mara_minidisk_ensemble_destroy": (ctypes.c_int, [_vp]),
})

SIGNATURES.update({
    "mara_srhd_tube_clock_bytes": (ctypes.c_int64, []),
    "mara_srhd_tube_workspace_bytes": (ctypes.c_int64, [ctypes.c_int32]),
    "mara_srhd_tube_initial": (ctypes.c_int, [ctypes.c_int32] + [ctypes.c_double] * 6 + [_vp, _vp, _vp]),
    "mara_srhd_tube_advance": (ctypes.c_int, [ctypes.c_int32, _vp, _vp, ctypes.c_int32] + [ctypes.c_double] * 4 +
                               [ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp]),
    "mara_srhd_riemann": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                                         _vp, _vp, _vp]),
    "mara_measure_fp64_rate": (ctypes.c_int, [c_double_p, _vp]),
    "mara_measure_host_link": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, c_double_p, _vp]),
    "mara_check_conversions": (ctypes.c_int, [ctypes.POINTER(ctypes.c_ulonglong), _vp]),
    "mara_minidisk_sweep_tma": (ctypes.c_int, [ctypes.c_int32]),
    # mhd_scheme_v2 block API and pointwise physics
    "mara_mhd_v2_primitive_array": (ctypes.c_int, [ctypes.c_int32] * 3 + [_vp] * 4 + [ctypes.c_double, _vp, _vp, _vp]),
    "mara_mhd_v2_godunov_fluxes": (ctypes.c_int, [ctypes.c_int32] * 3 + [_vp] * 4 + [ctypes.c_double] + [_vp] * 4),
    "mara_mhd_v2_electromotive_forces": (ctypes.c_int, [ctypes.c_int32] * 3 + [_vp] * 7),
    "mara_mhd_v2_updated_conserved_density": (ctypes.c_int, [ctypes.c_int32] * 3 + [_vp] * 4 +
                                              [ctypes.c_double] * 2 + [_vp, _vp]),
    "mara_mhd_v2_curl": (ctypes.c_int, [ctypes.c_int32] * 3 + [_vp] * 3 + [ctypes.c_double] + [_vp] * 4),
    "mara_mhd_v2_updated_magnetic_flux_density": (ctypes.c_int, [ctypes.c_int32] * 3 + [_vp] * 6 +
                                                  [ctypes.c_double] * 2 + [_vp] * 4),
    "mara_mhd_recover_primitive": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_double, _vp, _vp, _vp, _vp]),
    "mara_mhd_conserved_density": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_double, _vp, _vp]),
    "mara_mhd_flux": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _vp, _vp]),
    "mara_mhd_fast_speed_squared": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _vp, _vp]),
    "mara_mhd_fastest_speed": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_double, _vp, _vp]),
    "mara_mhd_riemann_hlle": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _vp,
                                             _vp]),
    "mara_iso2d_flux": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp]),
    "mara_iso2d_outer_wavespeeds": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp]),
    "mara_iso2d_fastest_wavespeed": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp]),
    "mara_iso2d_riemann_hlle": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp]),
})


class MaraError(RuntimeError):
    pass


def load(path: Path = LIB_PATH) -> ctypes.CDLL:
    if not path.exists():
        raise ImportError(
            f"{path.name} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA extension is required; there is no CPU fallback)")
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = load()


def check(status: int, what: str = "") -> None:
    """Raise MaraError with the library's message on a non-zero status."""
    if status != 0:
        msg = lib.mara_last_error().decode(errors="replace")
        raise MaraError(f"{what or 'mara call'} failed (status {status}): {msg}")
