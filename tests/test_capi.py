"""The C-ABI library: it loads, exports every function include/*.h declares,
and its host-only entry points and argument checks behave. No GPU work."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(mara_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from mara3p_gb300 import _capi
    names = declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(_capi.lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert set(names) <= set(_capi.SIGNATURES), "every declared function needs a ctypes signature"


def declarations() -> list[tuple[str, str, int]]:
    """(return type, name, parameter count) of every function include/*.h declares."""
    out = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"#.*", "", text)
        for ret, name, params in re.findall(r"([A-Za-z_][A-Za-z0-9_ *]*?)\b(mara_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;",
                                            text, flags=re.S):
            p = params.strip()
            out.append((ret.strip(), name, 0 if p in ("", "void") else len(p.split(","))))
    return out


def test_ctypes_signatures_match_the_header():
    """Every binding passes as many arguments as the C declaration takes and
    reads the declared return type, so no call through the ABI is misaligned."""
    from mara3p_gb300 import _capi
    rets = {"int": ctypes.c_int, "int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64,
            "const char*": ctypes.c_char_p, "const char *": ctypes.c_char_p}
    decls = declarations()
    assert len(decls) == len(declared_functions())
    wrong = []
    for ret, name, nparams in decls:
        restype, argtypes = _capi.SIGNATURES[name]
        if len(argtypes) != nparams or rets.get(ret) != restype:
            wrong.append((name, ret, nparams, restype, len(argtypes)))
    assert not wrong, wrong


def test_version_string():
    from mara3p_gb300 import _capi
    assert b"sm_103a" in _capi.lib.mara_version()


def test_binary_matches_reference_golden(golden):
    import mara3p_gb300.minidisk as md
    for i, (q, e, om) in enumerate(golden["binary/cases"]):
        sd = md.SolverData(mass_ratio=q, eccentricity=e, omega_frame=om)
        for j, t in enumerate(golden["binary/times"]):
            got = np.array(md.binary_state(sd, t))
            assert np.allclose(got, golden["binary/state"][i, j], rtol=1e-13, atol=1e-14)


def test_dt_formula_matches_oracle(oracle):
    import mara3p_gb300.minidisk as md
    from oracle.oracle import params
    sd = md.SolverData(block_size=64, depth=2, domain_radius=4.0, softening_length=0.05)
    for t in (0.0, 0.01, 0.04, 0.05, 1.0, 100.0):
        assert md.dt_formula(sd, t) == oracle.oracle_minidisk_dt_formula(ctypes.byref(params(sd)), ctypes.c_double(t))


@pytest.mark.parametrize("bad", [dict(block_size=0), dict(depth=-1), dict(mach_number=0.0), dict(eccentricity=1.0),
                                 dict(buffer_scale=0.0), dict(mass_ratio=-1.0)])
def test_invalid_params_rejected(bad):
    import mara3p_gb300.minidisk as md
    from mara3p_gb300._capi import MaraError
    with pytest.raises(MaraError):
        md.dt_formula(md.SolverData(**bad), 0.0)


def test_advance_rejects_bad_arguments_before_any_gpu_work():
    import mara3p_gb300.minidisk as md
    from mara3p_gb300._capi import lib
    c = md.SolverData().to_c()
    fake = ctypes.c_void_p(0x1000)   # never dereferenced: validation fails first
    assert lib.mara_minidisk_advance(ctypes.byref(c), fake, fake, 1, 3, 0, 0, fake, None) == 1
    assert b"rk_order" in lib.mara_last_error()
    assert lib.mara_minidisk_advance(ctypes.byref(c), fake, fake, 1, 2, 7, 0, fake, None) == 1
    assert lib.mara_minidisk_advance(ctypes.byref(c), None, fake, 1, 2, 0, 0, fake, None) == 1
    assert lib.mara_minidisk_workspace_bytes(ctypes.byref(c), 2, 1) == 3 * (64 << 1) ** 2 * 12 + 64


def test_make_solver_data_rejects_unknown_keys():
    import mara3p_gb300.minidisk as md
    assert md.make_solver_data({"block_size": 32, "nu": 1e-3}).nu == 1e-3
    with pytest.raises(ValueError):
        md.make_solver_data({"block_sise": 32})


def test_srhd_host_recovery_arguments_checked_before_any_gpu_work():
    """The host-buffer recovery's sizes and argument checks need no GPU."""
    from mara3p_gb300._capi import lib
    assert lib.mara_srhd_host_workspace_bytes(-1, 8) == -1
    assert lib.mara_srhd_host_workspace_bytes(100, 0) == -1
    one = lib.mara_srhd_host_workspace_bytes(1000, 1)
    assert one >= 3 * 10 * 1000 * 8 and lib.mara_srhd_host_workspace_bytes(1000, 8) < one
    failed = ctypes.c_ulonglong(7)
    # no zones: nothing to do, and the failure count is cleared
    assert lib.mara_srhd_recover_primitive_host(None, 0, 4.0 / 3, 0.0, None, 0, 0, None, 8, None,
                                                ctypes.byref(failed), None) == 0
    assert failed.value == 0
    fake = ctypes.c_void_p(16)
    assert lib.mara_srhd_recover_primitive_host(fake, 10, 4.0 / 3, 0.0, None, 0, 0, fake, 0, fake, None, None) == 1
    assert b"chunks" in lib.mara_last_error()
    assert lib.mara_srhd_recover_primitive_host(None, 10, 4.0 / 3, 0.0, None, 0, 0, fake, 4, fake, None, None) == 1

