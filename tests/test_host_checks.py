"""The Python host mirror rejects arrays whose sizes do not match the call
before anything reaches the device: the C ABI takes bare pointers, so a
short buffer would otherwise be read or written past its end. Runs on the
CPU (the checks come before any CUDA call)."""
from __future__ import annotations

import pytest

torch = pytest.importorskip("torch")

F64 = dict(dtype=torch.float64)


@pytest.fixture(scope="module")
def md():
    import mara3p_gb300.minidisk as md
    return md


def test_minidisk_run_and_substep_need_the_whole_mesh(md):
    sd = md.SolverData(block_size=64, depth=1)           # 128^2 cells
    with pytest.raises(ValueError, match="Run state u"):
        md.Run(sd, torch.zeros(3, 64, 64, **F64))
    with pytest.raises(ValueError, match="Run state u"):
        md.Run(sd, torch.zeros(3, 128, 128, dtype=torch.float32))
    with pytest.raises(ValueError, match="substep u"):
        md.substep(sd, torch.zeros(10, **F64), 0.0, 1e-3)
    with pytest.raises(ValueError, match="substep u_avg"):
        md.substep(sd, torch.zeros(3, 128, 128, **F64), 0.0, 1e-3, u_avg=torch.zeros(3, 127, 128, **F64))


def test_minidisk_rates_check_state_and_increment(md):
    sd = md.SolverData(block_size=64, depth=1)
    with pytest.raises(ValueError, match="rates u"):
        md.rates(sd, torch.zeros(3, 128, 64, **F64), 0.0)
    with pytest.raises(ValueError, match="rates d1"):
        md.rates(sd, torch.zeros(3, 128, 128, **F64), 0.0, d1=torch.zeros(3, 128, 128, **F64))


@pytest.mark.parametrize("shape,axis", [((4, 4), 0), ((6, 6, 2), 0), ((2, 6, 3), 0), ((6, 2, 3), 1), ((6, 6, 3), 2)])
def test_minidisk_estimate_gradient_shapes(md, shape, axis):
    with pytest.raises(ValueError, match="estimate_gradient"):
        md.estimate_gradient(torch.zeros(*shape, **F64), axis, 2.0)


def test_srhd_recovery_and_riemann_shapes():
    import mara3p_gb300.srhd as sr
    with pytest.raises(ValueError, match=r"\(5, n\)"):
        sr.recover_primitive(torch.zeros(4, 10, **F64))
    with pytest.raises(ValueError, match=r"\(n, 5\)"):
        sr.recover_primitive(torch.zeros(10, 4, **F64), layout="aos")
    with pytest.raises(ValueError, match="layout"):
        sr.recover_primitive(torch.zeros(5, 10, **F64), layout="tuple")
    with pytest.raises(ValueError, match="riemann"):
        sr.riemann(torch.zeros(3, 5, **F64), torch.zeros(4, 5, **F64), 1)
    with pytest.raises(ValueError, match="riemann"):
        sr.riemann(torch.zeros(3, 4, **F64), torch.zeros(3, 4, **F64), 1)


def test_mhd_state_sizes():
    import mara3p_gb300.mhd as mh
    cfg = mh.MhdConfig(N=8)
    good = [torch.zeros(9, 8, 8, **F64), torch.zeros(8, 9, 8, **F64), torch.zeros(8, 8, 9, **F64)]
    with pytest.raises(ValueError, match="MHD state of N = 8"):
        mh.Run(mh.State(cfg, torch.zeros(5, 8, 8, 7, **F64), good))
    with pytest.raises(ValueError, match="MHD state of N = 8"):
        mh.Run(mh.State(cfg, torch.zeros(5, 8, 8, 8, **F64), good[:2]))
    with pytest.raises(ValueError, match="MHD state of N = 8"):
        mh.advance_ct(mh.State(cfg, torch.zeros(5, 8, 8, 8, **F64), [good[0], good[1], torch.zeros(8, 8, 8, **F64)]))
    with pytest.raises(ValueError, match="uc_in"):
        mh.advance_ct(mh.State(cfg, torch.zeros(5, 8, 8, 8, **F64), good), uc_in=torch.zeros(8, 8, 8, 4, **F64),
                      layout="aos")
