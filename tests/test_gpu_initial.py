"""Initial fields built on the device against the host builder (the
reference's generators, initialize.cu:95-197, the Philox noise liquid and the
fcc seed): equal to rounding, since device and host libm differ in the last
bits of log/cos/exp."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases(X):
    L = 32 * 0.125
    yield X.default_params(Mx=32, My=32, Mz=32, Lx=L, Ly=L, Lz=L, ic_kind=X._lib.IC_NOISE, ic_amp=0.1, ic_seed=5,
                           psi0=0.04)
    yield X.default_params(Mx=48, My=32, Mz=64, Lx=6.0, Ly=4.0, Lz=8.0, ic_kind=X._lib.IC_FCC_SEED, ic_amp=0.05,
                           ic_seed=2, psi0=0.03, ic_seed_amp=0.3, ic_seed_radius=9.0)
    yield X.default_params(Mx=16, My=16, Mz=16, ic_kind=X._lib.IC_FCC_SEED, ic_amp=0.0, psi0=0.0,
                           ic_seed_amp=0.2, ic_seed_radius=0.0)
    for iconfig, iseed, ishape in ((0, 1, 0), (0, 1, 1), (1, 1, 0), (1, 0, 0), (1, 1, 1), (2, 0, 0)):
        yield X.default_params(Mx=64, My=48, Mz=1, Lx=12.0, Ly=9.0, Lz=1.0, ic_kind=X._lib.IC_REFERENCE,
                               iconfig=iconfig, iseed=iseed, ishape=ishape, A_10=0.2, A_11=0.1, A_tri=0.3,
                               h=6.0, k=4.5, roa=3.0, psi0=0.1)


def test_device_initial_fields_match_host():
    import torch

    import xpfc_cuda_gb300 as X
    for p in _cases(X):
        host = X.build_initial_field(p)
        dev = torch.empty(host.size, dtype=torch.float64, device="cuda")
        X.build_initial_field_device(p, dev.data_ptr())
        got = dev.cpu().numpy()
        assert np.max(np.abs(got - host)) <= 1e-13 * max(1.0, np.max(np.abs(host))), (p.ic_kind, p.iconfig)
        assert abs(got.mean() - p.psi0) < 1e-15


def test_initialize_on_device_equals_host_field():
    import xpfc_cuda_gb300 as X
    for p in list(_cases(X))[:2] + list(_cases(X))[3:4]:
        p.precision = X._lib.FP64
        with X.Xpfc(p) as x:
            x.initialize(None)
            a = x.copy2cpu().reshape(-1)
        with X.Xpfc(p) as y:
            y.initialize(X.build_initial_field(p))
            b = y.copy2cpu().reshape(-1)
        assert np.max(np.abs(a - b)) <= 1e-13


def test_vtk_restart_still_read_on_host(tmp_path):
    import xpfc_cuda_gb300 as X
    from tests_vtk import write_restart
    field = 0.05 + 0.1 * np.random.default_rng(3).standard_normal(32 * 32)
    write_restart(tmp_path / "r.vtk", field, 32, 32, 0.125)
    p = X.default_params(Mx=32, My=32, Mz=1, Lx=4.0, Ly=4.0, Lz=1.0, ic_kind=X._lib.IC_REFERENCE, iconfig=10,
                         vtk_path=str(tmp_path / "r.vtk"), psi0=0.05, precision=X._lib.FP64)
    with X.Xpfc(p) as x:
        x.initialize(None)
        got = x.copy2cpu().reshape(-1)
    assert np.max(np.abs(got - X.build_initial_field(p))) <= 1e-13
