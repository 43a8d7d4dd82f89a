"""GPU: the hand-written sm_103a transforms against numpy.fft (FP64 staged
buffers, packed real format unpacked by the library)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16, 1), (32, 64, 1), (48, 48, 1), (64, 96, 1), (256, 256, 1), (1024, 1024, 1),
          (16, 16, 16), (32, 32, 32), (24, 32, 48), (48, 48, 48), (96, 96, 96), (128, 128, 128),
          (64, 256, 512), (192, 192, 1), (48, 96, 192), (24, 48, 24), (4096, 64, 1), (512, 16, 16),
          (16, 512, 32), (512, 64, 1)]


@pytest.mark.parametrize("shape", SHAPES)
def test_forward_inverse_match_numpy(shape):
    import xpfc_cuda_gb300 as X
    Mx, My, Mz = shape
    p = X.default_params(Mx=Mx, My=My, Mz=Mz, Lx=8.0, Ly=8.0, Lz=8.0)
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(Mx * My * Mz)
    with X.Xpfc(p) as x:
        x.upload(X._lib.BUF_PSI, a)
        x.cufftXtExecDescriptor(X._lib.BUF_PSI, X._lib.FORWARD)
        spec = x.download_spectrum(X._lib.BUF_PSI)
        ref = np.fft.rfftn(a.reshape(Mx, My, Mz) if Mz > 1 else a.reshape(Mx, My))
        ref = ref.reshape(spec.shape)
        err = np.abs(spec - ref).max() / np.abs(ref).max()
        assert err < 1e-13, err
        x.cufftXtExecDescriptor(X._lib.BUF_PSI, X._lib.INVERSE)
        back = x.download(X._lib.BUF_PSI) / a.size
        assert np.abs(back - a).max() < 1e-13 * np.abs(a).max() * 10
