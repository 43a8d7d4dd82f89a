"""GPU parity against LC2500/XPFC_CUDA's own program run on a GB300.

tests/golden/gpu_<deck>.npz hold what the reference's own CUDA program
printed and wrote for six pfc.input decks when run on one GB300 (built for
sm_103a from its unmodified sources by baseline/ref_gpu.py, cuFFT for its
transforms, output precision raised to 17 digits; generator:
tests/golden/make_golden_gpu.py).  The library runs the same decks in
reference semantics (ref_compat: the float powf powers of
power_functions.cu:47, the reference's two-peak sum kernel, its ff_factor and
step count) from the same initial field and must reproduce:

* the per-stage entry points driven in main.cu's order (run_reference_loop):
  final field rel-L2 <= 1e-10, free energy rel <= 1e-12 at every printed
  iteration, residual RMS rel <= 1e-8 (it squares in float, as the reference
  does at sse_calculation.cu:38);
* the fused step in reference semantics: field <= 1e-10, F <= 1e-12.

Both sides compute the powers with the device's powf, so the only differences
are the transforms' rounding (cuFFT against the library's own FFT).  The
two 512^2 decks with noise 0.1 start at the explicit scheme's stability
edge; their measured tolerances are stated beside them.
"""
import json
import math
import os

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["tri32_gauss", "sq32_circle", "liq16", "vtk64_restart", "noise512_t60", "noise512_t2000",
         "noise512q_t2000"]


def _vtk_text(values, n, spacing=0.125):
    head = ("# vtk DataFile Version 3.0\nDensity Data\nASCII\nDATASET STRUCTURED_POINTS\n"
            f"DIMENSIONS {n} {n} 1\nORIGIN 0 0 0\nSPACING {spacing} {spacing} 1\n"
            f"POINT_DATA {n * n}\nSCALARS DensityData float\nLOOKUP_TABLE default\n")
    return head + "".join(f"{v:.17g}\n" for v in values)


def _case(X, name, tmp_path):
    z = np.load(os.path.join(GOLDEN, "gpu_%s.npz" % name))
    (tmp_path / "pfc.input").write_text(bytes(z["deck"]).decode())
    vtk = None
    if "vtk_in" in z.files:
        vtk = z["vtk_in"]
    elif "vtk_seed" in z.files:
        amp = float(z["vtk_amp"][0]) if "vtk_amp" in z.files else 0.1
        vtk = 0.05 + amp * np.random.default_rng(int(z["vtk_seed"][0])).standard_normal(512 * 512)
    if vtk is not None:
        (tmp_path / "initial_density_field.vtk").write_text(_vtk_text(vtk, int(round(math.sqrt(vtk.size)))))
    p = X.read_input(str(tmp_path / "pfc.input"))
    assert p.ref_compat == 1 and p.Mz == 1
    assert p.nsteps == int(z["final_iteration"][0])
    # the reference's restart stores the file's values in file order into its
    # [Mx][My] array (read_input.cu:208-218); xpfc_initialize pins the mean
    # as configure_avg_density does (Avg_calc.cu:21-43)
    psi0 = vtk.copy() if vtk is not None else X.build_initial_field(p)
    return z, p, psi0


def test_reference_fixtures_record_the_one_gpu_build():
    """The fixtures come from the reference program on one GB300; its build
    against cuFFT as shipped stops at cufftXtSetGPUs with one GPU."""
    z = np.load(os.path.join(GOLDEN, "gpu_liq16.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    assert "GB300" in meta["gpu"]
    assert meta["stock_cufft_xt_one_gpu"]["returncode"] != 0
    assert any("CUFFT_INVALID_VALUE" in ln for ln in meta["stock_cufft_xt_one_gpu"]["lines"])


# Tolerances: (field rel-L2, F rel, residual RMS rel, last iteration whose RMS
# is compared).  Measured on GB300: the four small decks and the quieter
# 512^2 liquid agree with the reference's run to F 1e-13 and field 3e-15.
# The 512^2 liquid with noise 0.1 starts with its minimum near -0.41 (the
# lowest of 262144 draws, 4.5 sigma below 0.05), where the explicit
# nonlinear term maps a high-k mode n to -N(n) with |N'| near 1: there the
# last-bit differences of two FFTs (cuFFT's and the library's) grow during
# the first steps, and the float powf of the reference semantics turns some of
# them into one-float-ulp jumps of n^2 and n^3.  Measured: F 3.1e-11 and field
# 5.7e-10 after 61 steps, F 2.9e-9 and field 1.2e-8 after 2001, with the
# residual RMS (a float-squared residual of a relaxed liquid) resolved only
# at the first sample.
TOL = {"noise512_t60": (2e-9, 1e-10, 1e-6, 0), "noise512_t2000": (5e-8, 1e-8, 1e-6, 0)}
DEFAULT_TOL = (1e-10, 1e-12, 1e-8, None)


@pytest.mark.parametrize("name", CASES)
def test_staged_loop_matches_reference_gpu_run(name, tmp_path):
    import xpfc_cuda_gb300 as X
    z, p, psi0 = _case(X, name, tmp_path)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        F, R = X.run_reference_loop(x, p.nsteps, p.t_sample)
        final = x.download(X._lib.BUF_PSI_NP1_R)
    ftol, Ftol, rtol, rlast = TOL.get(name, DEFAULT_TOL)
    for it, v in z["F"]:
        assert abs(F[int(it)] - v) <= Ftol * abs(v), (it, F[int(it)], v)
    for it, v in z["RMS"]:
        if rlast is None or it <= rlast:
            assert abs(R[int(it)] - v) <= rtol * abs(v) + 1e-14, (it, R[int(it)], v)
    assert rel_l2(final, z["psi_final"]) <= ftol


@pytest.mark.parametrize("name", CASES)
def test_fused_step_matches_reference_gpu_run(name, tmp_path):
    import xpfc_cuda_gb300 as X
    z, p, psi0 = _case(X, name, tmp_path)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        recs = x.step(p.nsteps)
        field = x.copy2cpu().reshape(-1)
    got = {r["iteration"]: r["F"] for r in recs if r["F"] is not None}
    ftol, Ftol, _, _ = TOL.get(name, DEFAULT_TOL)
    seen = 0
    for it, v in z["F"]:
        if int(it) in got:
            assert abs(got[int(it)] - v) <= Ftol * abs(v), (it, got[int(it)], v)
            seen += 1
    assert seen >= 2
    assert rel_l2(field, z["psi_final"]) <= ftol
