"""The oracle against the reference's own program run on a GB300 (CPU).

tests/golden/gpu_xp_noise512_*.npz hold what LC2500/XPFC_CUDA's CUDA program
printed and wrote for the 512^2 noise-liquid decks on one GB300, built with
17-digit output and its powers in double precision (power_functions.cu:47,
powf -> pow; tests/golden/make_golden_gpu.py --exact-powers).  With exact
powers the reference's step has no float rounding of psi, so the oracle (its
own FFT in place of cuFFT, the reference's kernels restated) must reproduce
that run to rounding: F at every printed iteration and the final field.  This
pins the oracle to the reference's GPU output as well as to its host-compiled
code (test_oracle_golden.py).
"""
import os

import numpy as np
import pytest

from helpers import oracle_params, rel_l2

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.timeout(600)
@pytest.mark.parametrize("name", ["noise512_t60", "noise512q_t2000"])
def test_oracle_matches_reference_gpu_run_exact_powers(oracle_mod, name, tmp_path):
    import xpfc_cuda_gb300 as X
    from tests_vtk import write_restart
    z = np.load(os.path.join(GOLDEN, "gpu_xp_%s.npz" % name))
    # the restart field (read_input.cu:208-218 keeps the file's order), from
    # the fixture's seed
    amp = float(z["vtk_amp"][0])
    psi = 0.05 + amp * np.random.default_rng(int(z["vtk_seed"][0])).standard_normal(512 * 512)
    (tmp_path / "pfc.input").write_text(bytes(z["deck"]).decode())
    # the deck's restart file sits beside it
    write_restart(tmp_path / "initial_density_field.vtk", psi, 512, 512, 0.125)
    p = X.read_input(str(tmp_path / "pfc.input"))
    p.ref_compat = 0
    n = int(z["final_iteration"][0])
    assert p.nsteps == n and p.Mx == p.My == 512 and p.Mz == 1
    # the reference's mean pin (Avg_calc.cu:3-43, one running sum)
    psi = oracle_mod.pin_mean(psi, p.psi0)
    final, F, _, _ = oracle_mod.run(oracle_params(oracle_mod, p), psi, n, p.t_sample)
    for it, v in z["F"]:
        assert abs(F[int(it)] - v) <= 1e-12 * abs(v), (it, F[int(it)], v)
    assert rel_l2(final, z["psi_final"]) <= 1e-10
