"""The oracle against golden vectors made by the reference's own code.

tests/golden/*.npz come from tests/golden/make_golden.py, which runs
LC2500/XPFC_CUDA's host code and kernel bodies (compiled from the reference
tree with g++, oracle/ref/Makefile) on 2-D square decks.  The oracle must
reproduce the k-grid, the DCF table, the initial conditions with mean pinning,
the free-energy and residual series and the final field.
"""
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["tri32_gauss", "sq32_circle", "liq16", "vtk64_restart"]
REF_PEAKS = ((2 * math.pi, 1.0, 1.0, 4.0), (2 * math.pi * math.sqrt(2), 1.0, 1 / math.sqrt(2), 4.0))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = json.loads(bytes(z["params"]).decode())
    return z, p


def ref_params(O, p):
    Mx, My = int(p["Mx"]), int(p["My"])
    # reference memory is psi[i*My + j]: j (My, Ly) is the fast axis
    return O.make_params(My, Mx, 1, L=(p["Ly"], p["Lx"], 1.0), a=p["a"], b=p["b"], eps=p["eps"],
                         Mo=p["Mo"], dt=p["dt"], sigma=p["s"], peaks=REF_PEAKS, envelope=0,
                         ref_compat=1, ff_factor=p["ff_factor"])


@pytest.mark.parametrize("name", CASES)
def test_kgrid_and_dcf(oracle_mod, name):
    z, p = load(name)
    k2, c2 = oracle_mod.k2_c2(ref_params(oracle_mod, p))
    np.testing.assert_array_equal(k2, z["k2"])
    np.testing.assert_array_equal(c2, z["c2"])


@pytest.mark.parametrize("name", ["tri32_gauss", "sq32_circle", "liq16"])
def test_initial_conditions(oracle_mod, name):
    z, p = load(name)
    d = bytes(z["deck"]).decode().splitlines()
    vals = lambda i: d[i].split()
    A10, A11 = float(vals(12)[0]), float(vals(12)[1])
    Atri = float(vals(13)[0])
    iseed, ishape = int(vals(15)[0]), int(vals(16)[0])
    h, k, roa = (float(v) for v in vals(17)[:3])
    Mx, My = int(p["Mx"]), int(p["My"])
    psi = oracle_mod.ic_reference(Mx, My, int(p["Lx"]), int(p["Ly"]), p["psi_0"], int(p["iconfig"]),
                                  A10, A11, Atri, iseed, ishape, h, k, roa)
    oracle_mod.pin_mean(psi, p["psi_0"])
    # oracle keeps physical x fastest; the reference stores x slowest
    ref = z["psi0"].reshape(Mx, My).T.reshape(-1)
    np.testing.assert_allclose(psi, ref, rtol=0, atol=1e-15)


@pytest.mark.parametrize("name", CASES)
def test_run_matches_reference(oracle_mod, name):
    z, p = load(name)
    P = ref_params(oracle_mod, p)
    nsteps = int(math.ceil(p["N_t_steps"]))          # for (n = 0; n < N_t_steps; n++)
    psi, F, mean, rms = oracle_mod.run(P, z["psi0"].copy(), nsteps, int(p["t_sample"]))
    for it, v in z["F"]:
        assert abs(F[int(it)] - v) <= 1e-13 * abs(v) + 1e-300, (it, F[int(it)], v)
    for it, v in z["RMS"]:
        assert abs(rms[int(it)] - v) <= 1e-9 * abs(v) + 1e-300, (it, rms[int(it)], v)
    assert int(z["FINAL"][0][0]) == nsteps
    assert abs(F[nsteps] - z["FINAL"][0][1]) <= 1e-13 * abs(z["FINAL"][0][1])
    ref = z["psi_final"]
    assert np.linalg.norm(psi - ref) <= 1e-13 * np.linalg.norm(ref)


def test_liquid_stays_uniform(oracle_mod):
    z, p = load("liq16")
    assert np.ptp(z["psi_final"]) <= 1e-16
    np.testing.assert_allclose(z["psi_final"], p["psi_0"], rtol=1e-14)
