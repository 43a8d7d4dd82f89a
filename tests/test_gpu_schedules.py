"""The step's schedule changes no result: the autotuned chunk count of the xy
passes and the replay of plain iterations from a captured CUDA graph give the
same bits as pass-by-pass launches with the default schedule.  Each variant
runs in a process of its own (the switches are read once per process)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, math, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import xpfc_cuda_gb300 as X
N, two_d, out = int(sys.argv[2]), sys.argv[3] == "1", sys.argv[4]
FCC = ((2 * math.pi, 1.0, 1.0, 8.0), (2 * math.pi * 2 / math.sqrt(3), 1.0, 1.0, 6.0))
L = N * 0.125
p = X.default_params(Mx=N, My=N, Mz=1 if two_d else N, Lx=L, Ly=L, Lz=1.0 if two_d else L,
                     precision=X._lib.MIXED, t_sample=50, ic_kind=X._lib.IC_NOISE, ic_amp=0.05, ic_seed=2,
                     psi0=0.04, sigma=0.22, peaks=FCC, envelope=X._lib.ENVELOPE_MAX,
                     ff_factor=0.125 ** (2 if two_d else 3), noise_amp=0.01, noise_seed=5)
with X.Xpfc(p) as x:
    x.initialize(None)
    r1 = x.step(73)
    x.step_async(40)
    r2 = x.collect()
    f = x.copy2cpu()
    n = x.launch_count
np.save(out, f)
print(json.dumps({"recs": r1 + r2, "launches": n}))
"""


def _run(tmp_path, tag, N, two_d, env):
    out = str(tmp_path / ("%s.npy" % tag))
    e = dict(os.environ)
    e.update(env)
    r = subprocess.run([sys.executable, "-c", SCRIPT, REPO, str(N), "1" if two_d else "0", out], env=e,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out), json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("N,two_d", [(64, False), (256, False), (512, True)])
def test_schedules_give_the_same_bits(tmp_path, N, two_d):
    base_f, base = _run(tmp_path, "plain", N, two_d, {"XPFC_AUTOTUNE": "0", "XPFC_GRAPH": "0"})
    for tag, env in (("tuned", {"XPFC_AUTOTUNE": "1", "XPFC_GRAPH": "0"}),
                     ("graph", {"XPFC_AUTOTUNE": "0", "XPFC_GRAPH": "1"}),
                     ("both", {"XPFC_AUTOTUNE": "1", "XPFC_GRAPH": "1"}),
                     ("chunks8", {"XPFC_AUTOTUNE": "0", "XPFC_GRAPH": "1", "XPFC_XY_CHUNKS": "8"})):
        f, info = _run(tmp_path, tag, N, two_d, env)
        assert np.array_equal(f, base_f), tag
        assert info["recs"] == base["recs"], tag
