"""CPU checks of the C-ABI library: it loads, exports every entry point that
include/xpfc.h declares, its parameter struct matches the header's layout, and
the host-side boundary (deck, VTK, initial fields, errors) works without a GPU."""
import ctypes as C
import json
import os
import re
import subprocess
import textwrap

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "xpfc.h")
GOLDEN = os.path.join(REPO, "tests", "golden")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xpfc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    import xpfc_cuda_gb300 as X
    L = X.load()
    names = declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", X._lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (xpfc_\w+)", out))
    assert set(names) <= exported, set(names) - exported


def test_binding_covers_the_header():
    from xpfc_cuda_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared()) <= bound, set(declared()) - bound


def test_params_layout_matches_header(tmp_path):
    from xpfc_cuda_gb300._lib import XpfcParams, XpfcDiag
    prog = tmp_path / "layout.c"
    fields = ["Mx", "Lx", "psi0", "nsteps", "t_sample", "npeaks", "pk_k", "pk_beta", "envelope", "ff_factor",
              "noise_seed", "ic_kind", "A_10", "roa", "ic_seed", "ic_seed_radius", "vtk_path", "device", "stream"]
    body = "".join('printf("%%s %%zu\\n", "%s", offsetof(xpfc_params, %s));\n' % (f, f) for f in fields)
    from xpfc_cuda_gb300 import _lib as LB
    server_body = ""
    for struct, cls in (("xpfc_server_config", LB.XpfcServerConfig), ("xpfc_request_info", LB.XpfcRequestInfo),
                        ("xpfc_server_stats", LB.XpfcServerStats)):
        server_body += 'printf("%s %%zu\\n", sizeof(%s));\n' % (struct, struct)
        server_body += "".join('printf("%s.%s %%zu\\n", offsetof(%s, %s));\n' % (struct, f, struct, f)
                               for f, _ in cls._fields_)
    prog.write_text(textwrap.dedent("""
        #include <stdio.h>
        #include <stddef.h>
        #include "xpfc.h"
        int main(void) {
        printf("sizeof %zu\\n", sizeof(xpfc_params));
        printf("diag %zu\\n", sizeof(xpfc_diag));
        """) + body + server_body + "return 0; }\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(prog), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")
               if line)
    assert int(out["sizeof"]) == C.sizeof(XpfcParams)
    assert int(out["diag"]) == C.sizeof(XpfcDiag)
    from xpfc_cuda_gb300 import _lib
    for struct, cls in (("xpfc_server_config", _lib.XpfcServerConfig), ("xpfc_request_info", _lib.XpfcRequestInfo),
                        ("xpfc_server_stats", _lib.XpfcServerStats)):
        assert int(out[struct]) == C.sizeof(cls), struct
        for f, _ in cls._fields_:
            assert int(out[struct + "." + f]) == getattr(cls, f).offset, (struct, f)
    for f in fields:
        assert int(out[f]) == getattr(XpfcParams, f).offset, f


def _golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return z, json.loads(bytes(z["params"]).decode())


@pytest.mark.parametrize("name", ["tri32_gauss", "sq32_circle", "liq16", "vtk64_restart"])
def test_read_input_matches_reference(name, tmp_path):
    import xpfc_cuda_gb300 as X
    from tests_vtk import write_restart
    z, meta = _golden(name)
    (tmp_path / "pfc.input").write_text(bytes(z["deck"]).decode())
    if "vtk_in" in z.files:
        write_restart(tmp_path / "initial_density_field.vtk", z["vtk_in"], 64, 64, 0.125)
    p = X.read_input(str(tmp_path / "pfc.input"))
    assert (p.Mx, p.My, p.Mz) == (int(meta["Mx"]), int(meta["My"]), 1)
    assert (p.Lx, p.Ly) == (meta["Lx"], meta["Ly"])          # incl. lattice scaling / VTK box size
    assert p.psi0 == meta["psi_0"] and p.sigma == meta["s"]
    assert p.a == meta["a"] and p.b == meta["b"] and p.eps == meta["eps"] and p.Mo == meta["Mo"]
    assert p.dt == meta["dt"] and p.t_sample == int(meta["t_sample"]) and p.iconfig == int(meta["iconfig"])
    assert p.ff_factor == meta["ff_factor"]
    import math
    assert p.nsteps == math.ceil(meta["N_t_steps"])
    assert p.npeaks == 2 and p.envelope == X._lib.ENVELOPE_SUM and p.ref_compat == 1


@pytest.mark.parametrize("name", ["tri32_gauss", "sq32_circle", "liq16"])
def test_initial_field_matches_reference(name, tmp_path):
    """initialize.cu's lattices, seeds and mean pinning, bit for bit."""
    import xpfc_cuda_gb300 as X
    z, meta = _golden(name)
    (tmp_path / "pfc.input").write_text(bytes(z["deck"]).decode())
    p = X.read_input(str(tmp_path / "pfc.input"))
    psi = X.build_initial_field(p)
    np.testing.assert_array_equal(psi, z["psi0"])


def test_restart_reader_and_pinning(tmp_path):
    """iconfig = 10: the field comes from the VTK file (x fastest in the file,
    stored [Mx][My]); the reference's reader stores the file sequentially,
    i.e. transposed, which for this square grid is its psi0 transposed."""
    import xpfc_cuda_gb300 as X
    from tests_vtk import write_restart
    z, meta = _golden("vtk64_restart")
    (tmp_path / "pfc.input").write_text(bytes(z["deck"]).decode())
    write_restart(tmp_path / "initial_density_field.vtk", z["vtk_in"], 64, 64, 0.125)
    p = X.read_input(str(tmp_path / "pfc.input"))
    psi = X.build_initial_field(p)
    ref_t = z["psi0"].reshape(64, 64).T.reshape(-1)
    np.testing.assert_allclose(psi, ref_t, rtol=0, atol=1e-15)
    assert abs(psi.mean() - p.psi0) < 1e-15


@pytest.mark.parametrize("name", ["tri32_gauss", "liq16"])
def test_vtk_writer_matches_reference_bytes(name, tmp_path):
    import xpfc_cuda_gb300 as X
    z, meta = _golden(name)
    out = tmp_path / "density_data0.vtk"
    X.writeVTKFile(str(out), z["psi0"], int(meta["Mx"]), int(meta["My"]), 1, meta["Lx"], meta["Ly"], 1.0, 6)
    assert out.read_bytes() == bytes(z["vtk0"])
    back, dims, box = X.read_density_field(str(out))
    assert dims == (int(meta["Mx"]), int(meta["My"]), 1)
    np.testing.assert_allclose(back, z["psi0"], rtol=1e-5)


def test_vtk_3d_round_trip(tmp_path):
    import xpfc_cuda_gb300 as X
    a = np.random.default_rng(3).standard_normal(6 * 8 * 10)
    X.writeVTKFile(str(tmp_path / "f.vtk"), a, 6, 8, 10, 3.0, 4.0, 5.0, 17)
    back, dims, box = X.read_density_field(str(tmp_path / "f.vtk"))
    assert dims == (6, 8, 10)
    np.testing.assert_allclose(box, (3.0, 4.0, 5.0), rtol=1e-6)
    np.testing.assert_array_equal(back, a)


def test_noise_initial_field_matches_oracle(oracle_mod):
    import xpfc_cuda_gb300 as X
    p = X.default_params(Mx=8, My=12, Mz=16, ic_kind=X._lib.IC_NOISE, ic_amp=0.1, ic_seed=5, psi0=0.03)
    psi = X.build_initial_field(p)
    ref = oracle_mod.ic_noise(16, 12, 8, 0.03, 0.1, 5)
    oracle_mod.pin_mean(ref, 0.03)
    np.testing.assert_array_equal(psi, ref)


def test_error_paths(tmp_path):
    import xpfc_cuda_gb300 as X
    with pytest.raises(X.XpfcError) as e:
        X.read_input(str(tmp_path / "missing.input"))
    assert e.value.status == X._lib.EIO
    (tmp_path / "short.input").write_text("1\n0.05 0.1\n1 3 0 1\n")
    with pytest.raises(X.XpfcError) as e:
        X.read_input(str(tmp_path / "short.input"))
    assert e.value.status == X._lib.EIO
    z, _ = _golden("liq16")
    bad = bytes(z["deck"]).decode().splitlines()
    bad[11] = "7 iconfig"
    (tmp_path / "bad.input").write_text("\n".join(bad) + "\n")
    with pytest.raises(X.XpfcError) as e:
        X.read_input(str(tmp_path / "bad.input"))
    assert e.value.status == X._lib.EINVAL
    for kw in (dict(Mx=31, My=32, Mz=1), dict(Mx=32, My=32, Mz=0), dict(Mx=32, My=1000, Mz=1), dict(dt=0.0)):
        with pytest.raises(X.XpfcError) as e:
            X.Xpfc(X.default_params(**kw))
        assert e.value.status == X._lib.EINVAL
    (tmp_path / "trunc.vtk").write_text("# vtk DataFile Version 3.0\nDensity Data\nASCII\nDATASET STRUCTURED_POINTS\n"
                                        "DIMENSIONS 4 4 1\nORIGIN 0 0 0\nSPACING 1 1 1\nPOINT_DATA 16\n"
                                        "SCALARS DensityData float\nLOOKUP_TABLE default\n0.1\n0.2\n")
    with pytest.raises(X.XpfcError) as e:
        X.read_density_field(str(tmp_path / "trunc.vtk"))
    assert e.value.status == X._lib.EIO


def test_extension_lines(tmp_path):
    import xpfc_cuda_gb300 as X
    z, _ = _golden("liq16")
    deck = bytes(z["deck"]).decode() + ("Mz = 16\nLz = 4\nprecision = mixed\nenvelope = max\nnoise_amp = 0.01\n"
                                        "peaks = 6.283185307179586,1,1,8; 7.255197456936871,1,1,6\nref_compat = 0\n")
    (tmp_path / "pfc.input").write_text(deck)
    p = X.read_input(str(tmp_path / "pfc.input"))
    assert p.Mz == 16 and p.Lz == 4.0 and p.precision == X._lib.MIXED and p.envelope == X._lib.ENVELOPE_MAX
    assert p.noise_amp == 0.01 and p.npeaks == 2 and p.pk_beta[1] == 6.0 and p.ref_compat == 0


def test_batch_rejects_bad_input():
    """xpfc_batch_create checks its arguments before touching a device."""
    import xpfc_cuda_gb300 as X
    with pytest.raises(X.XpfcError) as e:
        X.Batch([])
    assert e.value.status == X._lib.EINVAL
    ok = X.default_params(Mx=32, My=32, Mz=32, Lx=4.0, Ly=4.0, Lz=4.0)
    for bad in (dict(Lx=4.0, Ly=5.0), dict(Mx=31), dict(dt=0.0), dict(npeaks=0)):
        with pytest.raises(X.XpfcError) as e:
            X.Batch([ok, X.default_params(**dict(dict(Mx=32, My=32, Mz=32, Lx=4.0, Ly=4.0, Lz=4.0), **bad))])
        assert e.value.status == X._lib.EINVAL, bad
