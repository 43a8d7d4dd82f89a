"""Host-side mirror of LC2500/XPFC_CUDA's interface over libxpfc.

The reference is one program whose time loop (main.cu:306-435) calls host
wrappers declared at globals.cuh:117-141.  `Xpfc` exposes those wrappers
under the same names, taking buffer ids where the reference passes
cudaLibXtDesc descriptors, plus the fused `step` that replaces the loop body.
Every failure raises XpfcError carrying the C status (the reference exits the
process instead, helpers_header.cuh:84-85).
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import XpfcDiag, XpfcParams


class XpfcError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (_lib.STATUS_NAMES.get(status, status), message))
        self.status = status


def _check(rc, ctx=None):
    if rc != _lib.OK:
        L = _lib.load()
        msg = L.xpfc_last_error(ctx)
        raise XpfcError(rc, msg.decode() if msg else "")
    return rc


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_params(**kw):
    """xpfc_default_params plus keyword overrides (peaks given as
    [(k, alpha, rho, beta), ...])."""
    p = XpfcParams()
    _check(_lib.load().xpfc_default_params(C.byref(p)))
    set_params(p, **kw)
    return p


def set_params(p, **kw):
    for key, val in kw.items():
        if key == "peaks":
            p.npeaks = len(val)
            for i, (k, al, rho, beta) in enumerate(val):
                p.pk_k[i], p.pk_alpha[i], p.pk_rho[i], p.pk_beta[i] = k, al, rho, beta
        elif key == "vtk_path":
            p.vtk_path = val.encode()
        else:
            if not hasattr(p, key):
                raise AttributeError("xpfc_params has no field %r" % key)
            setattr(p, key, val)
    return p


def read_input(path):
    """read_input.cu:8-121: parse a pfc.input deck into xpfc_params."""
    p = XpfcParams()
    _check(_lib.load().xpfc_read_input(path.encode(), C.byref(p)))
    return p


def build_initial_field(p):
    """initialize.cu:95-204 as the library builds it (mean pinned)."""
    out = np.empty(p.Mx * p.My * p.Mz)
    _check(_lib.load().xpfc_build_initial_field(C.byref(p), _dp(out)))
    return out


def build_initial_field_device(p, dev_ptr, stream=None):
    """The same field built on the device into dev_ptr (Mx*My*Mz doubles)."""
    _check(_lib.load().xpfc_build_initial_field_device(C.byref(p), C.c_void_p(dev_ptr), C.c_void_p(stream or 0)))


def writeVTKFile(path, psi, Mx, My, Mz=1, Lx=1.0, Ly=1.0, Lz=1.0, precision=6):
    """write_vtk.cu:4-35 (x fastest in the file, `precision` significant digits)."""
    psi = np.ascontiguousarray(psi, dtype=np.float64)
    _check(_lib.load().xpfc_write_vtk(path.encode(), _dp(psi), Mx, My, Mz, Lx, Ly, Lz, precision))


def read_density_field(path):
    """read_input.cu:161-241: values in [Mx][My][Mz] order, with dims and L."""
    L = _lib.load()
    dims = (C.c_int * 3)()
    box = (C.c_double * 3)()
    _check(L.xpfc_read_vtk(path.encode(), None, 0, dims, box))
    n = dims[0] * dims[1] * dims[2]
    out = np.empty(n)
    _check(L.xpfc_read_vtk(path.encode(), _dp(out), n, dims, box))
    return out, tuple(dims), tuple(box)


class Xpfc:
    """One solve on one GPU (an xpfc_ctx)."""

    def __init__(self, params, stream=None):
        self._L = _lib.load()
        if stream is not None:
            params.stream = stream
        h = C.c_void_p()
        _check(self._L.xpfc_create(C.byref(params), C.byref(h)))
        self._h = h
        p = XpfcParams()
        self._L.xpfc_get_params(h, C.byref(p))
        self.params = p
        self.shape = (p.Mx, p.My, p.Mz)
        self.ncells = p.Mx * p.My * p.Mz

    def close(self):
        if getattr(self, "_h", None):
            self._L.xpfc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _c(self, rc):
        return _check(rc, self._h)

    # ---- lifecycle -------------------------------------------------------
    def initialize(self, psi=None):
        """initialize.cu:6-238 + main.cu:226 (pins the mean to psi0)."""
        if psi is None:
            self._c(self._L.xpfc_initialize(self._h, None))
        else:
            a = np.ascontiguousarray(psi, dtype=np.float64).reshape(-1)
            if a.size != self.ncells:
                raise ValueError("field has %d values, grid has %d" % (a.size, self.ncells))
            self._c(self._L.xpfc_initialize(self._h, _dp(a)))

    @property
    def stream(self):
        return self._L.xpfc_get_stream(self._h)

    @property
    def iteration(self):
        return self._L.xpfc_iteration(self._h)

    @property
    def launch_count(self):
        return self._L.xpfc_launch_count(self._h)

    # ---- fused path --------------------------------------------------------
    def step(self, nsteps, cap=None):
        """Advance nsteps iterations; returns the diagnostics records."""
        ts = self.params.t_sample
        if cap is None:
            cap = int(nsteps // ts + 4) if ts > 0 else 4
        recs = (XpfcDiag * cap)()
        cnt = C.c_int(0)
        self._c(self._L.xpfc_step(self._h, nsteps, recs, cap, C.byref(cnt)))
        return [dict(iteration=r.iteration, F=r.F if r.has & 1 else None, mean=r.mean if r.has & 1 else None,
                     rms=r.rms if r.has & 2 else None) for r in recs[:cnt.value]]

    def step_async(self, nsteps):
        """Enqueue nsteps iterations without waiting (periodic diagnostics only)."""
        self._c(self._L.xpfc_step_async(self._h, nsteps))

    def collect(self, cap=64):
        recs = (XpfcDiag * cap)()
        cnt = C.c_int(0)
        self._c(self._L.xpfc_collect(self._h, recs, cap, C.byref(cnt)))
        return [dict(iteration=r.iteration, F=r.F if r.has & 1 else None, mean=r.mean if r.has & 1 else None,
                     rms=r.rms if r.has & 2 else None) for r in recs[:cnt.value]]

    def set_profiling(self, enable):
        self._c(self._L.xpfc_set_profiling(self._h, 1 if enable else 0))

    def profile(self, npass=5):
        """{pass: (total ms, launches)} since profiling was enabled."""
        out = {}
        for ps in range(npass):
            ms = C.c_double()
            n = C.c_longlong()
            self._c(self._L.xpfc_get_profile(self._h, ps, C.byref(ms), C.byref(n)))
            out[ps] = (ms.value, n.value)
        return out

    def copy2cpu(self):
        """copy_to_cpu.cu:3-18: the current real field, [Mx][My][Mz]."""
        out = np.empty(self.ncells)
        self._c(self._L.xpfc_get_field(self._h, _dp(out)))
        return out.reshape(self.shape)

    get_field = copy2cpu

    # ---- staged path: the reference's per-stage wrappers ---------------------
    def pass_bytes(self, npass):
        """Algorithmic HBM bytes of one launch of a step pass (xpfc_pass_bytes)."""
        return self._L.xpfc_pass_bytes(self._h, npass)

    def copy2cpu_async(self):
        """Starts reading the current field back (copy_to_cpu.cu:3-18) on the
        context's copy stream; steps enqueued afterwards overlap the copy.
        copy2cpu_wait() returns (field, iteration)."""
        self._c(self._L.xpfc_get_field_async(self._h))

    def copy2cpu_wait(self):
        out = np.empty(self.ncells)
        it = C.c_longlong()
        self._c(self._L.xpfc_get_field_wait(self._h, _dp(out), C.byref(it)))
        return out.reshape(self.shape), it.value

    def save_state(self, path):
        """Checkpoint of the fused state at full precision (xpfc_save_state)."""
        self._c(self._L.xpfc_save_state(self._h, str(path).encode()))

    def load_state(self, path):
        """Resume from a checkpoint of the same grid and precision."""
        self._c(self._L.xpfc_load_state(self._h, str(path).encode()))

    def upload(self, buf, host):
        a = np.ascontiguousarray(host, dtype=np.float64).reshape(-1)
        self._c(self._L.xpfc_upload(self._h, buf, _dp(a)))

    def download(self, buf):
        out = np.empty(self.ncells)
        self._c(self._L.xpfc_download(self._h, buf, _dp(out)))
        return out

    def download_spectrum(self, buf):
        """Unpacked half spectrum [n2][n1][n0/2+1] (complex) of a packed buffer."""
        p = self.params
        if p.Mz > 1:
            n0, n1, n2 = p.Mz, p.My, p.Mx
        else:
            n0, n1, n2 = p.My, p.Mx, 1
        out = np.empty(2 * n2 * n1 * (n0 // 2 + 1))
        self._c(self._L.xpfc_download_spectrum(self._h, buf, _dp(out)))
        return out.view(np.complex128).reshape(n2, n1, n0 // 2 + 1)

    def cufftXtMemcpy(self, dst, src):
        self._c(self._L.xpfc_copy(self._h, src, dst))

    def cufftXtExecDescriptor(self, buf, direction):
        self._c(self._L.xpfc_fft(self._h, buf, direction))

    def power_function_wrapper(self, src, dst, p):
        self._c(self._L.xpfc_power_functions(self._h, src, dst, p))

    def scaling_step_wrapper(self, buf):
        self._c(self._L.xpfc_scaling_step(self._h, buf))

    def copy_matrix_wrapper(self, src, dst):
        self._c(self._L.xpfc_copy_matrix(self._h, src, dst))

    def convolution_wrapper(self, psi_k, out):
        self._c(self._L.xpfc_convolve_fields(self._h, psi_k, out))

    def euler_step_wrapper(self, n, psi_kp1, psi_k, psi2_k, psi3_k):
        self._c(self._L.xpfc_euler_step(self._h, n, psi_kp1, psi_k, psi2_k, psi3_k))

    def FE_calc_wrapper(self, n, psi, psi2, psi3, psi4, convl):
        F = C.c_double()
        self._c(self._L.xpfc_FE_calc(self._h, n, psi, psi2, psi3, psi4, convl, C.byref(F)))
        return F.value

    def SSE_calc_wrapper(self, n, psi_kp1, psi_k, psi2_k, psi3_k):
        r = C.c_double()
        self._c(self._L.xpfc_sse_calculation(self._h, n, psi_kp1, psi_k, psi2_k, psi3_k, C.byref(r)))
        return r.value

    def mean(self, buf=_lib.BUF_PSI):
        m = C.c_double()
        self._c(self._L.xpfc_Avg_calc(self._h, buf, C.byref(m)))
        return m.value


def _records(recs, cnt):
    return [dict(iteration=r.iteration, F=r.F if r.has & 1 else None, mean=r.mean if r.has & 1 else None,
                 rms=r.rms if r.has & 2 else None) for r in recs[:cnt]]


class Batch:
    """n independent solves advanced together (an xpfc_batch): instances that
    share grid, box and scheme constants form one group whose passes launch
    once over all of its fields; groups run concurrently."""

    def __init__(self, params_list):
        self._L = _lib.load()
        n = len(params_list)
        arr = (XpfcParams * n)(*params_list)
        h = C.c_void_p()
        rc = self._L.xpfc_batch_create(arr, n, C.byref(h))
        if rc != _lib.OK:
            msg = self._L.xpfc_batch_last_error(None)
            raise XpfcError(rc, msg.decode() if msg else "")
        self._h = h
        self.params = list(params_list)
        self.n = n

    def _c(self, rc):
        if rc != _lib.OK:
            msg = self._L.xpfc_batch_last_error(self._h)
            raise XpfcError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if getattr(self, "_h", None):
            self._L.xpfc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def groups(self):
        return self._L.xpfc_batch_groups(self._h)

    def group_of(self, i):
        return self._L.xpfc_batch_group_of(self._h, i)

    def initialize(self, fields=None):
        """fields: None or a list of n host fields (None entries: the
        instance's own generator); each mean is pinned to its psi0."""
        if fields is None:
            self._c(self._L.xpfc_batch_initialize(self._h, None))
            return
        keep = []
        ptrs = (C.POINTER(C.c_double) * self.n)()
        for i, f in enumerate(fields):
            if f is None:
                continue
            p = self.params[i]
            a = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
            if a.size != p.Mx * p.My * p.Mz:
                raise ValueError("field %d has %d values, grid has %d" % (i, a.size, p.Mx * p.My * p.Mz))
            keep.append(a)
            ptrs[i] = _dp(a)
        self._c(self._L.xpfc_batch_initialize(self._h, ptrs))

    def step(self, nsteps):
        self._c(self._L.xpfc_batch_step(self._h, nsteps))

    def step_async(self, nsteps):
        self._c(self._L.xpfc_batch_step_async(self._h, nsteps))

    def collect(self, i, cap=64):
        """Diagnostics of instance i from the last step call."""
        recs = (XpfcDiag * cap)()
        cnt = C.c_int(0)
        self._c(self._L.xpfc_batch_collect(self._h, i, recs, cap, C.byref(cnt)))
        return _records(recs, cnt.value)

    def get_field(self, i):
        p = self.params[i]
        out = np.empty(p.Mx * p.My * p.Mz)
        self._c(self._L.xpfc_batch_get_field(self._h, i, _dp(out)))
        return out.reshape(p.Mx, p.My, p.Mz)


class Server:
    """Solve requests on one GPU (an xpfc_server): admission under a device
    memory budget, up to max_running solves interleaved on their own streams;
    merge_max > 1 admits queued requests of the same grid and compatible
    params (step counts within 25 %) together as merged groups of up to
    merge_max solves that share every launch."""

    def __init__(self, hbm_budget_bytes=0, max_running=16, chunk_steps=16, device=0, merge_max=0):
        self._L = _lib.load()
        cfg = _lib.XpfcServerConfig(hbm_budget_bytes, max_running, chunk_steps, device, merge_max)
        h = C.c_void_p()
        rc = self._L.xpfc_server_create(C.byref(cfg), C.byref(h))
        if rc != _lib.OK:
            msg = self._L.xpfc_server_last_error(None)
            raise XpfcError(rc, msg.decode() if msg else "")
        self._h = h

    def _c(self, rc):
        if rc != _lib.OK:
            msg = self._L.xpfc_server_last_error(self._h)
            raise XpfcError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if getattr(self, "_h", None):
            self._L.xpfc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, params, nsteps, field=None, keep_field=False):
        """Queue a solve of nsteps iterations; returns its request id."""
        rid = C.c_longlong()
        if field is None:
            self._c(self._L.xpfc_server_submit(self._h, C.byref(params), None, nsteps, int(keep_field),
                                               C.byref(rid)))
        else:
            a = np.ascontiguousarray(field, dtype=np.float64).reshape(-1)
            if a.size != params.Mx * params.My * params.Mz:
                raise ValueError("field size does not match the grid")
            self._c(self._L.xpfc_server_submit(self._h, C.byref(params), _dp(a), nsteps, int(keep_field),
                                               C.byref(rid)))
        return rid.value

    def wait(self, rid, timeout=-1.0):
        self._c(self._L.xpfc_server_wait(self._h, rid, timeout))

    def info(self, rid):
        i = _lib.XpfcRequestInfo()
        self._c(self._L.xpfc_server_info(self._h, rid, C.byref(i)))
        return {"id": i.id, "state": i.state, "status": i.status, "t_submit": i.t_submit, "t_admit": i.t_admit,
                "t_done": i.t_done, "device_bytes": i.device_bytes}

    def result(self, rid, shape=None, cap=256):
        """(field or None, diagnostics) of a finished request; shape = the
        request's (Mx, My, Mz) when its field was kept."""
        recs = (XpfcDiag * cap)()
        cnt = C.c_int(0)
        out = None
        if shape is not None:
            out = np.empty(shape[0] * shape[1] * shape[2])
            self._c(self._L.xpfc_server_result(self._h, rid, _dp(out), recs, cap, C.byref(cnt)))
            out = out.reshape(shape)
        else:
            self._c(self._L.xpfc_server_result(self._h, rid, None, recs, cap, C.byref(cnt)))
        return out, _records(recs, cnt.value)

    def release(self, rid):
        self._c(self._L.xpfc_server_release(self._h, rid))

    def stats(self):
        st = _lib.XpfcServerStats()
        self._c(self._L.xpfc_server_stats_get(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}


def run_reference_loop(x, nsteps, t_sample):
    """main.cu:232-450 through the staged wrappers (FP64, reference order).

    x must be initialized.  Returns (F dict iteration -> value, RMS dict).
    """
    B = _lib
    F, R = {}, {}
    x.cufftXtMemcpy(B.BUF_PSI_NP1_R, B.BUF_PSI)
    x.power_function_wrapper(B.BUF_PSI, B.BUF_PSI2, 2)
    x.power_function_wrapper(B.BUF_PSI, B.BUF_PSI3, 3)
    x.power_function_wrapper(B.BUF_PSI, B.BUF_PSI4, 4)
    x.cufftXtMemcpy(B.BUF_PSI_K, B.BUF_PSI)
    x.cufftXtExecDescriptor(B.BUF_PSI_K, B.FORWARD)

    def free_energy(n):
        x.convolution_wrapper(B.BUF_PSI_K, B.BUF_CONVL)
        x.cufftXtExecDescriptor(B.BUF_CONVL, B.INVERSE)
        x.scaling_step_wrapper(B.BUF_CONVL)
        x.power_function_wrapper(B.BUF_PSI_NP1_R, B.BUF_PSI4, 4)
        return x.FE_calc_wrapper(n, B.BUF_PSI_NP1_R, B.BUF_PSI2, B.BUF_PSI3, B.BUF_PSI4, B.BUF_CONVL)

    F[0] = free_energy(0)
    n = 0
    for n in range(nsteps):
        x.cufftXtExecDescriptor(B.BUF_PSI2, B.FORWARD)
        x.cufftXtExecDescriptor(B.BUF_PSI3, B.FORWARD)
        x.euler_step_wrapper(n, B.BUF_PSI_NP1, B.BUF_PSI_K, B.BUF_PSI2, B.BUF_PSI3)
        if t_sample > 0 and n % t_sample == 0:
            R[n] = x.SSE_calc_wrapper(n, B.BUF_PSI_NP1, B.BUF_PSI_K, B.BUF_PSI2, B.BUF_PSI3)
        x.cufftXtExecDescriptor(B.BUF_PSI_NP1, B.INVERSE)
        x.scaling_step_wrapper(B.BUF_PSI_NP1)
        x.cufftXtMemcpy(B.BUF_PSI_NP1_R, B.BUF_PSI_NP1)
        x.copy_matrix_wrapper(B.BUF_PSI_NP1_R, B.BUF_PSI)
        x.power_function_wrapper(B.BUF_PSI, B.BUF_PSI2, 2)
        x.power_function_wrapper(B.BUF_PSI, B.BUF_PSI3, 3)
        x.cufftXtMemcpy(B.BUF_PSI_K, B.BUF_PSI)
        x.cufftXtExecDescriptor(B.BUF_PSI_K, B.FORWARD)
        if t_sample > 0 and (n + 1) % t_sample == 0 and n + 1 < nsteps:
            F[n + 1] = free_energy(n + 1)
    F[nsteps] = free_energy(nsteps)
    return F, R
