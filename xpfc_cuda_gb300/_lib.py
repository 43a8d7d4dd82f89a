"""ctypes binding of libxpfc.so (include/xpfc.h).

The library is built in-tree by xpfc_cuda_gb300/build.py.  Loading never
falls back to anything else: a missing or unloadable library raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("XPFC_LIB") or os.path.join(HERE, "_lib", "libxpfc.so")

MAX_PEAKS = 8

# xpfc_status
OK, EINVAL, ENOMEM, ECUDA, ENONFINITE, ETIMEDOUT, EIO, ESTATE = range(8)
STATUS_NAMES = {0: "XPFC_OK", 1: "XPFC_EINVAL", 2: "XPFC_ENOMEM", 3: "XPFC_ECUDA", 4: "XPFC_ENONFINITE",
                5: "XPFC_ETIMEDOUT", 6: "XPFC_EIO", 7: "XPFC_ESTATE"}
FP64, MIXED = 0, 1
ENVELOPE_SUM, ENVELOPE_MAX = 0, 1
FORWARD, INVERSE = -1, 1
IC_REFERENCE, IC_NOISE, IC_FCC_SEED = 0, 1, 2
(BUF_PSI, BUF_PSI_K, BUF_PSI_NP1, BUF_PSI_NP1_R, BUF_PSI2, BUF_PSI3, BUF_PSI4, BUF_CONVL, BUF_RES) = range(9)


class XpfcParams(C.Structure):
    _fields_ = [
        ("Mx", C.c_int), ("My", C.c_int), ("Mz", C.c_int),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("psi0", C.c_double), ("sigma", C.c_double), ("a", C.c_double), ("b", C.c_double),
        ("eps", C.c_double), ("Mo", C.c_double), ("dt", C.c_double),
        ("nsteps", C.c_longlong),
        ("t_sample", C.c_int),
        ("npeaks", C.c_int),
        ("pk_k", C.c_double * MAX_PEAKS), ("pk_alpha", C.c_double * MAX_PEAKS),
        ("pk_rho", C.c_double * MAX_PEAKS), ("pk_beta", C.c_double * MAX_PEAKS),
        ("envelope", C.c_int), ("precision", C.c_int), ("ref_compat", C.c_int),
        ("ff_factor", C.c_double),
        ("noise_amp", C.c_double), ("noise_seed", C.c_ulonglong),
        ("ic_kind", C.c_int), ("iconfig", C.c_int),
        ("A_10", C.c_double), ("A_11", C.c_double), ("A_tri", C.c_double),
        ("iseed", C.c_int), ("ishape", C.c_int),
        ("h", C.c_double), ("k", C.c_double), ("roa", C.c_double),
        ("ic_amp", C.c_double), ("ic_seed", C.c_ulonglong),
        ("ic_seed_amp", C.c_double), ("ic_seed_radius", C.c_double),
        ("vtk_path", C.c_char * 512),
        ("device", C.c_int),
        ("stream", C.c_void_p),
    ]


class XpfcDiag(C.Structure):
    _fields_ = [("iteration", C.c_longlong), ("F", C.c_double), ("mean", C.c_double), ("rms", C.c_double),
                ("has", C.c_int)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = range(4)


class XpfcServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_running", C.c_int), ("chunk_steps", C.c_int),
                ("device", C.c_int), ("merge_max", C.c_int)]


class XpfcRequestInfo(C.Structure):
    _fields_ = [("id", C.c_longlong), ("state", C.c_int), ("status", C.c_int), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("device_bytes", C.c_size_t)]


class XpfcServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("queued", C.c_longlong), ("running", C.c_longlong),
                ("done", C.c_longlong), ("failed", C.c_longlong), ("contexts_created", C.c_longlong),
                ("contexts_reused", C.c_longlong), ("bytes_in_use", C.c_size_t),
                ("peak_bytes_in_use", C.c_size_t), ("budget", C.c_size_t), ("merged_groups", C.c_longlong),
                ("merged_solves", C.c_longlong)]


# (name, restype, argtypes) for every entry point of include/xpfc.h
_dp = C.POINTER(C.c_double)
_ctx = C.c_void_p
SIGNATURES = [
    ("xpfc_default_params", C.c_int, [C.POINTER(XpfcParams)]),
    ("xpfc_read_input", C.c_int, [C.c_char_p, C.POINTER(XpfcParams)]),
    ("xpfc_create", C.c_int, [C.POINTER(XpfcParams), C.POINTER(C.c_void_p)]),
    ("xpfc_destroy", C.c_int, [_ctx]),
    ("xpfc_last_error", C.c_char_p, [_ctx]),
    ("xpfc_get_params", C.c_int, [_ctx, C.POINTER(XpfcParams)]),
    ("xpfc_get_stream", C.c_void_p, [_ctx]),
    ("xpfc_initialize", C.c_int, [_ctx, _dp]),
    ("xpfc_build_initial_field", C.c_int, [C.POINTER(XpfcParams), _dp]),
    ("xpfc_build_initial_field_device", C.c_int, [C.POINTER(XpfcParams), C.c_void_p, C.c_void_p]),
    ("xpfc_step", C.c_int, [_ctx, C.c_longlong, C.POINTER(XpfcDiag), C.c_int, C.POINTER(C.c_int)]),
    ("xpfc_step_async", C.c_int, [_ctx, C.c_longlong]),
    ("xpfc_collect", C.c_int, [_ctx, C.POINTER(XpfcDiag), C.c_int, C.POINTER(C.c_int)]),
    ("xpfc_set_profiling", C.c_int, [_ctx, C.c_int]),
    ("xpfc_get_profile", C.c_int, [_ctx, C.c_int, _dp, C.POINTER(C.c_longlong)]),
    ("xpfc_iteration", C.c_longlong, [_ctx]),
    ("xpfc_get_field", C.c_int, [_ctx, _dp]),
    ("xpfc_get_field_device_f32", C.c_int, [_ctx, C.c_void_p]),
    ("xpfc_get_field_async", C.c_int, [_ctx]),
    ("xpfc_get_field_wait", C.c_int, [_ctx, _dp, C.POINTER(C.c_longlong)]),
    ("xpfc_save_state", C.c_int, [_ctx, C.c_char_p]),
    ("xpfc_load_state", C.c_int, [_ctx, C.c_char_p]),
    ("xpfc_upload", C.c_int, [_ctx, C.c_int, _dp]),
    ("xpfc_download", C.c_int, [_ctx, C.c_int, _dp]),
    ("xpfc_download_spectrum", C.c_int, [_ctx, C.c_int, _dp]),
    ("xpfc_copy", C.c_int, [_ctx, C.c_int, C.c_int]),
    ("xpfc_fft", C.c_int, [_ctx, C.c_int, C.c_int]),
    ("xpfc_power_functions", C.c_int, [_ctx, C.c_int, C.c_int, C.c_int]),
    ("xpfc_scaling_step", C.c_int, [_ctx, C.c_int]),
    ("xpfc_copy_matrix", C.c_int, [_ctx, C.c_int, C.c_int]),
    ("xpfc_convolve_fields", C.c_int, [_ctx, C.c_int, C.c_int]),
    ("xpfc_euler_step", C.c_int, [_ctx, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("xpfc_FE_calc", C.c_int, [_ctx, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp]),
    ("xpfc_sse_calculation", C.c_int, [_ctx, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp]),
    ("xpfc_Avg_calc", C.c_int, [_ctx, C.c_int, _dp]),
    ("xpfc_write_vtk", C.c_int, [C.c_char_p, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                 C.c_int]),
    ("xpfc_read_vtk", C.c_int, [C.c_char_p, _dp, C.c_size_t, C.POINTER(C.c_int), _dp]),
    ("xpfc_batch_create", C.c_int, [C.POINTER(XpfcParams), C.c_int, C.POINTER(C.c_void_p)]),
    ("xpfc_batch_destroy", C.c_int, [C.c_void_p]),
    ("xpfc_batch_last_error", C.c_char_p, [C.c_void_p]),
    ("xpfc_batch_size", C.c_int, [C.c_void_p]),
    ("xpfc_batch_groups", C.c_int, [C.c_void_p]),
    ("xpfc_batch_group_of", C.c_int, [C.c_void_p, C.c_int]),
    ("xpfc_batch_initialize", C.c_int, [C.c_void_p, C.POINTER(_dp)]),
    ("xpfc_batch_step", C.c_int, [C.c_void_p, C.c_longlong]),
    ("xpfc_batch_step_async", C.c_int, [C.c_void_p, C.c_longlong]),
    ("xpfc_batch_collect", C.c_int, [C.c_void_p, C.c_int, C.POINTER(XpfcDiag), C.c_int, C.POINTER(C.c_int)]),
    ("xpfc_batch_get_field", C.c_int, [C.c_void_p, C.c_int, _dp]),
    ("xpfc_server_create", C.c_int, [C.POINTER(XpfcServerConfig), C.POINTER(C.c_void_p)]),
    ("xpfc_server_destroy", C.c_int, [C.c_void_p]),
    ("xpfc_server_last_error", C.c_char_p, [C.c_void_p]),
    ("xpfc_server_submit", C.c_int, [C.c_void_p, C.POINTER(XpfcParams), _dp, C.c_longlong, C.c_int,
                                     C.POINTER(C.c_longlong)]),
    ("xpfc_server_wait", C.c_int, [C.c_void_p, C.c_longlong, C.c_double]),
    ("xpfc_server_info", C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(XpfcRequestInfo)]),
    ("xpfc_server_result", C.c_int, [C.c_void_p, C.c_longlong, _dp, C.POINTER(XpfcDiag), C.c_int,
                                     C.POINTER(C.c_int)]),
    ("xpfc_server_release", C.c_int, [C.c_void_p, C.c_longlong]),
    ("xpfc_server_stats_get", C.c_int, [C.c_void_p, C.POINTER(XpfcServerStats)]),
    ("xpfc_FE_calc_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong,
                                        C.c_double, C.c_double, C.c_double, _dp, C.c_void_p]),
    ("xpfc_launch_count", C.c_longlong, [_ctx]),
    ("xpfc_pass_bytes", C.c_longlong, [_ctx, C.c_int]),
    ("xpfc_version", C.c_char_p, []),
]

_lib = None


def load():
    """Load libxpfc.so (building it first if absent); raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build
        build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libxpfc.so is missing: build it with xpfc_cuda_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
