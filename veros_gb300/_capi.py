"""ctypes binding of ``libveros_gb300.so`` (declarations in ``include/veros_gb300.h``).

The library is loaded once per process. There is no fallback: if the shared
object is missing or does not load, every entry point raises.
"""

import ctypes
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libveros_gb300.so")

VG_OK = 0
VG_ERR_SHAPE = 1
VG_ERR_STRIDE = 2
VG_ERR_ARG = 3
VG_ERR_LAUNCH = 4
VG_ERR_TIMEOUT = 5
VG_ERR_UNSUPPORTED = 6
VG_ERR_SCRATCH = 7

MASK_T, MASK_U, MASK_V, MASK_W = 1, 2, 4, 8

c_double_p = ctypes.POINTER(ctypes.c_double)


class VgDomain(ctypes.Structure):
    _fields_ = [("X", ctypes.c_int), ("Y", ctypes.c_int), ("Z", ctypes.c_int),
                ("pitch", ctypes.c_longlong), ("plane", ctypes.c_longlong)]


class VgGrid(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("dxt", "dxu", "dyt", "dyu", "cost", "cosu", "dzt", "dzw", "zt")]


class VgIsoSettings(ctypes.Structure):
    _fields_ = [("iso_slopec", ctypes.c_double), ("iso_dslope", ctypes.c_double),
                ("K_iso_steep", ctypes.c_double), ("dt_tracer", ctypes.c_double),
                ("grav", ctypes.c_double), ("rho_0", ctypes.c_double),
                ("eq_of_state_type", ctypes.c_int), ("enable_conserve_energy", ctypes.c_int)]


class VgTensorFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")] + [
        ("ai_stride_p", ctypes.c_longlong), ("ai_stride_r", ctypes.c_longlong)]


class VgTensorFieldsF32(ctypes.Structure):
    _fields_ = VgTensorFields._fields_


class VgTracerArgsF32(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("tr_tau", "tr_taup1", "dtracer_iso", "int_drhodX_tau", "P_diss")]


class VgTracerArgs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("tr_tau", "tr_taup1", "dtracer_iso", "int_drhodX_tau", "P_diss")]


class VgStepFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("temp_tau", "temp_taup1", "salt_tau", "salt_taup1", "K_iso",
                                                "mask_bits", "kbot")] + [("ten", VgTensorFields)] + [
        (n, ctypes.c_void_p) for n in ("dtemp_iso", "dsalt_iso", "int_drhodT_tau", "int_drhodS_tau", "P_diss_iso",
                                       "column_order", "pre_shares", "flux_shares")] + [
        ("pre_shares_n", ctypes.c_int), ("flux_shares_n", ctypes.c_int)]


class VgStepFieldsF32(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("temp_tau", "temp_taup1", "salt_tau", "salt_taup1", "K_iso",
                                                "mask_bits", "kbot")] + [("ten", VgTensorFieldsF32)] + [
        (n, ctypes.c_void_p) for n in ("dtemp_iso", "dsalt_iso", "int_drhodT_tau", "int_drhodS_tau", "P_diss_iso",
                                       "column_order", "pre_shares", "flux_shares")] + [
        ("pre_shares_n", ctypes.c_int), ("flux_shares_n", ctypes.c_int)]


class VgEnsembleTuning(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("pre_rows", "pre_kchunk", "flux_rows", "flux_kchunk", "solve_threads")]


class VgEnsembleMember(ctypes.Structure):
    _fields_ = [("dom", VgDomain), ("grid", VgGrid), ("set", VgIsoSettings), ("phase", VgStepFields * 3)]


class VgEnsembleMemberF32(ctypes.Structure):
    _fields_ = [("dom", VgDomain), ("grid", VgGrid), ("set", VgIsoSettings), ("phase", VgStepFieldsF32 * 3)]


class VgAdjointFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("temp", "salt", "temp_new", "salt_new", "K_iso", "mask_bits", "kbot",
                                                "gtemp_new", "gsalt_new", "gtemp", "gsalt", "gK_iso",
                                                "column_order")]


# name -> (restype, argtypes); the exported C ABI
SIGNATURES = {
    "vg_last_error": (ctypes.c_char_p, []),
    "vg_version": (ctypes.c_char_p, []),
    "vg_pack_masks": (ctypes.c_int, [ctypes.POINTER(VgDomain)] + [ctypes.c_void_p] * 5 + [ctypes.c_void_p]),
    "vg_layout_to_canonical_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                                  ctypes.c_void_p]),
    "vg_layout_from_canonical_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.c_int,
                                                    ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                                    ctypes.c_void_p]),
    "vg_isoneutral_pre_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                             ctypes.POINTER(VgIsoSettings), ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(VgTensorFields),
                                             ctypes.c_void_p]),
    "vg_isoneutral_pre_f32split": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                  ctypes.POINTER(VgIsoSettings), ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(VgTensorFieldsF32),
                                                  ctypes.c_void_p]),
    "vg_isoneutral_diffusion_f32split": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                        ctypes.POINTER(VgIsoSettings),
                                                        ctypes.POINTER(VgTensorFieldsF32), ctypes.c_void_p,
                                                        ctypes.c_void_p, ctypes.c_void_p,
                                                        ctypes.POINTER(VgTracerArgsF32), ctypes.c_int,
                                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "vg_isoneutral_diffusion_pair_f32split": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                             ctypes.POINTER(VgIsoSettings),
                                                             ctypes.POINTER(VgTensorFieldsF32), ctypes.c_void_p,
                                                             ctypes.c_void_p, ctypes.c_void_p,
                                                             ctypes.POINTER(VgTracerArgsF32),
                                                             ctypes.POINTER(VgTracerArgsF32), ctypes.c_void_p,
                                                             ctypes.c_size_t, ctypes.c_void_p]),
    "vg_isoneutral_step_f32split": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                   ctypes.POINTER(VgIsoSettings), ctypes.POINTER(VgStepFieldsF32),
                                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "vg_isoneutral_step_prepare_f32split": (ctypes.c_int, [ctypes.POINTER(VgDomain),
                                                           ctypes.POINTER(VgStepFieldsF32), ctypes.c_void_p]),
    "vg_isoneutral_diffusion_scratch_bytes": (ctypes.c_size_t, [ctypes.POINTER(VgDomain)]),
    "vg_isoneutral_diffusion_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                   ctypes.POINTER(VgIsoSettings), ctypes.POINTER(VgTensorFields),
                                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.POINTER(VgTracerArgs), ctypes.c_int, ctypes.c_void_p,
                                                   ctypes.c_size_t, ctypes.c_void_p]),
    "vg_isoneutral_diffusion_noalloc_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                           ctypes.POINTER(VgIsoSettings),
                                                           ctypes.POINTER(VgTensorFields), ctypes.c_void_p,
                                                           ctypes.c_void_p, ctypes.c_void_p,
                                                           ctypes.POINTER(VgTracerArgs), ctypes.c_int,
                                                           ctypes.c_void_p]),
    "vg_isoneutral_diffusion_noalloc_capacity": (ctypes.c_size_t, []),
    "vg_isoneutral_diffusion_noalloc_reset": (None, []),
    "vg_isoneutral_diffusion_pair_scratch_bytes": (ctypes.c_size_t, [ctypes.POINTER(VgDomain)]),
    "vg_isoneutral_diffusion_pair_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                        ctypes.POINTER(VgIsoSettings), ctypes.POINTER(VgTensorFields),
                                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                        ctypes.POINTER(VgTracerArgs), ctypes.POINTER(VgTracerArgs),
                                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "vg_isoneutral_diffusion_pair_ordered_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                                ctypes.POINTER(VgIsoSettings),
                                                                ctypes.POINTER(VgTensorFields), ctypes.c_void_p,
                                                                ctypes.c_void_p, ctypes.c_void_p,
                                                                ctypes.POINTER(VgTracerArgs),
                                                                ctypes.POINTER(VgTracerArgs), ctypes.c_void_p,
                                                                ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "vg_isoneutral_diffusion_pair_ordered_f32split": (ctypes.c_int, [ctypes.POINTER(VgDomain),
                                                                     ctypes.POINTER(VgGrid),
                                                                     ctypes.POINTER(VgIsoSettings),
                                                                     ctypes.POINTER(VgTensorFieldsF32),
                                                                     ctypes.c_void_p, ctypes.c_void_p,
                                                                     ctypes.c_void_p,
                                                                     ctypes.POINTER(VgTracerArgsF32),
                                                                     ctypes.POINTER(VgTracerArgsF32),
                                                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                                     ctypes.c_void_p]),
    "vg_isoneutral_step_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                              ctypes.POINTER(VgIsoSettings), ctypes.POINTER(VgStepFields),
                                              ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "vg_isoneutral_step_prepare_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgStepFields),
                                                      ctypes.c_void_p]),
    "vg_isoneutral_step_shares_size": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.c_int,
                                                      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                      ctypes.POINTER(ctypes.c_size_t)]),
    "vg_isoneutral_step_shares": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                 ctypes.c_void_p]),
    "vg_isoneutral_step_stage_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                    ctypes.POINTER(VgIsoSettings), ctypes.POINTER(VgStepFields),
                                                    ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                                    ctypes.c_void_p]),
    "vg_isoneutral_step_stage_f32split": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                         ctypes.POINTER(VgIsoSettings),
                                                         ctypes.POINTER(VgStepFieldsF32), ctypes.c_void_p,
                                                         ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]),
    "vg_vertmix_tempsalt_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                               ctypes.POINTER(VgIsoSettings)] + [ctypes.c_void_p] * 8 +
                                [ctypes.c_int, ctypes.c_void_p]),
    "vg_enforce_boundaries_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.c_void_p, ctypes.c_int,
                                                 ctypes.c_void_p]),
    "vg_isoneutral_streamfunction_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.c_void_p, ctypes.c_void_p,
                                                        ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong,
                                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "vg_isoneutral_step_adjoint_scratch_bytes": (ctypes.c_size_t, [ctypes.POINTER(VgDomain)]),
    "vg_isoneutral_step_adjoint_f64": (ctypes.c_int, [ctypes.POINTER(VgDomain), ctypes.POINTER(VgGrid),
                                                      ctypes.POINTER(VgIsoSettings), ctypes.POINTER(VgAdjointFields),
                                                      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "vg_ensemble_create_f64": (ctypes.c_int, [ctypes.POINTER(VgEnsembleMember), ctypes.c_int,
                                              ctypes.POINTER(VgEnsembleTuning), ctypes.POINTER(ctypes.c_void_p)]),
    "vg_ensemble_create_f32split": (ctypes.c_int, [ctypes.POINTER(VgEnsembleMemberF32), ctypes.c_int,
                                                   ctypes.POINTER(VgEnsembleTuning),
                                                   ctypes.POINTER(ctypes.c_void_p)]),
    "vg_ensemble_tune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(VgEnsembleTuning)]),
    "vg_ensemble_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "vg_ensemble_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "vg_solve_implicit_f64": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                                             ctypes.c_longlong, ctypes.c_longlong] + [ctypes.c_void_p] * 11),
    "vg_solve_implicit_f32": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                                             ctypes.c_longlong, ctypes.c_longlong] + [ctypes.c_void_p] * 11),
    "vg_tdma_cuda_double": (None, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                                   ctypes.c_size_t]),
    "vg_tdma_cuda_float": (None, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                                  ctypes.c_size_t]),
}

_lock = threading.Lock()
_lib = None


def load(path=None):
    """Load the library (once) and bind every exported symbol."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError(
                f"veros_gb300 CUDA library not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` or `python -m veros_gb300._build`")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error():
    return load().vg_last_error().decode(errors="replace")


def check(status, what):
    """Raise the Python exception matching a C-ABI status."""
    if status == VG_OK:
        return
    msg = f"{what}: {last_error()}"
    if status in (VG_ERR_SHAPE, VG_ERR_STRIDE, VG_ERR_ARG, VG_ERR_SCRATCH):
        raise ValueError(msg)
    if status == VG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)
