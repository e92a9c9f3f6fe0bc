"""Drop-ins for ``veros.core.isoneutral`` on the GB300 CUDA library.

Same call signatures as the reference:

* ``isoneutral_diffusion_pre(state) -> KernelOutput(Ai_ez, Ai_nz, Ai_bx, Ai_by, K_11, K_22, K_33)``
  (veros/core/isoneutral/isoneutral.py:18-229)
* ``isoneutral_diffusion(state, tr, istemp) -> None``
  (veros/core/isoneutral/diffusion.py:286-295)
* ``isoneutral_skew_diffusion(state, tr, istemp) -> None``
  (veros/core/isoneutral/diffusion.py:298-307)

``state`` is either a :class:`veros_gb300.state.DeviceState` (fields stay on
the GPU, all work is enqueued on torch's current stream, nothing synchronises)
or a NumPy-backend ``VerosState``, whose fields are mirrored on the device,
processed and written back (the reference's ``vs.update`` contract: pre
returns the new arrays, the diffusion routines mutate ``state.variables``).
Arrays returned to a NumPy state are read-only, as the NumPy backend's own
are, and a field is uploaded only when the state holds another array than the
one last transferred for it (``state.host_mirror``).
"""

import torch

from . import _capi
from .state import DeviceState, KernelOutput, FIELDS_MASK, host_mirror, mirror_download, mirror_written

PRE_OUT = ("Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "K_11", "K_22", "K_33")


def _stream(dev):
    return torch.cuda.current_stream(dev.device).cuda_stream


def _level(t, n):
    """Pointer of time level ``n`` of a (X, Y, Z, 3) tensor."""
    return t[..., n].data_ptr()


def run_pre(dev):
    """Enqueue the slope/tensor kernel on a DeviceState (in place)."""
    v = dev.variables
    dev.check_layout(("temp", "salt", "K_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by"))
    lib = _capi.load()
    fn = lib.vg_isoneutral_pre_f64 if dev.precision == "f64" else lib.vg_isoneutral_pre_f32split
    st = fn(dev.domain(), dev.grid(), dev.settings.to_struct(), _level(v.temp, v.tau), _level(v.salt, v.tau),
            v.K_iso.data_ptr(), dev.mask_bits().data_ptr(), dev.tensor_fields(), _stream(dev))
    _capi.check(st, "isoneutral_diffusion_pre")


def diffusion_scratch(dev):
    nbytes = _capi.load().vg_isoneutral_diffusion_scratch_bytes(dev.domain())
    return torch.empty(nbytes // 8, dtype=torch.float64, device=dev.device)


def run_diffusion(dev, istemp, skew=False, scratch=None):
    """Enqueue diffusion of temp (istemp) or salt on a DeviceState (in place)."""
    v = dev.variables
    tr = v.temp if istemp else v.salt
    dtr = v.dtemp_iso if istemp else v.dsalt_iso
    energy = bool(dev.settings.enable_conserve_energy)
    kfield = v.K_gm if skew else v.K_iso
    names = ["temp" if istemp else "salt", "dtemp_iso" if istemp else "dsalt_iso", "K_11", "K_22", "K_33",
             "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "K_gm" if skew else "K_iso"]
    if energy:
        names += ["int_drhodT" if istemp else "int_drhodS", "P_diss_skew" if skew else "P_diss_iso"]
    dev.check_layout(names)
    targs = _capi.VgTracerArgs if dev.precision == "f64" else _capi.VgTracerArgsF32
    if energy:
        idr = (v.int_drhodT if istemp else v.int_drhodS)
        P = v.P_diss_skew if skew else v.P_diss_iso
        tra = targs(_level(tr, v.tau), _level(tr, v.taup1), dtr.data_ptr(), _level(idr, v.tau), P.data_ptr())
    else:
        tra = targs(_level(tr, v.tau), _level(tr, v.taup1), dtr.data_ptr(), None, None)
    if scratch is None:
        scratch = diffusion_scratch(dev)
    kb = v.kbot
    if kb.stride(0) != 1 or kb.stride(1) != dev.pitch:
        raise ValueError("kbot is not in the canonical layout")
    lib = _capi.load()
    fn = lib.vg_isoneutral_diffusion_f64 if dev.precision == "f64" else lib.vg_isoneutral_diffusion_f32split
    st = fn(dev.domain(), dev.grid(), dev.settings.to_struct(), dev.tensor_fields(), kfield.data_ptr(),
            dev.mask_bits().data_ptr(), kb.data_ptr(), tra, 1 if skew else 0, scratch.data_ptr(),
            scratch.numel() * 8, _stream(dev))
    _capi.check(st, "isoneutral_skew_diffusion" if skew else "isoneutral_diffusion")


# ---------------------------------------------------------------------------
# reference-signature entry points


def _is_device_state(state):
    return isinstance(state, DeviceState)


def isoneutral_diffusion_pre(state):
    if _is_device_state(state):
        run_pre(state)
        v = state.variables
        return KernelOutput(**{n: getattr(v, n) for n in PRE_OUT})
    names = ("temp", "salt", "K_iso", "dxt", "dxu", "dyt", "dyu", "cost", "cosu", "dzt", "dzw", "zt",
             *FIELDS_MASK, *PRE_OUT)
    dev = host_mirror(state, names)
    mirror_written(dev, PRE_OUT)
    run_pre(dev)
    return KernelOutput(**{n: mirror_download(dev, n) for n in PRE_OUT})


def _diffusion_entry(state, tr, istemp, skew):
    name = "temp" if istemp else "salt"
    dname = "dtemp_iso" if istemp else "dsalt_iso"
    pname = "P_diss_skew" if skew else "P_diss_iso"
    if _is_device_state(state):
        v = state.variables
        target = getattr(v, name)
        if tr is not None and tr is not target:
            target.copy_(tr)  # the reference passes tr by value and writes back to temp/salt
        run_diffusion(state, istemp, skew=skew)
        return None
    energy = bool(state.settings.enable_conserve_energy)
    names = [name, dname, "K_gm" if skew else "K_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "kbot",
             "dxt", "dxu", "dyt", "dyu", "cost", "cosu", "dzt", "dzw", "zt", *FIELDS_MASK]
    if energy:
        names += ["int_drhodT" if istemp else "int_drhodS", pname]
    vs = state.variables
    if tr is not None and tr is not getattr(vs, name):
        names = [n for n in names if n != name]
    dev = host_mirror(state, names)
    if tr is not None and tr is not getattr(vs, name):
        dev.upload(name, tr)  # the reference diffuses the tr it is given (by value)
    written = [name, dname] + ([pname] if energy else [])
    mirror_written(dev, written)
    run_diffusion(dev, istemp, skew=skew)
    vs.update({n: mirror_download(dev, n) for n in written})
    return None


def isoneutral_diffusion(state, tr, istemp):
    """Isopycnal diffusion of ``tr`` (temp if ``istemp`` else salt); mutates the state."""
    return _diffusion_entry(state, tr, istemp, skew=False)


def isoneutral_skew_diffusion(state, tr, istemp):
    """Skew (GM) diffusion of ``tr``; mutates the state."""
    return _diffusion_entry(state, tr, istemp, skew=True)


def isoneutral_diag_streamfunction_kernel(state):
    """GM streamfunction diagnostics (veros/core/isoneutral/isoneutral.py:232-254):
    ``KernelOutput(B1_gm, B2_gm)``."""
    if not _is_device_state(state):
        dev = host_mirror(state, ("K_gm", "Ai_ez", "Ai_nz", "B1_gm", "B2_gm"))
        mirror_written(dev, ("B1_gm", "B2_gm"))
        _run_streamfunction(dev)
        return KernelOutput(B1_gm=mirror_download(dev, "B1_gm"), B2_gm=mirror_download(dev, "B2_gm"))
    _run_streamfunction(state)
    v = state.variables
    return KernelOutput(B1_gm=v.B1_gm, B2_gm=v.B2_gm)


def _run_streamfunction(dev):
    v = dev.variables
    dev.check_layout(("B1_gm", "B2_gm"))
    if v.K_gm.dtype != torch.float64 or v.Ai_ez.dtype != torch.float64:
        raise ValueError("the streamfunction diagnostics run on float64 fields")
    ai = v.Ai_ez
    lib = _capi.load()
    st = lib.vg_isoneutral_streamfunction_f64(dev.domain(), v.K_gm.data_ptr(), v.Ai_ez.data_ptr(), v.Ai_nz.data_ptr(),
                                              ai.stride(3), ai.stride(4), v.B1_gm.data_ptr(), v.B2_gm.data_ptr(),
                                              _stream(dev))
    _capi.check(st, "isoneutral_diag_streamfunction")


def isoneutral_diag_streamfunction(state):
    """Routine form (veros/core/isoneutral/isoneutral.py:257-269): runs only with
    neutral and skew diffusion enabled; mutates the state, returns None."""
    s = state.settings
    if not (getattr(s, "enable_neutral_diffusion", False) and getattr(s, "enable_skew_diffusion", False)):
        return None
    out = isoneutral_diag_streamfunction_kernel(state)
    state.variables.update(out)
    return None
