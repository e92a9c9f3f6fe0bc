"""Drop-in for ``veros.core.thermodynamics.vertmix_tempsalt``
(veros/core/thermodynamics.py:248-300), the implicit vertical mixing that
follows the isoneutral step: returns ``KernelOutput(dtemp_vmix, temp,
dsalt_vmix, salt)`` like the reference kernel. ``state`` is a
:class:`DeviceState` (in place on the GPU) or a NumPy ``VerosState``.

The reference ends with ``enforce_boundaries`` of the new temp and salt
levels (thermodynamics.py:292-298): on one process, with
``settings.enable_cyclic_x``, the periodic copy of the x halo columns
(veros/core/utilities.py:7-16), which the CUDA call performs; across several
processes it is the halo exchange of the domain decomposition
(utilities.py:18-20), which this single-GPU library does not do, so a
multi-process run raises ``NotImplementedError`` instead of returning stale
halos.
"""

import torch

from . import _capi
from .state import DeviceState, KernelOutput, host_mirror, mirror_download, mirror_written, require_single_process


def run_vertmix(dev):
    v = dev.variables
    dev.check_layout(("kappaH", "dtemp_vmix", "dsalt_vmix"))
    for n in ("forc_temp_surface", "forc_salt_surface", "kbot"):
        t = getattr(v, n)
        if t.stride(0) != 1 or t.stride(1) != dev.pitch:
            raise ValueError(f"{n} is not in the canonical layout")
    if v.temp.dtype != torch.float64:
        raise ValueError("vertmix_tempsalt runs on float64 tracers")
    lib = _capi.load()
    st = lib.vg_vertmix_tempsalt_f64(dev.domain(), dev.grid(), dev.settings.to_struct(), v.kappaH.data_ptr(),
                                     v.kbot.data_ptr(), v.temp[..., v.taup1].data_ptr(),
                                     v.salt[..., v.taup1].data_ptr(), v.forc_temp_surface.data_ptr(),
                                     v.forc_salt_surface.data_ptr(), v.dtemp_vmix.data_ptr(), v.dsalt_vmix.data_ptr(),
                                     int(bool(dev.settings.get("enable_cyclic_x", False))),
                                     torch.cuda.current_stream(dev.device).cuda_stream)
    _capi.check(st, "vertmix_tempsalt")


def vertmix_tempsalt(state):
    require_single_process("vertmix_tempsalt (its closing halo exchange)")
    names = ("dtemp_vmix", "temp", "dsalt_vmix", "salt")
    if isinstance(state, DeviceState):
        run_vertmix(state)
        v = state.variables
        return KernelOutput(**{n: getattr(v, n) for n in names})
    fields = ("temp", "salt", "kappaH", "kbot", "forc_temp_surface", "forc_salt_surface", "dxt", "dxu", "dyt", "dyu",
              "cost", "cosu", "dzt", "dzw", "zt", "maskT", "maskU", "maskV", "maskW")
    dev = host_mirror(state, fields)
    mirror_written(dev, names)
    run_vertmix(dev)
    return KernelOutput(**{n: mirror_download(dev, n) for n in names})
