"""The scratch-free diffusion entry point (vg_isoneutral_diffusion_noalloc_f64).

Callers that cannot allocate device memory (an XLA custom-call or FFI handler
that may only use the buffers it is handed, or a host model that fixes its
device memory at start-up) use this variant, which keeps the diffusion's flux
scratch in a static device array of the library. This test calls it through
the C ABI and checks it against the allocating entry point,
vg_isoneutral_diffusion_f64 with caller-provided scratch, over consecutive
calls that reuse the shared array. It lives in its own file, collected last,
and needs nothing from the other test files' state.
"""

import numpy as np
import pytest

from conftest import assert_field_close, p_diss_floor

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc_diffusion(dev, istemp):
    from veros_gb300 import _capi

    v = dev.variables
    tr = v.temp if istemp else v.salt
    dtr = v.dtemp_iso if istemp else v.dsalt_iso
    idr = v.int_drhodT if istemp else v.int_drhodS
    tra = _capi.VgTracerArgs(tr[..., v.tau].data_ptr(), tr[..., v.taup1].data_ptr(), dtr.data_ptr(),
                             idr[..., v.tau].data_ptr(), v.P_diss_iso.data_ptr())
    lib = _capi.load()
    st = lib.vg_isoneutral_diffusion_noalloc_f64(dev.domain(), dev.grid(), dev.settings.to_struct(),
                                                 dev.tensor_fields(), v.K_iso.data_ptr(), dev.mask_bits().data_ptr(),
                                                 v.kbot.data_ptr(), tra, 0,
                                                 torch.cuda.current_stream(dev.device).cuda_stream)
    _capi.check(st, "vg_isoneutral_diffusion_noalloc_f64")


def test_noalloc_diffusion_matches_allocating_entry():
    from veros_gb300 import _capi, synthetic
    from veros_gb300.isoneutral import run_diffusion, run_pre
    from veros_gb300.state import DeviceState

    lib = _capi.load()
    assert lib.vg_isoneutral_diffusion_noalloc_capacity() == 32 << 20

    # energy branch on, so the flux scratch is written and read back
    host = synthetic.make_state(40, 30, 15, seed=11, eq_of_state_type=3, k_iso_lognormal_sigma=0.3,
                                settings=dict(enable_conserve_energy=True))
    ref = DeviceState.from_host(host)
    new = DeviceState.from_host(host)
    assert lib.vg_isoneutral_diffusion_scratch_bytes(new.domain()) <= 32 << 20
    run_pre(ref)
    run_pre(new)
    torch.cuda.synchronize()
    dt = host.settings["dt_tracer"]

    # two rounds of temp then salt: four consecutive calls on the shared array
    for _ in range(2):
        for istemp in (True, False):
            run_diffusion(ref, istemp)
            _noalloc_diffusion(new, istemp)
            torch.cuda.synchronize()
            arrays = ref.to_host_dict(["temp", "salt", "int_drhodT", "int_drhodS", "K_33", "dzw"])
            floor = p_diss_floor(arrays, host.settings, ref.variables.tau)
            for name in ("temp", "salt", "dtemp_iso", "dsalt_iso", "P_diss_iso"):
                tracer = arrays["temp"] if name == "dtemp_iso" else arrays["salt"] if name == "dsalt_iso" else None
                assert_field_close(name, new.download(name), ref.download(name), tracer=tracer, dt=dt,
                                   floor=floor if name == "P_diss_iso" else 0.0)
    # the fields really moved: the comparison is not between two untouched copies
    assert not np.array_equal(new.download("temp"), host.temp)
    assert np.any(new.download("P_diss_iso") != 0.0)


def test_noalloc_rejects_domains_beyond_the_static_scratch():
    """A 0.25-degree domain needs more scratch than the static array holds: the
    call returns VG_ERR_SCRATCH before it enqueues anything. Every pointer is
    NULL, so a call that went past the capacity check would stop at the
    argument check (VG_ERR_ARG) instead of reaching the device."""
    from veros_gb300 import _capi

    lib = _capi.load()
    X, Y, Z = 1444, 724, 60
    pitch = 1456
    dom = _capi.VgDomain(X, Y, Z, pitch, pitch * Y)
    grid = _capi.VgGrid()
    ten = _capi.VgTensorFields()
    sett = _capi.VgIsoSettings(1e-3, 1e-3, 0.0, 43200.0, 9.81, 1024.0, 3, 1)
    tra = _capi.VgTracerArgs()
    st = lib.vg_isoneutral_diffusion_noalloc_f64(dom, grid, sett, ten, None, None, None, tra, 0, None)
    assert st == _capi.VG_ERR_SCRATCH
    assert "static buffer holds" in _capi.last_error()
