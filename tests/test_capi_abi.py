"""The C ABI without a GPU: the library loads, exports every declared symbol,
and rejects bad arguments with status codes (no CUDA call is reached).

Non-NULL pointer arguments come from ``_buffer``: where a GPU is present, real
zeroed device memory large enough for every access the small test domains
allow, so that a regression that let a call past its argument check would
compute on valid memory and fail the status assertion, not fault the GPU;
without a GPU, placeholder addresses that no call ever dereferences (a launch
would fail with "no device")."""

import ctypes
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "veros_gb300.h")


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from veros_gb300 import _build, _capi

    if not os.path.exists(_capi.LIB_PATH):
        _build.build()
    return _capi.load()


def test_every_declared_symbol_is_exported_and_bound(lib):
    from veros_gb300 import _capi

    names = _declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
        assert n in _capi.SIGNATURES, f"{n} has no ctypes signature"


def test_version_and_empty_error(lib):
    assert lib.vg_version().startswith(b"veros_gb300")


_KEEP = []


def _buffer(nbytes=1 << 16):
    """Address of ``nbytes`` of zeroed device memory (placeholder without a GPU)."""
    try:
        import torch

        if torch.cuda.is_available():
            t = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
            _KEEP.append(t)
            return t.data_ptr()
    except ImportError:
        pass
    return 1 << 40


def _dom(X=10, Y=9, Z=5, pitch=16):
    from veros_gb300 import _capi

    return _capi.VgDomain(X, Y, Z, pitch, pitch * Y)


def test_bad_domain_is_rejected(lib):
    from veros_gb300 import _capi

    st = lib.vg_pack_masks(_dom(X=3), None, None, None, None, None, None)
    assert st == _capi.VG_ERR_SHAPE
    assert "X=3" in _capi.last_error()
    st = lib.vg_pack_masks(_dom(pitch=4), None, None, None, None, None, None)
    assert st == _capi.VG_ERR_STRIDE
    st = lib.vg_pack_masks(_dom(Z=1), None, None, None, None, None, None)
    assert st == _capi.VG_ERR_SHAPE


def test_null_pointers_and_settings_are_rejected(lib):
    from veros_gb300 import _capi

    grid = _capi.VgGrid()
    sett = _capi.VgIsoSettings(1e-3, 1e-3, 0.0, 3600.0, 9.81, 1024.0, 3, 0)
    ten = _capi.VgTensorFields()
    st = lib.vg_isoneutral_pre_f64(_dom(), grid, sett, None, None, None, None, ten, None)
    assert st == _capi.VG_ERR_ARG
    with pytest.raises(ValueError):
        _capi.check(st, "pre")
    # an unsupported equation of state is reported before any launch
    buf = ctypes.c_void_p(_buffer())
    grid = _capi.VgGrid(*([buf] * 9))
    ten = _capi.VgTensorFields(*([buf] * 7), 1, 1)
    sett.eq_of_state_type = 5
    st = lib.vg_isoneutral_pre_f64(_dom(), grid, sett, buf, buf, buf, buf, ten, None)
    assert st == _capi.VG_ERR_UNSUPPORTED
    with pytest.raises(NotImplementedError):
        _capi.check(st, "pre")


def test_diffusion_scratch_contract(lib):
    from veros_gb300 import _capi

    d = _dom()
    need = lib.vg_isoneutral_diffusion_scratch_bytes(d)
    assert need == 3 * d.plane * d.Z * 8
    buf = ctypes.c_void_p(_buffer())
    grid = _capi.VgGrid(*([buf] * 9))
    ten = _capi.VgTensorFields(*([buf] * 7), 1, 1)
    sett = _capi.VgIsoSettings(1e-3, 1e-3, 0.0, 3600.0, 9.81, 1024.0, 1, 0)
    tr = _capi.VgTracerArgs(buf, buf, buf, None, None)
    st = lib.vg_isoneutral_diffusion_f64(d, grid, sett, ten, buf, buf, buf, tr, 0, buf, need - 8, None)
    assert st == _capi.VG_ERR_SCRATCH
    st = lib.vg_isoneutral_diffusion_f64(d, grid, sett, ten, buf, buf, buf, tr, 2, buf, need, None)
    assert st == _capi.VG_ERR_ARG
    sett.enable_conserve_energy = 1
    st = lib.vg_isoneutral_diffusion_f64(d, grid, sett, ten, buf, buf, buf, tr, 0, buf, need, None)
    assert st == _capi.VG_ERR_ARG


def test_tridiag_shape_checks(lib):
    from veros_gb300 import _capi

    st = lib.vg_solve_implicit_f64(4, 4, 0, 1, 4, 16, *([None] * 11))
    assert st == _capi.VG_ERR_SHAPE
    st = lib.vg_solve_implicit_f64(4, 4, 10, 1, 4, 16, *([None] * 11))
    assert st == _capi.VG_ERR_ARG
    # the output may not overlap an input (checked on the pointers, before any
    # launch; only overlapping cases here, all inside one buffer and 8-byte
    # aligned); 16 columns x 10 levels of doubles span 1280 bytes
    base = _buffer(8 * 4096) + 4096
    arrs = [base + n * 4096 for n in range(6)] + [None, None]  # a b c d water edge b_edge d_edge
    for out in (arrs[3], arrs[1] + 1272, arrs[4] - 1272, arrs[0] - 1272):
        st = lib.vg_solve_implicit_f64(4, 4, 10, 10, 40, 1, *arrs, out, None, None)
        assert st == _capi.VG_ERR_ARG and "overlaps" in _capi.last_error()
    # the XLA-style entry keeps the error instead of exiting
    desc = b"\x00" * 4
    lib.vg_tdma_cuda_double(None, (ctypes.c_void_p * 6)(), desc, len(desc))
    assert "descriptor" in _capi.last_error()
