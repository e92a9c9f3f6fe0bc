"""plugin.install() against stand-in Veros modules (no GPU, no Veros import):
every attribute the reference's callers look up is rebound to this library's
drop-in and uninstall() restores the originals."""

import sys
import types

import pytest


@pytest.fixture
def fake_veros(monkeypatch):
    from veros_gb300 import plugin

    originals = {}
    for modname, attr, _ in plugin._TARGETS:
        parts = modname.split(".")
        for n in range(1, len(parts) + 1):
            name = ".".join(parts[:n])
            if name not in sys.modules or not getattr(sys.modules[name], "_vg_fake", False):
                mod = types.ModuleType(name)
                mod._vg_fake = True
                monkeypatch.setitem(sys.modules, name, mod)
        mod = sys.modules[modname]
        sentinel = object()
        setattr(mod, attr, sentinel)
        originals[(modname, attr)] = sentinel
    return originals


def test_install_rebinds_every_call_site_and_uninstall_restores(fake_veros):
    from veros_gb300 import plugin

    handle = plugin.install()
    for modname, attr, fn in plugin._TARGETS:
        assert getattr(sys.modules[modname], attr) is fn, (modname, attr)
    handle.uninstall()
    for (modname, attr), orig in fake_veros.items():
        assert getattr(sys.modules[modname], attr) is orig, (modname, attr)


def test_the_reference_call_sites_are_covered():
    """The names the reference's callers resolve at call time
    (veros/core/thermodynamics.py:430-432, veros/core/utilities.py:4)."""
    from veros_gb300 import plugin

    targets = {(m, a) for m, a, _ in plugin._TARGETS}
    for need in (("veros.core.isoneutral", "isoneutral_diffusion_pre"),
                 ("veros.core.isoneutral", "isoneutral_diffusion"),
                 ("veros.core.utilities", "solve_implicit"),
                 ("veros.core.utilities", "solve_tridiagonal"),
                 ("veros.core.operators", "solve_tridiagonal")):
        assert need in targets, need


def test_install_on_the_reference_modules_when_present():
    """With a reference checkout given in REF_ROOT, every target module and
    attribute exists in the real Veros and is rebound (skipped without it)."""
    import importlib
    import os

    from oracle.ref_tdma import reference_root

    ref = reference_root()
    if ref is None:
        pytest.skip("no reference checkout (set REF_ROOT)")
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    try:
        import make_golden
    finally:
        sys.path.pop(0)
    make_golden._import_reference(ref)
    from veros_gb300 import plugin

    for modname, attr, _ in plugin._TARGETS:
        assert hasattr(importlib.import_module(modname), attr), (modname, attr)
    handle = plugin.install()
    try:
        for modname, attr, fn in plugin._TARGETS:
            assert getattr(importlib.import_module(modname), attr) is fn
    finally:
        handle.uninstall()


def test_vertmix_raises_on_several_processes(monkeypatch):
    """A multi-process Veros (runtime_state.proc_num > 1) would need the
    domain decomposition's halo exchange at the end of vertmix_tempsalt
    (veros/core/utilities.py:18-20): the drop-in refuses before any GPU work."""
    from veros_gb300 import thermodynamics

    fake = types.ModuleType("veros")
    fake.runtime_state = types.SimpleNamespace(proc_num=2)
    monkeypatch.setitem(sys.modules, "veros", fake)
    with pytest.raises(NotImplementedError, match="2 processes"):
        thermodynamics.vertmix_tempsalt(object())
    fake.runtime_state.proc_num = 1
    from veros_gb300.state import require_single_process

    require_single_process("one process")  # no error


def test_veros_like_state_keeps_the_reference_contract():
    """The stand-in state the GPU drop-in tests use behaves like the reference's
    VerosVariables (veros/state.py:70-90, :219-243)."""
    import collections

    import numpy as np

    from veros_like import VerosLikeState

    st = VerosLikeState(dict(nx=2, ny=2, nz=3), {"temp": np.zeros((6, 6, 3, 3)), "kbot": np.zeros((6, 6), int)})
    vs = st.variables
    assert not vs.temp.flags.writeable
    with pytest.raises(ValueError):
        vs.temp[0, 0, 0, 0] = 1.0
    assert vs.update(None) is vs  # a routine's None result changes nothing
    KO = collections.namedtuple("KernelOutput", ["temp"])
    vs.update(KO(temp=np.ones((6, 6, 3, 3), dtype=np.float32)))
    assert vs.temp.dtype == np.float64 and vs.temp[0, 0, 0, 0] == 1.0
    same = np.zeros((6, 6, 3, 3))
    vs.temp = same
    assert vs.temp is same  # asarray keeps the object when the dtype matches
    with pytest.raises(ValueError, match="unexpected shape"):
        vs.temp = np.ones((6, 6, 3))
    with pytest.raises(AttributeError):
        vs.update({"unknown": 1})
    assert vs.kbot.dtype.kind == "i"
