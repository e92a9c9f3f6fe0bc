"""A stand-in for the reference's NumPy-backend ``VerosState``, for tests.

The GPU machine has no Veros checkout, so the drop-ins' host-array branch (the
one a ``plugin.install()``-ed Veros takes) is driven through this object. It
keeps the parts of the reference's state contract that the drop-ins touch:

* ``state.settings.<name>`` (``nx``, ``ny``, ``nz`` and the model settings);
* ``state.variables.<field>`` as NumPy arrays, allocated read-only as the
  NumPy backend allocates them (veros/variables.py:941), so a drop-in that
  tried to write a host array in place would fail here as it would there;
* assignment stores ``asarray(val, dtype=...)`` (the given object when its
  dtype matches) and rejects a changed shape with ``ValueError``
  (veros/state.py:219-243);
* ``variables.update(other=None, **fields)`` takes a namedtuple
  (``KernelOutput``), a dict or nothing, and rejects unknown names with
  ``AttributeError`` (veros/state.py:70-90);
* ``tau``, ``taup1``, ``taum1`` integers.

``plugin_call_sites`` registers stand-in ``veros.core.*`` modules, installs
the drop-ins into them and returns those modules, so a test calls
``isoneutral.isoneutral_diffusion_pre(state)`` exactly as
veros/core/thermodynamics.py:430-432 does.
"""

import sys
import types

import numpy as np


class Namespace:
    def __init__(self, **kw):
        self.__dict__.update(kw)

    def get(self, name, default=None):
        return self.__dict__.get(name, default)


class VerosLikeVariables:
    def __init__(self, arrays, dtypes, tau, taup1, taum1):
        object.__setattr__(self, "_dtypes", dict(dtypes))
        object.__setattr__(self, "_names", set(arrays))
        object.__setattr__(self, "tau", int(tau))
        object.__setattr__(self, "taup1", int(taup1))
        object.__setattr__(self, "taum1", int(taum1))
        for k, v in arrays.items():
            object.__setattr__(self, k, self._readonly(np.array(v, dtype=self._dtypes[k])))

    @staticmethod
    def _readonly(arr):
        arr.flags.writeable = False
        return arr

    def __setattr__(self, key, val):
        if key.startswith("_") or key not in self._names:
            return object.__setattr__(self, key, val)
        # as the reference: asarray (the same object when the dtype already matches), shape check
        new = np.asarray(val, dtype=self._dtypes[key])
        old = getattr(self, key)
        if new.shape != old.shape:
            raise ValueError(f"Got unexpected shape for variable {key} (expected: {old.shape}, got: {new.shape})")
        object.__setattr__(self, key, new)

    def update(self, other=None, **new_fields):
        if other is not None:
            if new_fields:
                raise ValueError("Either other or new_fields can be given")
            if hasattr(other, "_fields"):
                new_fields = dict(zip(other._fields, other))
            elif isinstance(other, dict):
                new_fields = other
            else:
                raise TypeError(f"Cannot update from {type(other)} type")
        for key in new_fields:
            if key not in self._names:
                raise AttributeError(f"unknown attribute {key}")
        for key, val in new_fields.items():
            setattr(self, key, val)
        return self


class VerosLikeState:
    def __init__(self, settings, arrays, tau=1, taup1=2, taum1=0, float_type=np.float64):
        self.settings = Namespace(**settings)
        dtypes = {}
        for k, v in arrays.items():
            v = np.asarray(v)
            dtypes[k] = v.dtype if v.dtype.kind in "biu" else np.dtype(float_type)
        self.variables = VerosLikeVariables(arrays, dtypes, tau, taup1, taum1)


def state_from_golden(g, float_type=np.float64):
    """A VerosLikeState from a golden case's ``in_*`` arrays and ``setting_*`` values."""
    arrays = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    X, Y, Z = arrays["temp"].shape[:3]
    settings.update(nx=X - 4, ny=Y - 4, nz=Z)
    return VerosLikeState(settings, arrays, int(g["tau"]), int(g["taup1"]), int(g["taum1"]), float_type)


def plugin_call_sites(monkeypatch):
    """Stand-in ``veros``, ``veros.core`` and the target modules in
    ``sys.modules`` (undone by ``monkeypatch``), the drop-ins installed into
    them. Returns ``(modules by name, install handle)``."""
    from veros_gb300 import plugin

    mods = {}
    for modname, _, _ in plugin._TARGETS:
        parts = modname.split(".")
        for n in range(1, len(parts) + 1):
            name = ".".join(parts[:n])
            if name not in mods:
                mods[name] = types.ModuleType(name)
                monkeypatch.setitem(sys.modules, name, mods[name])
    for modname, attr, _ in plugin._TARGETS:
        setattr(mods[modname], attr, None)
    handle = plugin.install()
    return mods, handle
