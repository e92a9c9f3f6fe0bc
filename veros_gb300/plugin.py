"""Install the GB300 drop-ins into an imported Veros (NumPy backend).

Callers reach the hot path by attribute lookup at call time
(veros/core/thermodynamics.py:430-432 calls ``isoneutral.isoneutral_diffusion_pre``
and friends; veros/core/isoneutral/diffusion.py:165 and the other physics call
``utilities.solve_implicit``), and ``solve_tridiagonal`` is bound by name into
``veros.core.utilities`` at import (veros/core/utilities.py:4). ``install``
rebinds all of them and returns a handle whose ``uninstall()`` restores the
originals. A module reload of ``veros.core.*`` undoes the patch, so tests that
reload Veros must install inside the test.
"""

from . import isoneutral as _iso
from . import thermodynamics as _thermo
from . import utilities as _util

_TARGETS = (
    ("veros.core.isoneutral", "isoneutral_diffusion_pre", _iso.isoneutral_diffusion_pre),
    ("veros.core.isoneutral", "isoneutral_diffusion", _iso.isoneutral_diffusion),
    ("veros.core.isoneutral", "isoneutral_skew_diffusion", _iso.isoneutral_skew_diffusion),
    ("veros.core.isoneutral.isoneutral", "isoneutral_diffusion_pre", _iso.isoneutral_diffusion_pre),
    ("veros.core.isoneutral.diffusion", "isoneutral_diffusion", _iso.isoneutral_diffusion),
    ("veros.core.isoneutral.diffusion", "isoneutral_skew_diffusion", _iso.isoneutral_skew_diffusion),
    ("veros.core.isoneutral", "isoneutral_diag_streamfunction", _iso.isoneutral_diag_streamfunction),
    ("veros.core.isoneutral.isoneutral", "isoneutral_diag_streamfunction", _iso.isoneutral_diag_streamfunction),
    ("veros.core.isoneutral.isoneutral", "isoneutral_diag_streamfunction_kernel",
     _iso.isoneutral_diag_streamfunction_kernel),
    ("veros.core.thermodynamics", "vertmix_tempsalt", _thermo.vertmix_tempsalt),
    ("veros.core.utilities", "solve_implicit", _util.solve_implicit),
    ("veros.core.utilities", "solve_tridiagonal", _util.solve_tridiagonal),
    ("veros.core.operators", "solve_tridiagonal", _util.solve_tridiagonal),
)


class Installed:
    def __init__(self, saved):
        self._saved = saved

    def uninstall(self):
        for mod, name, orig in self._saved:
            setattr(mod, name, orig)
        self._saved = []


def install():
    import importlib

    saved = []
    for modname, attr, fn in _TARGETS:
        mod = importlib.import_module(modname)
        saved.append((mod, attr, getattr(mod, attr)))
        setattr(mod, attr, fn)
    return Installed(saved)
