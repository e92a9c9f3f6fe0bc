"""GB300-native (sm_103a) isoneutral mixing for the Veros ocean model.

Drop-in replacements, with the reference signatures, for
``veros.core.isoneutral.isoneutral_diffusion_pre``,
``isoneutral_diffusion`` / ``isoneutral_skew_diffusion`` and
``veros.core.utilities.solve_implicit`` / ``solve_tridiagonal``, running as
hand-written CUDA kernels behind a C ABI (``include/veros_gb300.h``).
"""

from .state import DeviceState, Settings, KernelOutput  # noqa: F401
from .isoneutral import isoneutral_diffusion_pre, isoneutral_diffusion, isoneutral_skew_diffusion  # noqa: F401
from .utilities import solve_implicit, solve_tridiagonal, create_water_masks  # noqa: F401
from .step import IsoneutralStepper  # noqa: F401

__version__ = "0.1.0"
