import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(autouse=True)
def _seed():
    import numpy as np

    np.random.seed(17)


def load_golden(name):
    import numpy as np

    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as f:
        return {k: f[k] for k in f.files}


# FP64 parity bar: relative max-norm per field.
TOL_F64 = 1e-12
TENDENCY_FIELDS = ("dtemp_iso", "dsalt_iso")


def field_error(got, ref):
    """max |got - ref| / max |ref| (absolute if ref is all zero)."""
    import numpy as np

    if ref.size == 0:
        return 0.0
    scale = float(np.max(np.abs(ref)))
    diff = float(np.max(np.abs(got - ref)))
    return diff / scale if scale > 0 else diff


def p_diss_floor(arrays, settings, tau):
    """Differencing floor of P_diss_iso: its vertical-mixing term carries
    K_33 (tr_new[k+1] - tr_new[k]) / dzw (veros/core/isoneutral/diffusion.py:266-279),
    so 4 ulp of each tracer times the largest coefficient of that difference."""
    import numpy as np

    g = settings["grav"] if isinstance(settings, dict) else settings.grav
    rho = settings["rho_0"] if isinstance(settings, dict) else settings.rho_0
    dzw = arrays["dzw"][:-1]
    K33 = arrays["K_33"][:, :, :-1]
    floor = 0.0
    for trn, idn in (("temp", "int_drhodT"), ("salt", "int_drhodS")):
        I = arrays[idn][..., tau]
        fxa = (I[:, :, :-1] - I[:, :, 1:]) / dzw
        coef = np.abs(g / rho * fxa * K33 / dzw)
        floor += 4.0 * float(np.spacing(np.max(np.abs(arrays[trn])))) * float(np.max(coef))
    return floor


def assert_field_close(name, got, ref, tracer=None, dt=None, tol=TOL_F64, floor=0.0):
    """Relative max-norm <= tol.

    The iso tendencies are (tr_new - tr_old) / dt of two numbers of the
    tracer's magnitude, so one unit in the last place of the tracer is already
    ~1e-12 of their max-norm; for them the bound adds that differencing floor,
    4 ulp(max|tracer|) / dt, to tol * max|ref|.
    """
    import numpy as np

    scale = float(np.max(np.abs(ref))) if ref.size else 0.0
    diff = float(np.max(np.abs(got - ref))) if ref.size else 0.0
    bound = tol * scale + floor
    if name in TENDENCY_FIELDS and tracer is not None and dt is not None:
        bound += 4.0 * float(np.spacing(np.max(np.abs(tracer)))) / dt
    assert diff <= bound or (scale == 0 and diff == 0), (
        f"{name}: max|diff| {diff:.3e} > bound {bound:.3e} (relative {diff / scale if scale else diff:.3e})")
