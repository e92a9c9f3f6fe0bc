"""GPU parity on edge-case domains.

The smallest domain the path accepts (one interior column, two levels), a
domain of land only, water at full depth everywhere, a single wet column in
land, extents that leave partial tiles in x and y (the kernels' 32-wide
rows and their 8- and 4-row tiles), and 160 levels (the per-level tables,
and the implicit solve's shared memory at half its column count). Each: one FP64 step against one oracle
step at the 1e-12 parity bar (energy branch on and off), and one split step
whose tracers stay within 1e-6 of the oracle's.
"""

import numpy as np
import pytest

from conftest import field_error
from test_gpu_parity import STEP_FIELDS, _check_state

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _edge_state(case, energy):
    """A synthetic state (eq. of state 3) of the named edge case."""
    from veros_gb300 import synthetic

    shapes = {"minimum": (1, 1, 2, 0.0), "all_land": (20, 12, 6, 1.0), "full_depth": (40, 17, 12, 0.0),
              "single_column": (9, 9, 10, 1.0), "partial_tiles": (33, 9, 7, 0.2),
              "partial_tiles_small": (31, 7, 3, 0.2), "deep": (36, 20, 160, 0.2)}
    nx, ny, nz, land = shapes[case]
    host = synthetic.make_state(nx, ny, nz, seed=sum(map(ord, case)), eq_of_state_type=3, land_fraction=land,
                                dz_bottom=250.0, settings=dict(enable_conserve_energy=energy))
    kb = None
    if case == "full_depth":
        kb = np.ones((nx, ny), dtype=np.int32)
    elif case == "single_column":
        kb = np.zeros((nx, ny), dtype=np.int32)
        kb[nx // 2, ny // 2] = 1
    if kb is not None:
        # new bottom: masks from kbot, tracers from the synthetic profiles on the new wet cells
        a = host.arrays
        full = np.zeros((nx + 4, ny + 4), dtype=np.int32)
        full[2:-2, 2:-2] = kb
        kbot, mT, mU, mV, mW = synthetic.calc_topo(full, nz)
        rng = np.random.default_rng(7)
        zt = a["zt"]
        shape = (nx + 4, ny + 4, nz)
        temp = ((2.0 + 20.0 * np.exp(zt / 800.0))[None, None, :] + rng.normal(0.0, 0.1, shape)) * mT
        salt = ((35.0 + 0.5 * np.exp(zt / 500.0))[None, None, :] + rng.normal(0.0, 0.01, shape)) * mT
        a.update(kbot=kbot, maskT=mT, maskU=mU, maskV=mV, maskW=mW,
                 temp=np.repeat(temp[..., None], 3, axis=-1), salt=np.repeat(salt[..., None], 3, axis=-1))
        p = np.abs(zt)[None, None, :, None]
        a["int_drhodT"] = synthetic.eos_int_drhodT(3, a["temp"], p) * np.ones_like(a["temp"])
        a["int_drhodS"] = synthetic.eos_int_drhodS(3, p) * np.ones_like(a["salt"])
    return host


CASES = ["minimum", "all_land", "full_depth", "single_column", "partial_tiles", "partial_tiles_small", "deep"]


@pytest.mark.parametrize("energy", [False, True])
@pytest.mark.parametrize("case", CASES)
def test_edge_domain_step_vs_oracle(case, energy):
    from oracle import isoneutral_oracle as orc
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = _edge_state(case, energy)
    dev = DeviceState.from_host(host)
    IsoneutralStepper(dev).step(1)
    torch.cuda.synchronize()
    vs = orc.OracleState({k: np.array(v, copy=True) for k, v in host.arrays.items()}, tau=host.tau,
                         taup1=host.taup1, taum1=host.taum1)
    tau_in = vs.tau
    orc.isoneutral_step(vs, host.settings)
    assert dev.variables.tau == vs.tau
    _check_state(dev, vs, STEP_FIELDS + (("P_diss_iso",) if energy else ()), host.settings, tau_in)
    land = ~host.arrays["maskT"].astype(bool)
    assert np.all(dev.download("temp")[..., vs.tau][land] == 0.0)
    if case == "all_land":
        for n in ("dtemp_iso", "dsalt_iso", "K_11", "K_33", "Ai_ez"):
            assert not np.any(dev.download(n)), n


@pytest.mark.parametrize("case", CASES)
def test_edge_domain_split_step_vs_oracle(case):
    from oracle import isoneutral_oracle as orc
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = _edge_state(case, False)
    dev = DeviceState.from_host(host, precision="f32split")
    IsoneutralStepper(dev).step(1)
    torch.cuda.synchronize()
    vs = orc.OracleState({k: np.array(v, copy=True) for k, v in host.arrays.items()}, tau=host.tau,
                         taup1=host.taup1, taum1=host.taum1)
    orc.isoneutral_step(vs, host.settings)
    for n in ("temp", "salt"):
        assert field_error(dev.download(n), getattr(vs, n)) <= 1e-6, n
