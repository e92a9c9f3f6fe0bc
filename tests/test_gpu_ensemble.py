"""Batched ensemble: one persistent launch per stage over members of uneven
extents must reproduce each member's single-domain step exactly (the same
tile bodies run on the same data), for every tiling and under graph replay."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FIELDS = ("temp", "salt", "dtemp_iso", "dsalt_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")


def _hosts():
    from veros_gb300 import synthetic

    shapes = [(37, 29, 15), (64, 33, 30), (45, 52, 45), (96, 40, 60), (33, 32, 30)]
    return [synthetic.make_state(nx, ny, nz, seed=20 + m, eq_of_state_type=3, land_fraction=0.15, dz_bottom=250.0)
            for m, (nx, ny, nz) in enumerate(shapes)]


def _pair(precision):
    from veros_gb300.state import DeviceState

    hosts = _hosts()
    return ([DeviceState.from_host(h, precision=precision) for h in hosts],
            [DeviceState.from_host(h, precision=precision) for h in hosts])


def _assert_same(a, b):
    for x, y in zip(a, b):
        assert x.variables.tau == y.variables.tau
        for n in FIELDS:
            np.testing.assert_array_equal(x.download(n), y.download(n), err_msg=n)


@pytest.mark.parametrize("precision", ["f64", "f32split"])
def test_ensemble_matches_single_domain_steps(precision):
    from veros_gb300.ensemble import Ensemble
    from veros_gb300.step import IsoneutralStepper

    batched, single = _pair(precision)
    ens = Ensemble(batched)
    ens.step(4)
    for dev in single:
        IsoneutralStepper(dev).step(4)
    torch.cuda.synchronize()
    _assert_same(batched, single)
    ens.close()


def test_every_tiling_gives_the_same_fields():
    from veros_gb300.ensemble import Ensemble
    from veros_gb300.step import IsoneutralStepper

    batched, single = _pair("f64")
    ens = Ensemble(batched)
    tilings = [dict(pre_rows=4, pre_kchunk=16, flux_rows=4, flux_kchunk=0, solve_threads=32),
               dict(pre_rows=8, pre_kchunk=0, flux_rows=8, flux_kchunk=16, solve_threads=64),
               dict(pre_rows=4, pre_kchunk=32, flux_rows=8, flux_kchunk=32, solve_threads=64),
               # equal shares of all members' tile-levels per resident CTA
               dict(pre_rows=8, pre_kchunk=-1, flux_rows=8, flux_kchunk=-1, solve_threads=64),
               dict(pre_rows=4, pre_kchunk=-1, flux_rows=4, flux_kchunk=-1, solve_threads=32)]
    for t in tilings:
        ens.tune(**t)
        ens.step(1)
    for dev in single:
        IsoneutralStepper(dev).step(len(tilings))
    torch.cuda.synchronize()
    _assert_same(batched, single)
    ens.close()


def test_graph_replay_matches_eager_and_autotune_runs():
    from veros_gb300.ensemble import Ensemble

    batched, eager = _pair("f64")
    e1, e2 = Ensemble(batched), Ensemble(eager)
    tuning, timings = e1.autotune(steps=1, kchunks=(0, 16))
    assert set(tuning) == {"pre_rows", "pre_kchunk", "flux_rows", "flux_kchunk", "solve_threads"}
    assert len(timings) >= 6
    e2.tune(**tuning)
    e2.step(e1.steps_taken)  # autotuning advanced e1 by the steps it timed
    assert e1.phase == e2.phase
    e1.replay(5)
    e1.replay(5)
    e2.step(10)
    torch.cuda.synchronize()
    _assert_same(batched, eager)
    e1.close()
    e2.close()


def test_members_against_the_oracle_at_their_own_shapes():
    """Each member of an uneven ensemble against one oracle step (the reference
    algorithm) from the same state, at its own extents: the smallest shapes of
    the benchmark's member distribution (nx = ny = 32 with 15 levels), a
    60-level member, and odd extents. Relative max-norm 1e-12 per field, as
    for the single-domain drop-in; land cells exactly zero."""
    from oracle import isoneutral_oracle as orc
    from veros_gb300 import synthetic
    from veros_gb300.ensemble import Ensemble
    from veros_gb300.state import DeviceState

    from conftest import assert_field_close

    shapes = [(32, 32, 15), (41, 33, 60), (70, 37, 30), (32, 45, 45)]
    hosts = [synthetic.make_state(nx, ny, nz, seed=40 + m, eq_of_state_type=3, land_fraction=0.3, dz_bottom=250.0)
             for m, (nx, ny, nz) in enumerate(shapes)]
    devs = [DeviceState.from_host(h) for h in hosts]
    ens = Ensemble(devs)
    ens.step(1)
    torch.cuda.synchronize()
    for h, dev in zip(hosts, devs):
        vs = orc.OracleState({k: v.copy() for k, v in h.arrays.items()})
        orc.isoneutral_step(vs, h.settings)
        dt = h.settings["dt_tracer"]
        for n in FIELDS:
            ref = getattr(vs, n)
            tracer = vs.temp if n == "dtemp_iso" else vs.salt if n == "dsalt_iso" else None
            assert_field_close(n, dev.download(n), ref, tracer=tracer, dt=dt)
        land = ~h.arrays["maskT"].astype(bool)
        assert np.all(dev.download("dtemp_iso")[land] == 0.0)
    ens.close()
