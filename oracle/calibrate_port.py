"""Test infrastructure: how fast the oracle port runs against the reference itself.

The benchmark's CPU legs (``cpu_baseline`` and ``bench.py --impl reference``)
time ``isoneutral_oracle.isoneutral_step``, the NumPy restatement of the
reference algorithm, because the reference cannot run on the GPU machine. This
script times both on the same host core and the same sample, so the port's
rate can be read as the reference's: one isoneutral step of a 360 x 24 x 60
y-band of the 1-degree workload (nonlinear EOS), the step of
veros/core/thermodynamics.py:226-241 and :425-432 with zero advection,
``perf_counter`` per step after 3 burn-in steps (the reference's
benchmarks/run_benchmarks.py:171 discards the first steps the same way).

The reference runs from its checkout (``REF_ROOT`` or the argument), in the
same process, through ``isoneutral_diffusion_pre`` and ``isoneutral_diffusion``
on a ``VerosState`` built like the golden fixtures. NumPy runs this path on
one core; the BLAS thread pools are pinned to one thread first so that the
reference's LAPACK call does not spread.

    python oracle/calibrate_port.py [reference checkout] [steps]

prints one JSON line.
"""

import json
import os
import sys
import time

for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ[var] = "1"

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))

NX, NY_BAND, NZ = 360, 24, 60
BURN_IN = 3


def band_state(seed=0):
    from veros_gb300 import synthetic

    return synthetic.make_state(NX, NY_BAND, NZ, seed=seed, y_origin=-30.0, dz_top=10.0, dz_bottom=250.0,
                                land_fraction=0.30, eq_of_state_type=3)


def time_port(host, steps):
    from oracle import isoneutral_oracle as orc

    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    times = []
    for n in range(BURN_IN + steps):
        t0 = time.perf_counter()
        orc.isoneutral_step(vs, host.settings)
        times.append(time.perf_counter() - t0)
    return times[BURN_IN:]


def time_reference(host, steps):
    import make_golden
    from veros.core import isoneutral
    from veros.core.operators import at, update

    state = make_golden._reference_state_from_host(host)
    vs = state.variables
    times = []
    for n in range(BURN_IN + steps):
        t0 = time.perf_counter()
        # thermodynamics.py:226-241 with zero advection: the new level starts as the old one
        vs.temp = update(vs.temp, at[..., vs.taup1], vs.temp[..., vs.tau] * vs.maskT)
        vs.salt = update(vs.salt, at[..., vs.taup1], vs.salt[..., vs.tau] * vs.maskT)
        # thermodynamics.py:425-432
        vs.P_diss_iso = update(vs.P_diss_iso, at[...], 0.0)
        vs.dtemp_iso = update(vs.dtemp_iso, at[...], 0.0)
        vs.dsalt_iso = update(vs.dsalt_iso, at[...], 0.0)
        vs.update(isoneutral.isoneutral_diffusion_pre(state))
        vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.temp, istemp=True))
        vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.salt, istemp=False))
        # veros.py:321-322
        vs.taum1, vs.tau, vs.taup1 = vs.tau, vs.taup1, vs.taum1
        times.append(time.perf_counter() - t0)
    return times[BURN_IN:]


def main():
    args = sys.argv[1:]
    ref = args.pop(0) if args and not args[0].isdigit() else None
    if ref is None:
        from oracle.ref_tdma import reference_root

        ref = reference_root()
    if ref is None or not os.path.isdir(os.path.join(ref, "veros")):
        sys.exit("usage: calibrate_port.py <reference checkout> [steps]  (or set REF_ROOT)")
    steps = int(args[0]) if args else 5
    import make_golden

    make_golden._import_reference(ref)
    host = band_state()
    cells = NX * NY_BAND * NZ
    ref_t = time_reference(host, steps)
    port_t = time_port(host, steps)
    out = {
        "sample": f"{NX}x{NY_BAND}x{NZ} y-band of the 1-degree workload, eq 3, one step = pre + diffusion of "
                  f"temp and salt; {steps} steps after {BURN_IN} burn-in",
        "cores": 1,
        "host_cpus": os.cpu_count(),
        "reference_s_per_step": {"best": min(ref_t), "mean": float(np.mean(ref_t))},
        "port_s_per_step": {"best": min(port_t), "mean": float(np.mean(port_t))},
        "reference_cells_per_s": cells / float(np.mean(ref_t)),
        "port_cells_per_s": cells / float(np.mean(port_t)),
        "port_over_reference_speed": float(np.mean(ref_t) / np.mean(port_t)),
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
