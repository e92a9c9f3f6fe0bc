"""Test infrastructure: the adjoint at its full workload against central
differences of the forward oracle in extended precision.

Workload (the adjoint benchmark's): 360 x 180 x 30 at 1 degree, eq. of state
3, lognormal K_iso (sigma 0.3), 8 steps, loss = sum over wet cells of
(temp after 8 steps - target)^2 with target = initial temp + N(0, 0.05).

At this size the loss gradient reaches 1e13 (temp) to 1e14 (salt) in a few
cells whose vertical density gradient nearly vanishes while their slope lies
in the taper's transition, so one unit in the last place of a tracer there
moves the loss by ~1e-2: central differences of an FP64 forward cannot get
below ~1e-4 relative at any step. This check therefore evaluates the forward
oracle (the reference algorithm, ``isoneutral_oracle.isoneutral_step``) in
``np.longdouble`` (64-bit significand on x86-64, 2^11 times finer than FP64)
and compares its central differences along 16 seeded random unit directions
(6 temp, 5 salt, 5 K_iso) with the CUDA adjoint's directional derivatives.

    python oracle/adjoint_fd_check.py cpu CPU.json [procs]       # longdouble differences + NumPy adjoint
    python oracle/adjoint_fd_check.py kinkfree CPU.json [procs]  # smaller steps, slope sign changes
                                                                 # counted; the adjoint in longdouble
    python oracle/adjoint_fd_check.py gpu GPU.json               # on a GPU: the CUDA adjoint
    python oracle/adjoint_fd_check.py compare CPU.json GPU.json

The CPU mode evaluates the longdouble central differences and, on the same
inputs, the directional derivatives of the NumPy FP64 adjoint
(``isoneutral_adjoint.rollout_grad``, which the GPU tests pin the CUDA
adjoint to at this size). The GPU mode records the CUDA adjoint's directional
derivatives and FP64 central differences of the CUDA forward. Both rebuild
the state and the directions from their seeds and record checksums of the
inputs: the synthetic state goes through exp and cos, whose last bits may
differ between hosts, so the GPU figures are compared with the longdouble
differences only where the checksums agree.
"""

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

NSTEPS = 8
NDIR = {"T": 6, "S": 5, "K": 5}
EPS_LD = {"T": (1e-11, 1e-12), "S": (1e-11, 1e-12), "K": (1e-7, 1e-8)}
# kink-free steps: small enough that no slope of the rollout changes sign between x - h u and x + h u
EPS_KF = {"T": (1e-13, 1e-14), "S": (1e-13, 1e-14), "K": (1e-10, 1e-11)}
EPS_64 = {"T": (1e-11,), "S": (1e-11,), "K": (1e-7,)}


def workload():
    from veros_gb300 import synthetic
    from oracle import isoneutral_adjoint as A

    host = synthetic.global_1deg_state(seed=0, nz=30, k_iso_lognormal_sigma=0.3)
    rng = np.random.default_rng(4)
    T0 = host.arrays["temp"][..., 1].copy()
    S0 = host.arrays["salt"][..., 1].copy()
    K = host.arrays["K_iso"].copy()
    wet = A.wet_interior(host)
    target = T0 + rng.normal(0.0, 0.05, T0.shape) * wet
    return host, T0, S0, K, target, wet


def directions(shape):
    rng = np.random.default_rng(2024)
    out = []
    for which, n in NDIR.items():
        for _ in range(n):
            u = rng.standard_normal(shape)
            out.append((which, u / np.linalg.norm(u)))
    return out


def checksums(arrays):
    import hashlib

    return {n: hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()[:16]
            for n, a in arrays.items()}


def run_gpu(path):
    import torch

    from veros_gb300.adjoint import IsoneutralAdjoint
    from veros_gb300.state import DeviceState

    host, T0, S0, K, target, wet = workload()
    model = IsoneutralAdjoint(DeviceState.from_host(host, device="cuda"))
    leaves = [model.field(x).requires_grad_() for x in (T0, S0, K)]
    T, _ = model.rollout(*leaves, NSTEPS)
    tgt, w = model.field(target), model.field(wet)
    loss = ((T - tgt) ** 2 * w).sum()
    loss.backward()
    grads = {n: leaf.grad.cpu().numpy() for n, leaf in zip("TSK", leaves)}

    def loss_of(x):
        Tx, Sx, Kx = (model.field(v) for v in (x["T"], x["S"], x["K"]))
        with torch.no_grad():
            for _ in range(NSTEPS):
                Tx, Sx = model.forward_step(Tx, Sx, Kx)
            return float(((Tx - tgt) ** 2 * w).sum())

    base = {"T": T0, "S": S0, "K": K}
    rows = []
    for which, u in directions(T0.shape):
        g = grads[which]
        row = {"which": which, "ad": float(np.sum(g * u)), "scale": float(np.linalg.norm(g) / np.sqrt(g.size)),
               "fd64": {}}
        for eps in EPS_64[which]:
            h = eps * float(np.linalg.norm(base[which]))
            plus = dict(base, **{which: base[which] + h * u})
            minus = dict(base, **{which: base[which] - h * u})
            row["fd64"][str(eps)] = (loss_of(plus) - loss_of(minus)) / (2 * h)
        rows.append(row)
    out = {"loss": float(loss.item()), "grad_norm": {n: float(np.linalg.norm(g)) for n, g in grads.items()},
           "checksums": checksums({"T0": T0, "S0": S0, "K": K, "target": target}), "directions": rows}
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({"loss": out["loss"], "grad_norm": out["grad_norm"]}))


def _ld_state():
    host, T0, S0, K, target, wet = workload()
    ld = lambda v: v.astype(np.longdouble) if v.dtype == np.float64 else v  # noqa: E731
    host.arrays = {k: ld(v) for k, v in host.arrays.items()}
    return host, ld(T0), ld(S0), ld(K), ld(target), ld(wet)


def _ld_loss(job):
    """The longdouble oracle's loss at base + sign * h * u (one rollout)."""
    idx, which, eps, sign = job
    from oracle import isoneutral_adjoint as A

    host, T0, S0, K, target, wet = _ld_state()
    dirs = directions(T0.shape)
    which_d, u = dirs[idx]
    assert which_d == which
    base = {"T": T0, "S": S0, "K": K}
    x = base[which]
    h = np.longdouble(eps) * np.sqrt(np.sum(x * x))
    base[which] = x + sign * h * u.astype(np.longdouble)
    T, S = base["T"], base["S"]
    for _ in range(NSTEPS):
        T, S, _ = A.forward_step(host, T, S, base["K"])
    L = np.sum(wet * (T - target) ** 2)
    return idx, str(eps), sign, str(L), str(h)


def _ld_cd(job):
    """Central difference of the longdouble oracle along direction idx with
    relative step eps, and the number of slopes (Ai components of every step)
    whose sign differs between the two rollouts."""
    idx, which, eps = job
    host, T0, S0, K, target, wet = _ld_state()
    which_d, u = directions(T0.shape)[idx]
    assert which_d == which
    x = {"T": T0, "S": S0, "K": K}[which]
    h = np.longdouble(eps) * np.sqrt(np.sum(x * x))
    from oracle import isoneutral_adjoint as A

    out = []
    for sign in (1, -1):
        base = {"T": T0, "S": S0, "K": K}
        base[which] = x + sign * h * u.astype(np.longdouble)
        T, S, signs = base["T"], base["S"], []
        for _ in range(NSTEPS):
            T, S, vs = A.forward_step(host, T, S, base["K"])
            signs.append(np.concatenate([np.sign(getattr(vs, n)).astype(np.int8).ravel()
                                         for n in ("Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")]))
        out.append((np.sum(wet * (T - target) ** 2), np.concatenate(signs)))
    (Lp, sp), (Lm, sm) = out
    return idx, str(eps), str((Lp - Lm) / (2 * h)), int(np.count_nonzero(sp != sm))


def _ld_adjoint(_):
    """The NumPy adjoint of the rollout, evaluated in longdouble."""
    from oracle import isoneutral_adjoint as A

    host, T0, S0, K, target, wet = _ld_state()
    L, gT, gS, gK = A.rollout_grad(host, T0, S0, K, target, NSTEPS)
    return [str(float(np.sum(g * u.astype(np.longdouble))))
            for (w, u), g in ((d, {"T": gT, "S": gS, "K": gK}[d[0]]) for d in directions(T0.shape))]


def run_cpu_kinkfree(path, procs):
    """Kink-free central differences and the longdouble adjoint, added to the CPU file."""
    import multiprocessing as mp

    with open(path) as f:
        data = json.load(f)
    jobs = [(idx, row["which"], eps) for idx, row in enumerate(data["directions"]) for eps in EPS_KF[row["which"]]]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(procs) as pool:
        adj = pool.map_async(_ld_adjoint, [0])
        results = pool.map(_ld_cd, jobs)
        ad_ld = adj.get()[0]
    worst = {}
    for idx, eps, fd, nflip in results:
        row = data["directions"][idx]
        row["ad_longdouble"] = float(ad_ld[idx])
        fd = float(np.longdouble(fd))
        sc = max(abs(row["ad_longdouble"]), row["scale"])
        e_ld = abs(fd - row["ad_longdouble"]) / sc
        row.setdefault("kink_free", {})[eps] = {"fd": fd, "slope_sign_changes": nflip,
                                                "rel_err_longdouble_adjoint": e_ld,
                                                "rel_err_numpy_adjoint": abs(fd - row["ad_numpy"]) / sc}
        key = f"{row['which']} eps={eps}"
        if nflip == 0:
            worst[key] = max(worst.get(key, 0.0), e_ld)
    for row in data["directions"]:
        row["numpy_fp64_vs_longdouble_adjoint"] = abs(row["ad_numpy"] - row["ad_longdouble"]) / max(
            abs(row["ad_longdouble"]), row["scale"])
    data["kink_free"] = {"eps": EPS_KF, "worst_rel_err_longdouble_adjoint_no_sign_change": worst,
                         "worst_numpy_fp64_vs_longdouble_adjoint": max(
                             r["numpy_fp64_vs_longdouble_adjoint"] for r in data["directions"]),
                         "seconds": time.perf_counter() - t0}
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print(json.dumps(data["kink_free"], indent=1))


def run_cpu(path, procs):
    import multiprocessing as mp

    from oracle import isoneutral_adjoint as A

    jobs = []
    for idx, (which, _) in enumerate(directions(workload()[1].shape)):
        for eps in EPS_LD[which]:
            for sign in (1, -1):
                jobs.append((idx, which, eps, sign))
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(procs) as pool:
        results = pool.map(_ld_loss, jobs)
    t_ld = time.perf_counter() - t0
    vals = {(idx, eps, sign): (np.longdouble(L), np.longdouble(h)) for idx, eps, sign, L, h in results}
    # the NumPy FP64 adjoint on the same inputs
    host, T0, S0, K, target, wet = workload()
    t0 = time.perf_counter()
    L64, gT, gS, gK = A.rollout_grad(host, T0, S0, K, target, NSTEPS)
    t_adj = time.perf_counter() - t0
    grads = {"T": gT, "S": gS, "K": gK}
    rows, worst = [], {}
    for idx, (which, u) in enumerate(directions(T0.shape)):
        g = grads[which]
        ad = float(np.sum(g * u))
        scale = float(np.linalg.norm(g) / np.sqrt(g.size))
        row = {"which": which, "ad_numpy": ad, "scale": scale, "fd_longdouble": {}}
        for eps in EPS_LD[which]:
            (Lp, h), (Lm, _) = vals[(idx, str(eps), 1)], vals[(idx, str(eps), -1)]
            fd = float((Lp - Lm) / (2 * h))
            err = abs(fd - ad) / max(abs(ad), scale)
            row["fd_longdouble"][str(eps)] = {"fd": fd, "rel_err_numpy_adjoint": err}
            worst[f"{which} eps={eps}"] = max(worst.get(f"{which} eps={eps}", 0.0), err)
        rows.append(row)
    out = {"loss_fp64": L64, "grad_norm": {n: float(np.linalg.norm(g)) for n, g in grads.items()},
           "checksums": checksums({"T0": T0, "S0": S0, "K": K, "target": target}),
           "longdouble_eps": float(np.finfo(np.longdouble).eps), "eps": EPS_LD,
           "worst_rel_err_numpy_adjoint": worst, "seconds": {"longdouble_rollouts": t_ld, "numpy_adjoint": t_adj},
           "procs": procs, "directions": rows}
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("worst_rel_err_numpy_adjoint", "seconds", "grad_norm")}, indent=1))


def compare(cpu_path, gpu_path):
    with open(cpu_path) as f:
        cpu = json.load(f)
    with open(gpu_path) as f:
        gpu = json.load(f)
    same = cpu["checksums"] == gpu["checksums"]
    out = {"same_inputs": same, "rows": []}
    for c, g in zip(cpu["directions"], gpu["directions"]):
        r = {"which": c["which"], "ad_cuda_vs_numpy": abs(g["ad"] - c["ad_numpy"]) / max(abs(c["ad_numpy"]), c["scale"]),
             "fd64_cuda_forward": {e: abs(v - g["ad"]) / max(abs(g["ad"]), g["scale"]) for e, v in g["fd64"].items()}}
        if same:
            r["ad_cuda_vs_fd_longdouble"] = {e: abs(v["fd"] - g["ad"]) / max(abs(g["ad"]), g["scale"])
                                             for e, v in c["fd_longdouble"].items()}
        out["rows"].append(r)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    mode = sys.argv[1]
    if mode == "gpu":
        run_gpu(sys.argv[2])
    elif mode == "cpu":
        run_cpu(sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else (os.cpu_count() or 1))
    elif mode == "kinkfree":
        run_cpu_kinkfree(sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else (os.cpu_count() or 1))
    else:
        compare(sys.argv[2], sys.argv[3])
