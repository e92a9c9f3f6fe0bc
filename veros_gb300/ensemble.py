"""Batched ensembles: many domains stepped together on one GPU.

An :class:`Ensemble` holds :class:`DeviceState` members of uneven extents
(nx, ny, nz, kbot) sharing one precision. Each step is one persistent launch
per stage over a work list of (member, tile) items (``vg_ensemble_step``), so
the whole ensemble costs four launches per step however many members it has,
and a rollout can be recorded once as a CUDA graph and replayed.

The tile shape (columns per CTA of the slope and flux kernels), their
k-chunks and the implicit-solve CTA size are chosen by :meth:`autotune`, which
times candidate tilings on the ensemble itself with CUDA events and keeps the
fastest (the result is cached per ensemble shape for the process).
"""

import ctypes
import itertools

import torch

from . import _capi

_TUNE_CACHE = {}

DEFAULT_TUNING = dict(pre_rows=8, pre_kchunk=0, flux_rows=8, flux_kchunk=0, solve_threads=64)


def _rotate(idx, p):
    taum1, tau, taup1 = idx
    for _ in range(p):
        taum1, tau, taup1 = tau, taup1, taum1
    return taum1, tau, taup1


class Ensemble:
    def __init__(self, states, tuning=None):
        if not states:
            raise ValueError("an ensemble needs at least one member")
        prec = {s.precision for s in states}
        if len(prec) != 1:
            raise ValueError("all members must share one precision")
        self.states = list(states)
        self.precision = prec.pop()
        self.device = self.states[0].device
        if any(s.device != self.device for s in self.states):
            raise ValueError("all members must live on one device")
        if any(bool(s.settings.enable_conserve_energy) for s in self.states):
            raise NotImplementedError("the batched ensemble does not include the energy branch")
        self.lib = _capi.load()
        f64 = self.precision == "f64"
        self._member_t = _capi.VgEnsembleMember if f64 else _capi.VgEnsembleMemberF32
        self._fields_t = _capi.VgStepFields if f64 else _capi.VgStepFieldsF32
        members = (self._member_t * len(self.states))()
        self._start = []
        for m, dev in zip(members, self.states):
            v = dev.variables
            idx = (v.taum1, v.tau, v.taup1)
            self._start.append(idx)
            m.dom = dev.domain()
            m.grid = dev.grid()
            m.set = dev.settings.to_struct()
            for p in range(3):
                m.phase[p] = self._fields(dev, _rotate(idx, p))
        self._members = members  # keep the host copy alive while the handle exists
        self.handle = ctypes.c_void_p()
        tun = _capi.VgEnsembleTuning(**(tuning or DEFAULT_TUNING))
        create = self.lib.vg_ensemble_create_f64 if f64 else self.lib.vg_ensemble_create_f32split
        _capi.check(create(members, len(self.states), ctypes.byref(tun), ctypes.byref(self.handle)),
                    "vg_ensemble_create")
        self.tuning = dict(tuning or DEFAULT_TUNING)
        self.phase = 0
        self.steps_taken = 0
        self._graphs = {}

    def _fields(self, dev, idx):
        v = dev.variables
        _, tau, taup1 = idx
        lvl = lambda t, n: t[..., n].data_ptr()  # noqa: E731
        return self._fields_t(lvl(v.temp, tau), lvl(v.temp, taup1), lvl(v.salt, tau), lvl(v.salt, taup1),
                              v.K_iso.data_ptr(), dev.mask_bits().data_ptr(), v.kbot.data_ptr(), dev.tensor_fields(),
                              v.dtemp_iso.data_ptr(), v.dsalt_iso.data_ptr(), None, None, v.P_diss_iso.data_ptr(),
                              dev.column_order().data_ptr())

    @property
    def cells(self):
        return sum(s.nx * s.ny * s.nz for s in self.states)

    def _advance(self, n):
        self.phase = (self.phase + n) % 3
        self.steps_taken += n
        for dev, idx in zip(self.states, self._start):
            v = dev.variables
            v.taum1, v.tau, v.taup1 = _rotate(idx, self.phase)

    def step(self, n=1):
        """Run ``n`` steps of every member on torch's current stream."""
        stream = torch.cuda.current_stream(self.device).cuda_stream
        for i in range(n):
            _capi.check(self.lib.vg_ensemble_step(self.handle, (self.phase + i) % 3, stream), "vg_ensemble_step")
        self._advance(n)

    def capture(self, nsteps):
        """Record ``nsteps`` steps from the current phase as a CUDA graph (cached per phase)."""
        key = (self.phase, nsteps, tuple(sorted(self.tuning.items())))
        if key not in self._graphs:
            stream = torch.cuda.Stream(self.device)
            stream.wait_stream(torch.cuda.current_stream(self.device))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(stream):
                with torch.cuda.graph(g, stream=stream):
                    s = stream.cuda_stream
                    for i in range(nsteps):
                        _capi.check(self.lib.vg_ensemble_step(self.handle, (self.phase + i) % 3, s),
                                    "vg_ensemble_step")
            torch.cuda.current_stream(self.device).wait_stream(stream)
            self._graphs[key] = g
        return self._graphs[key]

    def replay(self, nsteps):
        """Run ``nsteps`` steps by replaying the recorded graph for the current phase."""
        g = self.capture(nsteps)
        g.replay()
        self._advance(nsteps)

    def tune(self, **kw):
        t = dict(self.tuning)
        t.update(kw)
        tun = _capi.VgEnsembleTuning(**t)
        _capi.check(self.lib.vg_ensemble_tune(self.handle, ctypes.byref(tun)), "vg_ensemble_tune")
        self.tuning = t
        self._graphs.clear()

    def _time(self, steps):
        torch.cuda.synchronize(self.device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        self.step(steps)
        b.record()
        torch.cuda.synchronize(self.device)
        return a.elapsed_time(b) / steps

    def signature(self):
        return (self.precision, tuple((s.X, s.Y, s.Z) for s in self.states))

    def autotune(self, steps=2, kchunks=(0, 32, 16, -1)):
        """Pick the tiling by timing candidates on this ensemble; advances the
        members by the steps it times. Returns ``(tuning, {candidate: ms})``."""
        sig = self.signature()
        if sig in _TUNE_CACHE:
            self.tune(**_TUNE_CACHE[sig])
            return self.tuning, {}
        timings = {}
        best = dict(self.tuning)
        self.step(1)  # warm-up
        # coordinate search: each stage's knobs with the others fixed
        for knobs in (("pre_rows", "pre_kchunk"), ("flux_rows", "flux_kchunk"), ("solve_threads",)):
            space = {"pre_rows": (4, 8), "flux_rows": (4, 8), "pre_kchunk": kchunks, "flux_kchunk": kchunks,
                     "solve_threads": (32, 64)}
            for values in itertools.product(*(space[k] for k in knobs)):
                cand = dict(best)
                cand.update(dict(zip(knobs, values)))
                self.tune(**cand)
                ms = self._time(steps)
                timings[tuple(sorted(cand.items()))] = ms
            best = dict(min(timings.items(), key=lambda kv: kv[1])[0])
        self.tune(**best)
        _TUNE_CACHE[sig] = dict(best)
        return self.tuning, timings

    def close(self):
        if self.handle:
            self.lib.vg_ensemble_destroy(self.handle)
            self.handle = ctypes.c_void_p()
            self._graphs.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
