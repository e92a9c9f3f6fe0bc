"""Rollouts of the isoneutral step on a :class:`DeviceState`.

One step is the caller-side sequence of veros/core/thermodynamics.py:226-241
(zero advection) and :425-432, followed by the time-level rotation of
veros/veros.py:321-322; see ``vg_isoneutral_step_f64`` in
``include/veros_gb300.h``. The whole step is one C call, so a rollout can be
captured in a CUDA graph: ``capture(n)`` records ``n`` steps (the rotation of
time levels is a pointer permutation with period 3, so graphs are recorded
for each of the three phases and replayed in turn).
"""

import ctypes

import torch

from . import _capi


class IsoneutralStepper:
    def __init__(self, dev):
        self.dev = dev
        self.lib = _capi.load()
        nbytes = self.lib.vg_isoneutral_diffusion_pair_scratch_bytes(dev.domain())
        self.scratch = torch.empty(nbytes // 8, dtype=torch.float64, device=dev.device)
        self._graphs = {}

    def _fields(self):
        dev, v = self.dev, self.dev.variables
        lvl = lambda t, n: t[..., n].data_ptr()  # noqa: E731
        energy = bool(dev.settings.enable_conserve_energy)
        dev.check_layout(("temp", "salt", "K_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by",
                          "dtemp_iso", "dsalt_iso", "P_diss_iso", "int_drhodT", "int_drhodS"))
        cls = _capi.VgStepFields if dev.precision == "f64" else _capi.VgStepFieldsF32
        pre_sh, flux_sh = dev.step_shares()
        ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        nshares = lambda t: 0 if t is None else t.numel() - 1  # noqa: E731
        return cls(
            lvl(v.temp, v.tau), lvl(v.temp, v.taup1), lvl(v.salt, v.tau), lvl(v.salt, v.taup1), v.K_iso.data_ptr(),
            dev.mask_bits().data_ptr(), v.kbot.data_ptr(), dev.tensor_fields(), v.dtemp_iso.data_ptr(),
            v.dsalt_iso.data_ptr(), lvl(v.int_drhodT, v.tau) if energy else None,
            lvl(v.int_drhodS, v.tau) if energy else None, v.P_diss_iso.data_ptr(), dev.column_order().data_ptr(),
            ptr(pre_sh), ptr(flux_sh), nshares(pre_sh), nshares(flux_sh))

    def _fn(self, name):
        suffix = "_f64" if self.dev.precision == "f64" else "_f32split"
        return getattr(self.lib, name + suffix)

    def _launch(self, stream):
        dev = self.dev
        st = self._fn("vg_isoneutral_step")(dev.domain(), dev.grid(), dev.settings.to_struct(), self._fields(),
                                            self.scratch.data_ptr(), self.scratch.numel() * 8, stream)
        _capi.check(st, "isoneutral step")

    def _rotate(self):
        v = self.dev.variables
        v.taum1, v.tau, v.taup1 = v.tau, v.taup1, v.taum1

    def step(self, n=1):
        """Run ``n`` steps eagerly on torch's current stream (one C call each)."""
        stream = torch.cuda.current_stream(self.dev.device).cuda_stream
        for _ in range(n):
            self._launch(stream)
            self._rotate()

    def step_stages(self, events=None):
        """One step as three C calls, the stages of ``vg_isoneutral_step_*``:
        the rim's preparation, pre, and diffusion of temp and salt (with the
        interior's preparation fused in). The same kernels as ``step``.

        ``events``: optional list of 4 ``torch.cuda.Event`` recorded on the
        current stream before, between and after the stages.
        """
        dev = self.dev
        stream_obj = torch.cuda.current_stream(dev.device)
        stream = stream_obj.cuda_stream
        f = self._fields()
        dom, grid, sett = dev.domain(), dev.grid(), dev.settings.to_struct()
        nbytes = self.scratch.numel() * 8
        fn = self._fn("vg_isoneutral_step_stage")
        for stage in range(3):
            if events:
                events[stage].record(stream_obj)
            _capi.check(fn(dom, grid, sett, f, self.scratch.data_ptr(), nbytes, stage, stream),
                        ("step rim", "pre", "diffusion")[stage])
        if events:
            events[3].record(stream_obj)
        self._rotate()

    def step_unfused(self):
        """One step as a separate preparation of every cell, pre and the
        temp+salt diffusion (no fused preparation): the same results as
        ``step``, bit for bit, at one extra pass over the tracer fields."""
        dev = self.dev
        stream = torch.cuda.current_stream(dev.device).cuda_stream
        f = self._fields()
        dom, grid, sett = dev.domain(), dev.grid(), dev.settings.to_struct()
        _capi.check(self._fn("vg_isoneutral_step_prepare")(dom, f, stream), "step prepare")
        _capi.check(self._fn("vg_isoneutral_pre")(dom, grid, sett, f.temp_tau, f.salt_tau, f.K_iso, f.mask_bits,
                                                  f.ten, stream), "pre")
        targs = _capi.VgTracerArgs if dev.precision == "f64" else _capi.VgTracerArgsF32
        trT = targs(f.temp_tau, f.temp_taup1, f.dtemp_iso, f.int_drhodT_tau, f.P_diss_iso)
        trS = targs(f.salt_tau, f.salt_taup1, f.dsalt_iso, f.int_drhodS_tau, f.P_diss_iso)
        _capi.check(self._fn("vg_isoneutral_diffusion_pair_ordered")(dom, grid, sett, f.ten, f.K_iso, f.mask_bits,
                                                                     f.kbot, trT, trS, f.column_order,
                                                                     self.scratch.data_ptr(),
                                                                     self.scratch.numel() * 8, stream),
                    "diffusion")
        self._rotate()

    def step_host(self, temp_tau, salt_tau, out_temp, out_salt, out_dtemp, out_dsalt, staging=None):
        """One step from and to host buffers in the reference layout.

        ``temp_tau``/``salt_tau``: (X, Y, Z) float64 CPU tensors (pinned for
        asynchronous copies) holding the current level; the new level and the
        tendencies ``dtemp_iso``/``dsalt_iso`` land in the ``out_*`` CPU tensors.
        Copies and kernels are enqueued on the current stream; the host waits
        only for the final device-to-host copies.
        """
        v = self.dev.variables
        shape = (self.dev.X, self.dev.Y, self.dev.Z)
        if staging is None:
            staging = torch.empty((6, *shape), dtype=torch.float64, device=self.dev.device)
        stream = torch.cuda.current_stream(self.dev.device).cuda_stream
        staging[0].copy_(temp_tau, non_blocking=True)
        staging[1].copy_(salt_tau, non_blocking=True)
        _to_canonical(self.dev, staging[:2], [v.temp[..., v.tau], v.salt[..., v.tau]], stream)
        self.step(1)
        new = v.tau  # the level just written, after the rotation
        _from_canonical(self.dev, [v.temp[..., new], v.salt[..., new], v.dtemp_iso, v.dsalt_iso], staging[2:6],
                        stream)
        out_temp.copy_(staging[2], non_blocking=True)
        out_salt.copy_(staging[3], non_blocking=True)
        out_dtemp.copy_(staging[4], non_blocking=True)
        out_dsalt.copy_(staging[5], non_blocking=True)
        torch.cuda.current_stream(self.dev.device).synchronize()

    def pipeline(self):
        """A :class:`HostPipeline` of this stepper (independent host batches, copies overlapped)."""
        return HostPipeline(self)

    def launches_per_step(self):
        """Kernels of this library one step enqueues: prepare, pre, one flux
        kernel for temp and salt, one shared implicit solve and, with the
        energy branch, one energy kernel for both tracers."""
        return 1 + 1 + 1 + 1 + (1 if self.dev.settings.enable_conserve_energy else 0)


def convert_layout(dev, to_canonical, src, dst, stream):
    """FP64 fields between the reference's (X, Y, Z) C-order layout and the
    state's canonical layout in one launch (vg_layout_*_canonical_f64); ``src``
    and ``dst`` are equal-length lists of device tensors (views of the right
    layout). Returns False, leaving the copies to the caller, when a field is
    not FP64."""
    if any(t.dtype != torch.float64 for t in list(src) + list(dst)):
        return False
    n = len(src)
    ps = (ctypes.c_void_p * n)(*(t.data_ptr() for t in src))
    pd = (ctypes.c_void_p * n)(*(t.data_ptr() for t in dst))
    lib = _capi.load()
    fn = lib.vg_layout_to_canonical_f64 if to_canonical else lib.vg_layout_from_canonical_f64
    _capi.check(fn(dev.domain(), n, ps, pd, stream), "layout conversion")
    return True


def _convert(dev, to_canonical, src, dst, stream):
    """The FP64 pairs in one conversion launch, the others (FP32 tendencies
    of the split form) by torch copies."""
    pairs = list(zip(src, dst))
    f64 = [(a, b) for a, b in pairs if a.dtype == torch.float64 and b.dtype == torch.float64]
    if f64:
        convert_layout(dev, to_canonical, [a for a, _ in f64], [b for _, b in f64], stream)
    for a, b in pairs:
        if not (a.dtype == torch.float64 and b.dtype == torch.float64):
            b.copy_(a)


def _to_canonical(dev, stage, levels, stream):
    _convert(dev, True, list(stage), levels, stream)


def _from_canonical(dev, fields, stage, stream):
    _convert(dev, False, fields, list(stage), stream)


class HostPipeline:
    """Independent batches from and to host buffers with the copies overlapped.

    Each :meth:`submit` is one step of :meth:`IsoneutralStepper.step_host`:
    temp and salt at tau from pinned host tensors in the reference layout in,
    the new level and ``dtemp_iso``/``dsalt_iso`` out to pinned host tensors.
    The upload of a batch runs on its own stream while the previous batch's
    kernels run, and its download on a second stream while the next batch's
    kernels run; device staging is double buffered and guarded by events, so
    batch n's results equal those of a lone ``step_host`` call.

    :meth:`submit` returns without waiting: the input tensors must not be
    changed, nor the outputs read, before the returned event has completed
    (``event.synchronize()``) or :meth:`finish` has returned.
    """

    def __init__(self, stepper):
        self.st = stepper
        dev = stepper.dev
        self.device = dev.device
        shape = (dev.X, dev.Y, dev.Z)
        self.stage_in = [torch.empty((2, *shape), dtype=torch.float64, device=self.device) for _ in range(2)]
        self.stage_out = [torch.empty((4, *shape), dtype=torch.float64, device=self.device) for _ in range(2)]
        self.h2d = torch.cuda.Stream(self.device)
        self.d2h = torch.cuda.Stream(self.device)
        self.in_free = [None, None]  # compute done reading stage_in[b]
        self.out_free = [None, None]  # download done reading stage_out[b]
        self.n = 0

    def submit(self, temp_tau, salt_tau, out_temp, out_salt, out_dtemp, out_dsalt):
        b = self.n % 2
        v = self.st.dev.variables
        compute = torch.cuda.current_stream(self.device)
        stage_in, stage_out = self.stage_in[b], self.stage_out[b]
        with torch.cuda.stream(self.h2d):
            if self.in_free[b] is not None:
                self.h2d.wait_event(self.in_free[b])
            stage_in[0].copy_(temp_tau, non_blocking=True)
            stage_in[1].copy_(salt_tau, non_blocking=True)
            uploaded = torch.cuda.Event()
            uploaded.record(self.h2d)
        compute.wait_event(uploaded)
        _to_canonical(self.st.dev, stage_in, [v.temp[..., v.tau], v.salt[..., v.tau]], compute.cuda_stream)
        self.in_free[b] = torch.cuda.Event()
        self.in_free[b].record(compute)
        self.st.step(1)
        if self.out_free[b] is not None:
            compute.wait_event(self.out_free[b])
        new = v.tau
        _from_canonical(self.st.dev, [v.temp[..., new], v.salt[..., new], v.dtemp_iso, v.dsalt_iso], stage_out,
                        compute.cuda_stream)
        ready = torch.cuda.Event()
        ready.record(compute)
        with torch.cuda.stream(self.d2h):
            self.d2h.wait_event(ready)
            out_temp.copy_(stage_out[0], non_blocking=True)
            out_salt.copy_(stage_out[1], non_blocking=True)
            out_dtemp.copy_(stage_out[2], non_blocking=True)
            out_dsalt.copy_(stage_out[3], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.d2h)
        self.out_free[b] = done
        self.n += 1
        return done

    def finish(self):
        """Wait for every submitted batch."""
        torch.cuda.synchronize(self.device)
