"""Differentiable FP64 isoneutral steps (torch.autograd) with hand-written adjoints.

Veros itself has no derivative of this path. Here one step
``(temp, salt, K_iso) -> (temp_new, salt_new)`` is the FP64 step of
``vg_isoneutral_step_f64`` (veros/core/thermodynamics.py:226-241 with zero
advection, then :425-432) wrapped in a ``torch.autograd.Function`` whose
backward is ``vg_isoneutral_step_adjoint_f64``: the transposed flux stencils,
the slope and taper derivatives and the reverse Thomas solve of the
transposed tridiagonal system, all in CUDA.

Checkpointing is per step: the autograd graph of an n-step rollout keeps the
tracer levels T_0..T_n and S_0..S_n (the steps' own inputs and outputs, no
copies) and nothing else; the backward of each step recomputes that step's
diffusion tensor from its checkpoint. Memory is 2 (n + 1) tracer fields plus
one shared workspace.

Usage::

    model = IsoneutralAdjoint(dev)            # grid, masks, kbot, settings of a DeviceState
    T0, S0, K = model.field(t0), model.field(s0), model.field(k_iso)   # canonical leaves
    T0.requires_grad_(); K.requires_grad_()
    T, S = model.rollout(T0, S0, K, 8)
    loss = ((T - target) ** 2 * wet).sum()
    loss.backward()                           # T0.grad, K.grad
"""

import torch

from . import _capi
from .state import canonical_empty, is_canonical


class IsoneutralAdjoint:
    def __init__(self, dev):
        if dev.precision != "f64":
            raise ValueError("the adjoint is FP64: build the DeviceState with precision='f64'")
        self.dev = dev
        self.lib = _capi.load()
        self.X, self.Y, self.Z = dev.X, dev.Y, dev.Z
        dom = dev.domain()
        self._dom = dom
        self._grid = dev.grid()
        self._set = dev.settings.to_struct()
        self._set.enable_conserve_energy = 0  # the energy branch does not change the tracers
        nbytes = self.lib.vg_isoneutral_step_adjoint_scratch_bytes(dom)
        if nbytes == 0:
            raise ValueError(_capi.last_error())
        # zeroed once: the tensor sub-ranges the pre kernel never writes stay 0
        self._work = torch.zeros(nbytes // 8, dtype=torch.float64, device=dev.device)
        pair = self.lib.vg_isoneutral_diffusion_pair_scratch_bytes(dom)
        self._pair = torch.empty(max(pair, 8) // 8, dtype=torch.float64, device=dev.device)
        self._diag = [self.empty() for _ in range(2)]  # dtemp_iso, dsalt_iso of the forward
        F = dev.plane * dev.Z
        base = self._work.data_ptr()
        ptr = lambda n: base + n * F * 8  # noqa: E731
        # the forward's tensor lives in the first 19 fields of the adjoint workspace
        self._ten = _capi.VgTensorFields(ptr(0), ptr(1), ptr(2), ptr(3), ptr(7), ptr(11), ptr(15), 2 * F, F)
        self._zeros = None

    # ---- canonical fields ---------------------------------------------------------------
    def empty(self):
        return canonical_empty(self.X, self.Y, self.Z, dtype=torch.float64, device=self.dev.device)

    def field(self, data):
        """A canonical float64 (X, Y, Z) tensor holding ``data`` (array or tensor)."""
        t = self.empty()
        t.copy_(torch.as_tensor(data, dtype=torch.float64))
        return t

    def _canonical(self, t):
        """``t`` itself if it is a canonical float64 field on this device, else a canonical copy
        (``None``: a shared zero field)."""
        if t is None:
            if self._zeros is None:
                self._zeros = self.empty().zero_()
            return self._zeros
        t = t.detach()
        if t.dtype == torch.float64 and t.device == self.dev.device and is_canonical(t, self.X, self.Y, self.Z) \
                and t.stride(1) == self.dev.pitch:
            return t
        return self.field(t)

    def _check(self, name, t):
        if t.dtype != torch.float64 or t.device != self.dev.device:
            raise ValueError(f"{name}: needs float64 on {self.dev.device}")
        if not is_canonical(t, self.X, self.Y, self.Z) or t.stride(1) != self.dev.pitch:
            raise ValueError(f"{name}: strides {tuple(t.stride())} are not the canonical layout; use model.field()")

    def _stream(self):
        return torch.cuda.current_stream(self.dev.device).cuda_stream

    # ---- raw forward / backward ------------------------------------------------------------
    def forward_step(self, T, S, K):
        """One step without autograd: returns new canonical ``(T_new, S_new)``."""
        for n, t in (("temp", T), ("salt", S), ("K_iso", K)):
            self._check(n, t)
        dev = self.dev
        T_new, S_new = self.empty(), self.empty()
        pre_sh, flux_sh = dev.step_shares()
        ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        f = _capi.VgStepFields(T.data_ptr(), T_new.data_ptr(), S.data_ptr(), S_new.data_ptr(), K.data_ptr(),
                               dev.mask_bits().data_ptr(), dev.variables.kbot.data_ptr(), self._ten,
                               self._diag[0].data_ptr(), self._diag[1].data_ptr(), None, None, None,
                               dev.column_order().data_ptr(), ptr(pre_sh), ptr(flux_sh),
                               0 if pre_sh is None else pre_sh.numel() - 1,
                               0 if flux_sh is None else flux_sh.numel() - 1)
        _capi.check(self.lib.vg_isoneutral_step_f64(self._dom, self._grid, self._set, f, self._pair.data_ptr(),
                                                    self._pair.numel() * 8, self._stream()), "isoneutral step")
        return T_new, S_new

    def backward_step(self, T, S, K, T_new, S_new, gT_new, gS_new, gK):
        """Adjoint of one step: returns ``(gT, gS)`` and adds dL/dK into ``gK``."""
        gT_new, gS_new = self._canonical(gT_new), self._canonical(gS_new)
        self._check("gK_iso", gK)
        gT, gS = self.empty(), self.empty()
        dev = self.dev
        f = _capi.VgAdjointFields(T.data_ptr(), S.data_ptr(), T_new.data_ptr(), S_new.data_ptr(), K.data_ptr(),
                                  dev.mask_bits().data_ptr(), dev.variables.kbot.data_ptr(), gT_new.data_ptr(),
                                  gS_new.data_ptr(), gT.data_ptr(), gS.data_ptr(), gK.data_ptr(),
                                  dev.column_order().data_ptr())
        _capi.check(self.lib.vg_isoneutral_step_adjoint_f64(self._dom, self._grid, self._set, f, self._work.data_ptr(),
                                                            self._work.numel() * 8, self._stream()),
                    "isoneutral step adjoint")
        return gT, gS

    # ---- autograd ---------------------------------------------------------------------------
    def step(self, T, S, K):
        """One differentiable step."""
        return _IsoneutralStep.apply(T, S, K, self)

    def rollout(self, T0, S0, K, nsteps):
        """``nsteps`` differentiable steps; returns the final ``(T, S)``."""
        T, S = T0, S0
        for _ in range(nsteps):
            T, S = self.step(T, S, K)
        return T, S

    # launches per forward and backward step (for launch accounting)
    forward_launches = 1 + 1 + 1 + 1  # rim preparation, pre, flux (temp and salt), implicit
    backward_launches = 6  # tables, pre, transposed solve, active list, slopes, gather


class _IsoneutralStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, T, S, K, model):
        # inputs in another layout are copied once into canonical storage
        T, S, K = (model._canonical(t) for t in (T, S, K))
        T_new, S_new = model.forward_step(T, S, K)
        ctx.model = model
        ctx.save_for_backward(T, S, K, T_new, S_new)
        return T_new, S_new

    @staticmethod
    def backward(ctx, gT_new, gS_new):
        T, S, K, T_new, S_new = ctx.saved_tensors
        m = ctx.model
        gK = m.empty().zero_()
        gT, gS = m.backward_step(T.detach(), S.detach(), K.detach(), T_new, S_new, gT_new, gS_new, gK)
        return gT, gS, (gK if ctx.needs_input_grad[2] else None), None
