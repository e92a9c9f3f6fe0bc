"""Drop-ins for the column utilities of ``veros.core.utilities`` / ``operators``.

* ``create_water_masks(ks, nz)``     veros/core/utilities.py:38-48
* ``solve_implicit(a, b, c, d, water_mask, edge_mask, b_edge=None, d_edge=None)``
                                     veros/core/utilities.py:51-59
* ``solve_tridiagonal(a, b, c, d, water_mask, edge_mask)``
                                     veros/core/operators.py:60-77 (NumPy), :102-156 (JAX)

Arguments may be NumPy arrays (uploaded, solved, returned as NumPy) or CUDA
tensors (solved on torch's current stream, returned as a CUDA tensor). The
GPU solver treats each column as the reference's masks describe it (water
from ``kbot - 1`` to the top, edge at ``kbot - 1``); masks of any other form
raise ``ValueError`` when validation is on (the default for NumPy input,
where the host waits for the result anyway; opt-in for device tensors since
it costs a synchronisation: pass ``validate=True`` once per new mask set, or
a device ``bad_columns`` tensor that receives the count without a wait).

Precision follows the reference's NumPy solve: LAPACK ``dgtsv`` computes in
float64 whatever the inputs, and the solution takes the dtype of ``a``
(operators.py:64, :75-76). Float32 systems (``runtime_settings.float_type =
"float32"``) therefore solve in float64 and round the solution to float32
once, which the float32 entry point does without widening copies.
"""

import numpy as np
import torch

from . import _capi
from .state import to_host


def create_water_masks(ks, nz):
    """``(land_mask, water_mask, edge_mask)`` from kbot (1-based, 0 = land)."""
    if isinstance(ks, torch.Tensor):
        ks = ks - 1
        land = ks >= 0
        kk = torch.arange(nz, device=ks.device)[None, None, :]
        water = land[:, :, None] & (kk >= ks[:, :, None])
        edge = land[:, :, None] & (kk == ks[:, :, None])
        return land, water, edge
    ks = np.asarray(ks) - 1
    land = ks >= 0
    kk = np.arange(nz)[None, None, :]
    return land, land[:, :, None] & (kk >= ks[:, :, None]), land[:, :, None] & (kk == ks[:, :, None])


def _as_cuda(x, dtype, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype)
    return torch.from_numpy(np.ascontiguousarray(x)).to(device=device, dtype=dtype)


_FLOAT_DTYPES = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
                 torch.float64: torch.float64, torch.float32: torch.float32}


def _torch_dtype(x):
    dt = x.dtype if isinstance(x, torch.Tensor) else np.asarray(x).dtype
    if dt not in _FLOAT_DTYPES:
        raise ValueError(f"the GPU solver takes float64 or float32 systems, got {dt}")
    return _FLOAT_DTYPES[dt]


def solve_implicit(a, b, c, d, water_mask, edge_mask, b_edge=None, d_edge=None, validate=None, bad_columns=None):
    """``bad_columns``: optional int32 CUDA tensor of one element; the number of
    columns whose masks are not of the create_water_masks form is added to it
    on the device (no host synchronisation)."""
    host = not isinstance(d, torch.Tensor)
    device = torch.device("cuda", torch.cuda.current_device()) if host else d.device
    if validate is None:
        validate = host
    shape = tuple(d.shape)
    if len(shape) < 2:
        raise ValueError("arrays need at least 2 dimensions (columns, levels)")
    coefs = (("a", a), ("b", b), ("c", c), ("d", d), ("b_edge", b_edge), ("d_edge", d_edge))
    for name, arr in coefs + (("water_mask", water_mask), ("edge_mask", edge_mask)):
        if arr is not None and tuple(arr.shape) != shape:
            raise ValueError(f"{name} has shape {tuple(arr.shape)}, expected {shape}")
    out_dtype = _torch_dtype(a)  # the reference's output: np.zeros(a.shape, dtype=a.dtype)
    dtypes = {_torch_dtype(arr) for _, arr in coefs if arr is not None}
    # all float32: the float32 entry point; any float64 operand: widen to float64 (dgtsv's own copies)
    work = torch.float32 if dtypes == {torch.float32} else torch.float64

    nz = shape[-1]
    ncols = int(np.prod(shape[:-1]))
    arrs = [_as_cuda(x, work, device).reshape(ncols, nz).contiguous() for x in (a, b, c, d)]
    wm = _as_cuda(water_mask, torch.bool, device).reshape(ncols, nz).contiguous().view(torch.uint8)
    em = _as_cuda(edge_mask, torch.bool, device).reshape(ncols, nz).contiguous().view(torch.uint8)
    be = None if b_edge is None else _as_cuda(b_edge, work, device).reshape(ncols, nz).contiguous()
    de = None if d_edge is None else _as_cuda(d_edge, work, device).reshape(ncols, nz).contiguous()
    out = torch.empty((ncols, nz), dtype=work, device=device)
    if bad_columns is not None:
        if not (isinstance(bad_columns, torch.Tensor) and bad_columns.dtype == torch.int32
                and bad_columns.device == device and bad_columns.numel() >= 1):
            raise ValueError("bad_columns must be an int32 tensor on the solve's device")
        bad = bad_columns
    else:
        bad = torch.zeros(1, dtype=torch.int32, device=device)
    lib = _capi.load()
    fn = lib.vg_solve_implicit_f32 if work == torch.float32 else lib.vg_solve_implicit_f64
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    st = fn(ncols, 1, nz, nz, 0, 1, *(ptr(t) for t in arrs), ptr(wm), ptr(em), ptr(be), ptr(de), ptr(out), ptr(bad),
            torch.cuda.current_stream(device).cuda_stream)
    _capi.check(st, "solve_implicit")
    if validate and int(bad.item()) != 0:
        raise ValueError(f"{int(bad.item())} columns have water/edge masks not of the create_water_masks form")
    out = out.reshape(shape)
    if out.dtype != out_dtype:
        out = out.to(out_dtype)
    if host:
        return to_host(out.contiguous())
    return out


def solve_tridiagonal(a, b, c, d, water_mask, edge_mask, validate=None, bad_columns=None):
    return solve_implicit(a, b, c, d, water_mask, edge_mask, validate=validate, bad_columns=bad_columns)
