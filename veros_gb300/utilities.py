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
it costs a synchronisation).
"""

import numpy as np
import torch

from . import _capi


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


def solve_implicit(a, b, c, d, water_mask, edge_mask, b_edge=None, d_edge=None, validate=None):
    host = not isinstance(d, torch.Tensor)
    device = torch.device("cuda", torch.cuda.current_device()) if host else d.device
    if validate is None:
        validate = host
    shape = tuple(d.shape)
    if len(shape) < 2:
        raise ValueError("arrays need at least 2 dimensions (columns, levels)")
    for name, arr in (("a", a), ("b", b), ("c", c), ("water_mask", water_mask), ("edge_mask", edge_mask),
                      ("b_edge", b_edge), ("d_edge", d_edge)):
        if arr is not None and tuple(arr.shape) != shape:
            raise ValueError(f"{name} has shape {tuple(arr.shape)}, expected {shape}")
    if host and np.asarray(d).dtype != np.float64:
        raise ValueError("the GPU solver is float64")
    if not host and d.dtype != torch.float64:
        raise ValueError("the GPU solver is float64")

    nz = shape[-1]
    ncols = int(np.prod(shape[:-1]))
    arrs = [_as_cuda(x, torch.float64, device).reshape(ncols, nz).contiguous() for x in (a, b, c, d)]
    wm = _as_cuda(water_mask, torch.bool, device).reshape(ncols, nz).contiguous().view(torch.uint8)
    em = _as_cuda(edge_mask, torch.bool, device).reshape(ncols, nz).contiguous().view(torch.uint8)
    be = None if b_edge is None else _as_cuda(b_edge, torch.float64, device).reshape(ncols, nz).contiguous()
    de = None if d_edge is None else _as_cuda(d_edge, torch.float64, device).reshape(ncols, nz).contiguous()
    out = torch.empty((ncols, nz), dtype=torch.float64, device=device)
    bad = torch.zeros(1, dtype=torch.int32, device=device)
    lib = _capi.load()
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    st = lib.vg_solve_implicit_f64(ncols, 1, nz, nz, 0, 1, *(ptr(t) for t in arrs), ptr(wm), ptr(em), ptr(be),
                                   ptr(de), ptr(out), ptr(bad), torch.cuda.current_stream(device).cuda_stream)
    _capi.check(st, "solve_implicit")
    if validate and int(bad.item()) != 0:
        raise ValueError(f"{int(bad.item())} columns have water/edge masks not of the create_water_masks form")
    out = out.reshape(shape)
    if host:
        return out.cpu().numpy()
    return out


def solve_tridiagonal(a, b, c, d, water_mask, edge_mask, validate=None):
    return solve_implicit(a, b, c, d, water_mask, edge_mask, validate=validate)
