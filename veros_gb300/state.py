"""Device-resident state in the canonical GB300 layout.

``DeviceState`` duck-types the parts of ``veros.state.VerosState`` that the
isoneutral path touches: ``state.variables.<field>``, ``state.variables.tau``
and friends, ``state.variables.update(...)`` and ``state.settings.<name>``.
Fields are torch CUDA tensors with the reference's logical shapes
(``(X, Y, Z)``, tracers ``(X, Y, Z, 3)``, ``Ai_*`` ``(X, Y, Z, 2, 2)``) but
x-fastest storage: element (i, j, k) sits at ``i + j*pitch + k*plane`` with
the row pitch rounded up to 16 elements (16-byte aligned rows for every
element size, as the tensor-memory-access engine requires). Time levels and
tensor components are whole x-y-z blocks.
"""

import ctypes
import warnings
import weakref
from collections import namedtuple

import numpy as np
import torch

from . import _capi

PITCH_ALIGN = 16

FIELDS_3D = ("K_iso", "K_gm", "K_11", "K_22", "K_33", "dtemp_iso", "dsalt_iso", "P_diss_iso", "P_diss_skew")
# fields of the neighbouring routines (vertical mixing, streamfunction diagnostics): always float64
FIELDS_3D_F64 = ("kappaH", "dtemp_vmix", "dsalt_vmix", "B1_gm", "B2_gm")
FIELDS_2D = ("forc_temp_surface", "forc_salt_surface")
FIELDS_TIME = ("temp", "salt", "int_drhodT", "int_drhodS")
FIELDS_TENSOR = ("Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")
FIELDS_MASK = ("maskT", "maskU", "maskV", "maskW")
FIELDS_X = ("dxt", "dxu")
FIELDS_Y = ("dyt", "dyu", "cost", "cosu")
FIELDS_Z = ("dzt", "dzw", "zt")

SETTING_NAMES = ("iso_slopec", "iso_dslope", "K_iso_steep", "dt_tracer", "grav", "rho_0",
                 "eq_of_state_type", "enable_conserve_energy", "enable_skew_diffusion",
                 "enable_neutral_diffusion", "enable_cyclic_x")


def require_single_process(what):
    """Raise ``NotImplementedError`` when an imported Veros runs on several
    processes (``runtime_state.proc_num > 1``, veros/runtime.py:183): ``what``
    would need the domain decomposition's halo exchange
    (veros/core/utilities.py:18-20), which this one-GPU library does not
    perform. Without an importable Veros there is one process."""
    try:
        from veros import runtime_state

        nproc = int(runtime_state.proc_num)
    except Exception:
        return
    if nproc > 1:
        raise NotImplementedError(f"{what}: {nproc} processes; the GPU drop-in runs one process per domain")


def KernelOutput(**kwargs):
    """Same factory as veros/state.py:16-20: a namedtuple named KernelOutput."""
    try:
        from veros.state import KernelOutput as ref_factory
    except Exception:  # veros not importable: identical local factory
        return namedtuple("KernelOutput", list(kwargs.keys()))(*kwargs.values())
    return ref_factory(**kwargs)


def pitch_for(X):
    return -(-X // PITCH_ALIGN) * PITCH_ALIGN


def canonical_empty(X, Y, Z, extra=(), dtype=torch.float64, device="cuda"):
    """Uninitialised tensor of logical shape (X, Y, Z, *extra) in canonical layout."""
    P = pitch_for(X)
    store = torch.empty((*extra, Z, Y, P), dtype=dtype, device=device)
    ne = len(extra)
    perm = (ne + 2, ne + 1, ne) + tuple(range(ne))
    return store.permute(*perm)[:X]


def canonical_zeros(X, Y, Z, extra=(), dtype=torch.float64, device="cuda"):
    t = canonical_empty(X, Y, Z, extra, dtype, device)
    t.zero_()
    return t


def canonical_empty_2d(X, Y, dtype=torch.int32, device="cuda"):
    P = pitch_for(X)
    return torch.empty((Y, P), dtype=dtype, device=device).permute(1, 0)[:X]


def is_canonical(t, X, Y, Z):
    """True if ``t`` has x stride 1, y stride = pitch and z stride = pitch*Y."""
    if t.shape[:3] != (X, Y, Z) or t.stride(0) != 1:
        return False
    P = t.stride(1)
    return P >= X and (Z == 1 or t.stride(2) == P * Y)



def to_host(t):
    """A NumPy array holding the device tensor ``t``, in page-locked memory.

    The copy runs at the host link's DMA rate instead of through the driver's
    staging of pageable memory. The array is a view of a pinned tensor from
    torch's caching host allocator: while the array lives it keeps the block,
    and once it is freed the block serves the next download of that size.
    """
    if t.device.type != "cuda":
        return t.numpy()
    out = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    out.copy_(t)
    return out.numpy()

class Settings:
    """Attribute namespace of model settings."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def get(self, name, default=None):
        return self.__dict__.get(name, default)

    def to_struct(self):
        return _capi.VgIsoSettings(
            float(self.iso_slopec), float(self.iso_dslope), float(self.K_iso_steep), float(self.dt_tracer),
            float(self.grav), float(self.rho_0), int(self.eq_of_state_type), int(bool(self.enable_conserve_energy)))


class DeviceVariables:
    """Attribute container of device tensors plus the time-level indices."""

    def __init__(self):
        object.__setattr__(self, "_fields", {})
        self.tau, self.taup1, self.taum1 = 1, 2, 0

    def __getattr__(self, name):
        f = object.__getattribute__(self, "_fields")
        if name in f:
            return f[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in ("tau", "taup1", "taum1"):
            object.__setattr__(self, name, int(value))
            return
        f = object.__getattribute__(self, "_fields")
        if name in f and isinstance(value, torch.Tensor) and value is not f[name]:
            cur = f[name]
            if value.shape != cur.shape:
                raise ValueError(f"{name}: shape {tuple(value.shape)} does not match {tuple(cur.shape)}")
            cur.copy_(value)  # keep the canonical storage
            return
        f[name] = value

    def fields(self):
        return list(object.__getattribute__(self, "_fields").keys())

    def update(self, other=None, **new_fields):
        """Same contract as VerosVariables.update (veros/state.py:70-90)."""
        if other is not None:
            if new_fields:
                raise ValueError("Either other or new_fields can be given")
            if hasattr(other, "_fields"):
                new_fields = dict(zip(other._fields, other))
            elif isinstance(other, dict):
                new_fields = other
            else:
                raise TypeError(f"Cannot update from {type(other)} type")
        for k, v in new_fields.items():
            setattr(self, k, v)


PRECISIONS = ("f64", "f32split")


class DeviceState:
    """One ocean domain resident on a CUDA device in the canonical layout.

    ``precision``: ``"f64"`` (the drop-in: every field float64) or
    ``"f32split"`` (diffusivities, tensors, tendencies and dissipation stored
    as float32; tracers, grid, the slope denominators and slopes and the
    implicit vertical solve stay float64).
    """

    def __init__(self, nx, ny, nz, settings, device="cuda", precision="f64"):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {PRECISIONS}")
        self.precision = precision
        self.fdtype = torch.float64 if precision == "f64" else torch.float32
        self.nx, self.ny, self.nz = nx, ny, nz
        self.X, self.Y, self.Z = nx + 4, ny + 4, nz
        device = torch.device(device)
        if device.type == "cuda" and device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        self.settings = settings if isinstance(settings, Settings) else Settings(**settings)
        self.variables = DeviceVariables()
        self.dimensions = dict(xt=nx, xu=nx, yt=ny, yu=ny, zt=nz, zw=nz, timesteps=3, isle=1, tensor1=2, tensor2=2)
        self.pitch = pitch_for(self.X)
        self.plane = self.pitch * self.Y
        self._mask_bits = None
        self._mask_version = None

    # ---- allocation -------------------------------------------------------
    def alloc_fields(self):
        X, Y, Z, dev = self.X, self.Y, self.Z, self.device
        v = self.variables
        fd = self.fdtype
        for n in FIELDS_3D:
            setattr(v, n, canonical_zeros(X, Y, Z, dtype=fd, device=dev))
        for n in FIELDS_TIME:
            dt_ = torch.float64 if n in ("temp", "salt") else fd
            setattr(v, n, canonical_zeros(X, Y, Z, (3,), dtype=dt_, device=dev))
        for n in FIELDS_TENSOR:
            setattr(v, n, canonical_zeros(X, Y, Z, (2, 2), dtype=fd, device=dev))
        for n in FIELDS_3D_F64:
            setattr(v, n, canonical_zeros(X, Y, Z, dtype=torch.float64, device=dev))
        for n in FIELDS_2D:
            t2 = canonical_empty_2d(X, Y, dtype=torch.float64, device=dev)
            t2.zero_()
            setattr(v, n, t2)
        for n in FIELDS_MASK:
            setattr(v, n, canonical_zeros(X, Y, Z, dtype=torch.bool, device=dev))
        kb = canonical_empty_2d(X, Y, device=dev)
        kb.zero_()
        v.kbot = kb
        for n in FIELDS_X:
            setattr(v, n, torch.zeros(X, dtype=torch.float64, device=dev))
        for n in FIELDS_Y:
            setattr(v, n, torch.zeros(Y, dtype=torch.float64, device=dev))
        for n in FIELDS_Z:
            setattr(v, n, torch.zeros(Z, dtype=torch.float64, device=dev))

    @classmethod
    def from_host(cls, host, device="cuda", fields=None, precision="f64"):
        """Upload a ``synthetic.HostState`` or a NumPy ``VerosState``."""
        if hasattr(host, "variables"):  # a VerosState
            vs = host.variables
            nx, ny, nz = host.settings.nx, host.settings.ny, host.settings.nz
            settings = {n: getattr(host.settings, n) for n in SETTING_NAMES if hasattr(host.settings, n)}
            get = lambda n: getattr(vs, n, None)  # noqa: E731
            taus = (vs.tau, vs.taup1, vs.taum1)
        else:
            nx, ny, nz = host.nx, host.ny, host.nz
            settings = {n: host.settings[n] for n in SETTING_NAMES if n in host.settings}
            get = lambda n: host.arrays.get(n)  # noqa: E731
            taus = (host.tau, host.taup1, host.taum1)
        st = cls(nx, ny, nz, settings, device=device, precision=precision)
        st.alloc_fields()
        v = st.variables
        v.tau, v.taup1, v.taum1 = (int(t) for t in taus)
        for n in v.fields():
            if fields is not None and n not in fields:
                continue
            arr = get(n)
            if arr is None:
                continue
            st.upload(n, np.asarray(arr))
        return st

    # bytes moved by upload() / download() in this process (host <-> device)
    transfer_bytes = {"h2d": 0, "d2h": 0}

    def upload(self, name, arr):
        dst = getattr(self.variables, name)
        src = np.ascontiguousarray(arr)
        with warnings.catch_warnings():  # read-only host arrays (the NumPy backend's) are only read here
            warnings.simplefilter("ignore", UserWarning)
            src = torch.from_numpy(src)
        if src.dtype != dst.dtype:
            src = src.to(dst.dtype)
        dst.copy_(src, non_blocking=False)
        DeviceState.transfer_bytes["h2d"] += src.numel() * src.element_size()
        if name in FIELDS_MASK:
            self._mask_version = None

    def download(self, name):
        t = getattr(self.variables, name)
        if isinstance(t, torch.Tensor):
            DeviceState.transfer_bytes["d2h"] += t.numel() * t.element_size()
            # the reference layout (C order of the logical shape) formed on the device, then one copy
            return to_host(t.detach().contiguous())
        return t

    # ---- derived device views --------------------------------------------
    def domain(self):
        return _capi.VgDomain(self.X, self.Y, self.Z, self.pitch, self.plane)

    def grid(self):
        v = self.variables
        return _capi.VgGrid(*(getattr(v, n).data_ptr() for n in ("dxt", "dxu", "dyt", "dyu", "cost", "cosu",
                                                                   "dzt", "dzw", "zt")))

    def mask_bits(self, stream=None):
        """Packed T/U/V/W mask bytes; rebuilt whenever a mask tensor changed."""
        v = self.variables
        version = tuple((getattr(v, n).data_ptr(), getattr(v, n)._version) for n in FIELDS_MASK)
        if self._mask_bits is None or self._mask_version != version:
            if self._mask_bits is None:
                self._mask_bits = canonical_empty(self.X, self.Y, self.Z, dtype=torch.uint8, device=self.device)
            lib = _capi.load()
            dom = self.domain()
            s = stream if stream is not None else torch.cuda.current_stream(self.device).cuda_stream
            _capi.check(lib.vg_pack_masks(dom, *(getattr(v, n).data_ptr() for n in FIELDS_MASK),
                                          self._mask_bits.data_ptr(), s), "vg_pack_masks")
            self._mask_version = version
        return self._mask_bits

    def step_shares(self, stream=None):
        """Work shares of the step's pre and flux kernels for these masks on
        this device (vg_isoneutral_step_shares): two int64 device tensors of
        CTA starts, or None for a kernel that runs one CTA per tile. Cached
        per mask version; only the distribution of the work depends on them."""
        bits = self.mask_bits(stream)
        key = (self._mask_version, self.precision, str(self.device))
        if getattr(self, "_shares_key", None) != key:
            lib = _capi.load()
            dom = self.domain()
            prec = 0 if self.precision == "f64" else 1
            n_pre, n_flux, nbytes = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
            _capi.check(lib.vg_isoneutral_step_shares_size(dom, prec, ctypes.byref(n_pre), ctypes.byref(n_flux),
                                                           ctypes.byref(nbytes)), "vg_isoneutral_step_shares_size")
            mk = lambda n: torch.empty(n + 1, dtype=torch.int64, device=self.device) if n > 0 else None  # noqa: E731
            pre, flux = mk(n_pre.value), mk(n_flux.value)
            if pre is not None or flux is not None:
                scratch = torch.empty(max(1, nbytes.value // 8), dtype=torch.float64, device=self.device)
                s = stream if stream is not None else torch.cuda.current_stream(self.device).cuda_stream
                ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
                _capi.check(lib.vg_isoneutral_step_shares(dom, prec, bits.data_ptr(), ptr(pre), ptr(flux),
                                                          scratch.data_ptr(), nbytes.value, s),
                            "vg_isoneutral_step_shares")
            self._shares = (pre, flux)
            self._shares_key = key
        return self._shares

    def column_order(self):
        """Interior columns, as indices (i-2) + (j-2)*(X-4), deepest first
        (land last): the order in which the implicit solve takes them, so that
        the lanes of a warp walk columns of similar length. Cached per kbot."""
        kb = self.variables.kbot
        key = (kb.data_ptr(), kb._version)
        if getattr(self, "_order_key", None) != key:
            inner = kb[2:-2, 2:-2].to(torch.int64)
            depth = torch.where(inner > 0, self.Z - (inner - 1), torch.zeros_like(inner))
            flat = depth.t().reshape(-1)  # index (i-2) + (j-2)*(X-4)
            self._column_order = torch.argsort(-flat, stable=True).to(torch.int32).contiguous()
            self._order_key = key
        return self._column_order

    def tensor_fields(self):
        v = self.variables
        ai = v.Ai_ez
        for n in FIELDS_TENSOR + ("K_11", "K_22", "K_33"):
            t = getattr(v, n)
            want = torch.float64 if n in ("temp", "salt") + FIELDS_3D_F64 else self.fdtype
            if t.dtype != want:
                raise ValueError(f"{n}: dtype {t.dtype} but the state's precision needs {want}")
            if n in FIELDS_TENSOR and t.stride()[3:] != ai.stride()[3:]:
                raise ValueError(f"{n}: component strides {t.stride()[3:]} differ from Ai_ez {ai.stride()[3:]}")
        cls = _capi.VgTensorFields if self.precision == "f64" else _capi.VgTensorFieldsF32
        return cls(v.K_11.data_ptr(), v.K_22.data_ptr(), v.K_33.data_ptr(), v.Ai_ez.data_ptr(),
                                    v.Ai_nz.data_ptr(), v.Ai_bx.data_ptr(), v.Ai_by.data_ptr(),
                                    ai.stride(3), ai.stride(4))

    def check_layout(self, names):
        v = self.variables
        for n in names:
            t = getattr(v, n)
            if not t.is_cuda or t.device != self.device:
                raise ValueError(f"{n} is not on {self.device}")
            want = torch.float64 if n in ("temp", "salt") + FIELDS_3D_F64 else self.fdtype
            if t.dtype != want:
                raise ValueError(f"{n}: dtype {t.dtype} but the state's precision needs {want}")
            if not is_canonical(t, self.X, self.Y, self.Z) or t.stride(1) != self.pitch:
                raise ValueError(f"{n}: strides {t.stride()} are not the canonical layout (pitch {self.pitch})")

    def to_host_dict(self, names=None):
        names = names or self.variables.fields()
        return {n: self.download(n) for n in names}


# ---- device mirrors for the drop-ins' host-array path ------------------------
#
# A plugin-installed NumPy-backend Veros hands the drop-ins a VerosState of
# host arrays on every call. Uploading every field a call reads, every call,
# would move the whole state over the host link each time, although most of
# it has not changed since the previous call: the grid and masks never change,
# and the tensors and tracers a call reads are usually the very arrays an
# earlier drop-in call returned. The NumPy backend never modifies a state
# array in place: its update() works on a copy (veros/core/operators.py:19-45)
# and setattr stores the array it is given (veros/state.py:219-243). So a
# device field can stand for a host array as long as that array object is
# alive and read-only: the drop-ins return read-only arrays (as the NumPy
# backend allocates its own, veros/variables.py:941) and remember them, and a
# call uploads a field only when the state holds a different or writeable
# array. One mirror per domain shape and device is kept for the process.

_MIRRORS = {}


def host_mirror(host, fields, precision="f64", device=None):
    """The device mirror of a NumPy-backend VerosState with ``fields`` current.

    Fields whose host array is the read-only array last transferred for them
    are not uploaded again. The mirror's settings and time-level indices are
    the state's."""
    vs = host.variables
    s = host.settings
    nx, ny, nz = int(s.nx), int(s.ny), int(s.nz)
    device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    key = (nx, ny, nz, precision, str(device))
    dev = _MIRRORS.get(key)
    settings = {n: getattr(s, n) for n in SETTING_NAMES if hasattr(s, n)}
    if dev is None:
        dev = DeviceState(nx, ny, nz, settings, device=device, precision=precision)
        dev.alloc_fields()
        dev._host_src = {}
        _MIRRORS[key] = dev
    dev.settings = Settings(**settings)
    v = dev.variables
    v.tau, v.taup1, v.taum1 = int(vs.tau), int(vs.taup1), int(vs.taum1)
    for n in fields:
        try:
            arr = getattr(vs, n)
        except (AttributeError, RuntimeError):  # absent, or inactive in this configuration
            continue
        if arr is None or n not in v.fields():
            continue
        ref = dev._host_src.get(n)
        if ref is not None and ref() is arr and isinstance(arr, np.ndarray) and not arr.flags.writeable:
            continue  # the device field holds this very array
        dev.upload(n, np.asarray(arr))
        keep = isinstance(arr, np.ndarray) and not arr.flags.writeable
        dev._host_src[n] = weakref.ref(arr) if keep else None
    return dev


def mirror_written(dev, names):
    """Fields a kernel wrote no longer stand for any host array."""
    for n in names:
        dev._host_src[n] = None


def mirror_download(dev, name):
    """A read-only host copy of a device field, remembered as its host array."""
    arr = dev.download(name)
    arr.flags.writeable = False
    dev._host_src[name] = weakref.ref(arr)
    return arr


def release_host_mirrors():
    """Free the device mirrors of the host-array path."""
    _MIRRORS.clear()
