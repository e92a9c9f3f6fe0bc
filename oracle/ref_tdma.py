"""Test infrastructure, not product code: the reference's own CUDA TDMA kernel
(``TridiagKernel`` of veros/core/special/cuda_tdma_kernels.cu:19-63) for an
A/B against ``vg_tdma_cuda_{double,float}`` on the same GPU.

* ``build_cubin(ref_root)`` compiles the reference source where it lies (the
  checkout given as the argument or by ``REF_ROOT``) for sm_103a into
  ``oracle/_ref/cuda_tdma_kernels.cubin`` with nvcc, nothing else; without a
  checkout it does nothing, and a cubin built earlier is used as is.
* ``build_launcher()`` compiles ``oracle/ref_tdma_launch.c`` (a driver-API
  launcher with the reference launcher's configuration) into
  ``oracle/_ref/libref_tdma_launch.so``.
* ``ReferenceTdma`` loads both into the current CUDA context and runs the
  kernel on an XLA-style buffer list.

Only the tests and bench.py's reference arm use this module.
"""

import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT, "cuda_tdma_kernels.cubin")
LAUNCHER = os.path.join(OUT, "libref_tdma_launch.so")
REF_SOURCE = os.path.join("veros", "core", "special", "cuda_tdma_kernels.cu")


def reference_root(root=None):
    """The reference checkout (the argument, else the ``REF_ROOT`` environment
    variable) if it holds the Veros sources, else None. There is no default:
    GPU machines have no checkout, and there the cubin built beforehand is used."""
    root = root or os.environ.get("REF_ROOT")
    return root if root and os.path.isdir(os.path.join(root, "veros")) else None


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else shutil.which("nvcc")


def build_cubin(ref_root=None):
    """Compile the reference kernel source for sm_103a; returns the cubin path or None."""
    root = reference_root(ref_root)
    src = os.path.join(root, REF_SOURCE) if root else None
    if src is None or not os.path.exists(src):
        return CUBIN if os.path.exists(CUBIN) else None
    nvcc = _nvcc()
    if nvcc is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= os.path.getmtime(src):
        return CUBIN
    subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", CUBIN, src],
                   check=True, capture_output=True)
    return CUBIN


def build_launcher():
    """Compile the driver-API launcher; returns its path or None without a C compiler or cuda.h."""
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    inc = os.path.join(cuda, "include")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None or not os.path.exists(os.path.join(inc, "cuda.h")):
        return None
    src = os.path.join(HERE, "ref_tdma_launch.c")
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(LAUNCHER) and os.path.getmtime(LAUNCHER) >= os.path.getmtime(src):
        return LAUNCHER
    libdirs = [os.path.join(cuda, d) for d in ("lib64/stubs", "lib64", "targets/sbsa-linux/lib/stubs",
                                                "targets/x86_64-linux/lib/stubs")]
    cmd = [cc, "-O2", "-shared", "-fPIC", "-I", inc, "-o", LAUNCHER, src]
    cmd += [f"-L{d}" for d in libdirs if os.path.isdir(d)] + ["-lcuda"]
    subprocess.run(cmd, check=True, capture_output=True)
    return LAUNCHER


def build(ref_root=None):
    """Both parts; returns (cubin, launcher), either None when it cannot be built here."""
    try:
        cubin = build_cubin(ref_root)
    except (subprocess.CalledProcessError, OSError):
        cubin = None
    try:
        launcher = build_launcher()
    except (subprocess.CalledProcessError, OSError):
        launcher = None
    return cubin, launcher


def available():
    return os.path.exists(CUBIN) and os.path.exists(LAUNCHER)


class ReferenceTdma:
    """The reference kernel in the current CUDA context (torch's primary context)."""

    def __init__(self):
        if not available():
            raise RuntimeError("reference TDMA kernel not built (oracle/_ref)")
        import torch

        torch.cuda.init()
        torch.empty(1, device="cuda")  # make the primary context current on this thread
        self.lib = ctypes.CDLL(LAUNCHER)
        self.lib.ref_tdma_load.argtypes = [ctypes.c_char_p]
        self.lib.ref_tdma_load.restype = ctypes.c_int
        self.lib.ref_tdma_launch.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int]
        self.lib.ref_tdma_launch.restype = ctypes.c_int
        st = self.lib.ref_tdma_load(CUBIN.encode())
        if st != 0:
            raise RuntimeError(f"reference TDMA cubin did not load (code {st})")

    def __call__(self, stream, buffers, num_systems, system_depth, is_double=True):
        """``buffers``: six device pointers {a, b, c, d, out, workspace} (system-fastest)."""
        arr = (ctypes.c_void_p * 6)(*buffers)
        st = self.lib.ref_tdma_launch(ctypes.c_void_p(stream), arr, num_systems, system_depth, int(is_double))
        if st != 0:
            raise RuntimeError(f"reference TDMA launch failed (code {st})")
