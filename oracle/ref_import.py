"""Import the reference dynamix package's own Python code -- TEST
INFRASTRUCTURE ONLY (fixture scripts, the checker tests and the CPU legs of
``bench.py``).

The correlator modules import pyopencl / silx at module level
(``dynamix/correlator/common.py:1-7``, ``dense.py:4-10``, ``event.py:3``) and
the legacy engines import numba / WXPCS / h5py / fabio (``correlator/event_y.py:1-10``,
``io/readdata.py:1-20``).  None of those packages exists here.  The modules
are satisfied with stub modules: the OpenCL / HDF5 ones are inert (an object
that is called raises), and ``numba`` maps ``jit`` / ``njit`` to the identity
decorator and ``prange`` to ``range``, so the numba functions run as the plain
Python they are written in.  No stubbed OpenCL object is called on the paths
used (``MatMulCorrelator``, ``FramesCompressor``, ``nbecorrts_q``,
``neigercompress``).

Where the package lies: ``root`` argument, else ``$DYNAMIX_REFERENCE_ROOT``,
else a ``reference`` checkout beside this repository, else the package
installed under ``baseline/_ref``.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def candidate_roots():
    out = []
    env = os.environ.get("DYNAMIX_REFERENCE_ROOT")
    if env:
        out.append(env)
    out.append(os.path.abspath(os.path.join(REPO, "..", "reference")))
    out.append(os.path.join(REPO, "baseline", "_ref"))
    return out


def find_root(root=None):
    """The first directory holding ``dynamix/correlator/dense.py``, or None."""
    for r in ([root] if root else candidate_roots()):
        if r and os.path.exists(os.path.join(r, "dynamix", "correlator", "dense.py")):
            return r
    return None


class _Inert:
    """Placeholder for classes that are only referenced, never used."""

    def __init__(self, *a, **k):
        raise RuntimeError("stub object used")


def _mod(name, **attrs):
    m = sys.modules.get(name)
    if m is None:
        m = types.ModuleType(name)
        sys.modules[name] = m
    for k, v in attrs.items():
        setattr(m, k, v)
    return m


def install_stubs():
    """Register the stub modules (only those not importable for real)."""
    def missing(name):
        if name in sys.modules:
            return False
        try:
            importlib.import_module(name)
            return False
        except Exception:
            return True

    if missing("pyopencl"):
        _mod("pyopencl.array", Array=_Inert, zeros=None, to_device=None, empty=None)
        _mod("pyopencl.tools", dtype_to_ctype=lambda d: "float")
        _mod("pyopencl", array=sys.modules["pyopencl.array"], tools=sys.modules["pyopencl.tools"],
             mem_flags=None, LocalMemory=_Inert)
    if missing("silx"):
        _mod("silx")
        _mod("silx.opencl")
        _mod("silx.opencl.common", pyopencl=sys.modules["pyopencl"], ocl=None)
        _mod("silx.opencl.processing", OpenclProcessing=_Inert, KernelContainer=_Inert)
        _mod("silx.math")
        _mod("silx.math.fft")
        _mod("silx.math.fft.fftw", FFTW=_Inert)
    if missing("numba"):
        def jit(*a, **k):
            if len(a) == 1 and callable(a[0]) and not k:
                return a[0]
            return lambda f: f
        _mod("numba", jit=jit, njit=jit, prange=range)
    for name in ("h5py", "hdf5plugin", "fabio"):
        if missing(name):
            _mod(name, File=_Inert, open=_Inert)
    if missing("psutil"):
        _mod("psutil", cpu_count=lambda logical=True: os.cpu_count())
    # the Fortran extension (setup.py builds it with numpy.distutils; no
    # Fortran compiler here): only referenced at import time on these paths
    if "dynamix.correlator.WXPCS" not in sys.modules:
        _mod("dynamix.correlator.WXPCS", fecorrt=_Inert, fecorr=_Inert, dropimgood=_Inert, eigerpix=_Inert,
             droplet3=_Inert)


def import_module(name, root=None):
    """Import ``dynamix.<...>`` module ``name`` from the reference checkout,
    with the stubs installed.  Raises ImportError when no checkout is found."""
    r = find_root(root)
    if r is None:
        raise ImportError("the dynamix reference package is not available")
    install_stubs()
    if r not in sys.path:
        sys.path.insert(0, r)
    return importlib.import_module(name)
