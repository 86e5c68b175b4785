"""Build recipe of the C oracle (test infrastructure, never linked by the product).

``build()`` compiles ``oracle/g2_oracle.c`` with the host compiler into
``oracle/_build/libg2_oracle.so`` (git-ignored), and ``load()`` binds it with
ctypes.  Portable C (POSIX threads only), so the same recipe runs on x86-64
and on Arm hosts.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "g2_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libg2_oracle.so")

_lib = None


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-pthread", SRC, "-o", tmp],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        p, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        lib.g2o_event_pairsum.argtypes = [p, p, ctypes.c_int, p, p, p, i64, i32, i32, p, p, ctypes.c_int]
        lib.g2o_event_pairsum.restype = ctypes.c_int
        _lib = lib
    return _lib


# ---- the reference's own event kernels, compiled as C (only where the
# reference sources are present; the outputs stay in oracle/_ref/)


def reference_root():
    """Where the dynamix sources are: ``$DYNAMIX_REFERENCE_ROOT`` when set, else
    a ``reference`` checkout beside this repository, else the package
    installed under ``baseline/_ref`` (see ``oracle/ref_import.py``)."""
    from oracle.ref_import import candidate_roots, find_root
    return find_root() or candidate_roots()[0]


REF_ROOT = reference_root()
REF_OPENCL = os.path.join(REF_ROOT, "dynamix", "resources", "opencl")
REF_CL = os.path.join(REF_OPENCL, "evtcorrelator.cl")
REF_DIR = os.path.join(HERE, "_ref")
REF_MAX_EVT_COUNT = 4096
REF_DTYPES = {"u8": "uchar", "u16": "ushort"}

_ref = {}


def ref_lib_path(tag):
    return os.path.join(REF_DIR, "libevtcorrelator_%s.so" % tag)


def build_ref(force=False):
    """Compile evtcorrelator.cl (event_correlator + normalize_correlation) with
    opencl_shim.h and ref_driver.c, once per event dtype.  Returns the list of
    built libraries, or [] when the reference sources are absent."""
    if not os.path.exists(REF_CL):
        return []
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(HERE, "opencl_shim.h")
    drv = os.path.join(HERE, "ref_driver.c")
    out = []
    for tag, ctype in REF_DTYPES.items():
        lib = ref_lib_path(tag)
        newest = max(os.path.getmtime(p) for p in (REF_CL, shim, drv))
        if force or not os.path.exists(lib) or os.path.getmtime(lib) < newest:
            defs = ["-DIMAGE_WIDTH=g2r_image_width", "-DNUM_BINS=g2r_num_bins",
                    "-DMAX_EVT_COUNT=%d" % REF_MAX_EVT_COUNT, "-DDTYPE=%s" % ctype]
            tmp = lib + ".%d.tmp" % os.getpid()
            subprocess.run(["gcc", "-O2", "-std=gnu11", "-w", "-fPIC", "-shared", "-pthread", "-I", HERE] + defs +
                           ["-include", shim, "-x", "c", REF_CL, "-x", "none", drv, "-o", tmp], check=True)
            os.replace(tmp, lib)
        out.append(lib)
    return out


def load_ref(tag):
    """ctypes handle of the reference's event kernels for data dtype ``tag``
    ('u8' or 'u16'), or None when they cannot be built here."""
    if tag not in _ref:
        libs = build_ref()
        if not libs:
            return None
        lib = ctypes.CDLL(ref_lib_path(tag))
        p, i = ctypes.c_void_p, ctypes.c_int
        lib.g2r_event_correlate.argtypes = [p, p, p, p, p, p, p, p, i, i, i, i, i, i]
        lib.g2r_event_correlate.restype = i
        lib.g2r_max_evt_count.restype = i
        _ref[tag] = lib
    return _ref[tag]


# ---- the reference's dense and CSR kernels (work-group barriers and local
# memory), compiled as C with opencl_wg_shim.h and run by ref_wg_driver.c
REF_WG_FILES = {"dense": "densecorrelator.cl", "csr": "correlator.cl"}


def build_ref_wg(kind, defines, force=False):
    """Compile the reference's ``densecorrelator.cl`` (kind "dense") or
    ``correlator.cl`` (kind "csr") with the compile-time parameters the
    reference passes to the OpenCL compiler (``defines``: name -> value, e.g.
    IMAGE_WIDTH, NUM_BINS, DTYPE), into ``oracle/_ref/``.  Returns the library
    path, or None when the reference sources are absent."""
    cl = os.path.join(REF_OPENCL, REF_WG_FILES[kind])
    if not os.path.exists(cl):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(HERE, "opencl_wg_shim.h")
    drv = os.path.join(HERE, "ref_wg_driver.c")
    tag = "_".join("%s%s" % (k, str(v).replace(" ", "")) for k, v in sorted(defines.items()))
    lib = os.path.join(REF_DIR, "lib%s_%s.so" % (kind, tag))
    newest = max(os.path.getmtime(p) for p in (cl, shim, drv))
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        defs = ["-D%s=%s" % (k, v) for k, v in sorted(defines.items())]
        defs.append("-DG2W_DENSE" if kind == "dense" else "-DG2W_CSR")
        tmp = lib + ".%d.tmp" % os.getpid()
        subprocess.run(["gcc", "-O1", "-std=gnu11", "-w", "-fPIC", "-shared", "-pthread", "-fsigned-char", "-I", HERE]
                       + defs + ["-include", shim, "-x", "c", cl, "-x", "none", drv, "-o", tmp], check=True)
        os.replace(tmp, lib)
    return lib


def load_ref_wg(kind, defines):
    """ctypes handle of :func:`build_ref_wg`'s library, or None."""
    path = build_ref_wg(kind, defines)
    if path is None:
        return None
    lib = ctypes.CDLL(path)
    p, i = ctypes.c_void_p, ctypes.c_int
    if kind == "dense":
        lib.g2w_dense_sums.argtypes = [p, p, p, i, i]
        lib.g2w_dense_corr1d.argtypes = [p, p, i, i]
        lib.g2w_dense_numerator.argtypes = [p, p, p, p, i, i, i]
    else:
        lib.g2w_csr_sums.argtypes = [p, p, p, i]
        lib.g2w_csr_correlate.argtypes = [p, p, p, p, p, p, p, i, i]
    return lib
