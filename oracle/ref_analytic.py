"""The reference's own analytic Stokes solutions, compiled from the reference
tree -- TEST INFRASTRUCTURE.

``build()`` compiles ``ref_analytic.cpp`` (a C entry point of this repository)
together with the reference's ``Velic_sol*.c`` sources and its header-only
``AnalyticSol*.hpp`` wrappers, where they lie in the reference tree, into
``oracle/_ref/libref_analytic.so``.  The reference tree exists only on the
development machine; where it is absent ``available()`` is False and the tests
that use this module skip.  Only ``tests/`` import it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_TREE = os.environ.get("UW_REFERENCE_TREE", "/root/reference")
_REF = REFERENCE_TREE
_LIBUW = os.path.join(_REF, "src", "underworld", "libUnderworld")
_FNSRC = os.path.join(_LIBUW, "Underworld", "Function", "src")
_VELIC = os.path.join(_LIBUW, "Underworld", "SysTest", "AnalyticPlugins")
_OUT = os.path.join(_HERE, "_ref")
_SO = os.path.join(_OUT, "libref_analytic.so")
_SOLS = ("A", "B", "C", "Cx", "DA", "H", "Kx", "Kz")
_lib = None


def _sources():
    return [os.path.join(_VELIC, "Velic_sol%s" % s, "sol%s.c" % s) for s in _SOLS]


def build(force=False):
    """Compile the library (about ten seconds); returns its path, or None when
    the reference tree is absent."""
    if not os.path.isdir(_FNSRC):
        return None
    os.makedirs(_OUT, exist_ok=True)
    shim = os.path.join(_HERE, "ref_analytic.cpp")
    srcs = _sources() + [shim]
    if not force and os.path.exists(_SO) and all(os.path.getmtime(_SO) >= os.path.getmtime(s) for s in srcs):
        return _SO
    objs = []
    for s in _sources():
        o = os.path.join(_OUT, os.path.basename(s)[:-2] + ".o")
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-w", "-I", _LIBUW, "-c", s, "-o", o])
        objs.append(o)
    tmp = _SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-fPIC", "-shared", "-w", "-std=c++14", "-I", _LIBUW, "-I", _FNSRC,
                           shim, "-o", tmp] + objs + ["-lm"])
    os.replace(tmp, _SO)
    return _SO


def available():
    try:
        return build() is not None
    except (OSError, subprocess.CalledProcessError):
        return False


def evaluate(name, params, pts):
    """Fields of the reference's solution `name` (constructor parameters in the
    order of the Python interface) at points [n, dim]: a dict with velocity,
    pressure, stress, strainRate, viscosity and bodyforce arrays."""
    global _lib
    if _lib is None:
        if build() is None:
            raise RuntimeError("reference tree not available")
        _lib = ctypes.CDLL(_SO)
        _lib.uwref_analytic.restype = ctypes.c_int
        _lib.uwref_analytic.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long,
                                        ctypes.c_void_p]
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, dim = pts.shape
    ns = 3 if dim == 2 else 6
    stride = 2 * dim + 2 + 2 * ns
    prm = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel() if len(params) else np.zeros(1))
    out = np.zeros((n, stride))
    rc = _lib.uwref_analytic(name.encode(), prm.ctypes.data, pts.ctypes.data, n, out.ctypes.data)
    if rc != 0:
        raise RuntimeError("uwref_analytic(%s) returned %d" % (name, rc))
    o = 0
    res = {}
    for key, k in (("velocity", dim), ("pressure", 1), ("stress", ns), ("strainRate", ns), ("viscosity", 1),
                   ("bodyforce", dim)):
        res[key] = out[:, o:o + k]
        o += k
    return res
