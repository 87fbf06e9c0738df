"""ctypes binding of the oracle (oracle/_build/libollin_oracle.so).

Test infrastructure: only tests, ``__graft_entry__.smoke`` and the CPU-baseline
leg of ``bench.py`` use it, always as the checker.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "libollin_oracle.so")

_lib = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build_oracle()
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.ollin_oracle_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(vp)]
        L.ollin_oracle_destroy.argtypes = [vp]
        L.ollin_oracle_initialize.argtypes = [vp]
        L.ollin_oracle_initial_data.argtypes = [vp]
        L.ollin_oracle_step.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        L.ollin_oracle_num_levels.argtypes = [vp]
        L.ollin_oracle_dims.argtypes = [vp, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3
        L.ollin_oracle_time.argtypes = [vp, ctypes.c_int]
        L.ollin_oracle_time.restype = ctypes.c_double
        L.ollin_oracle_get.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int]
        L.ollin_oracle_set.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int]
        L.ollin_oracle_aux.argtypes = [vp, ctypes.c_int]
        L.ollin_oracle_constraints.argtypes = [vp, ctypes.c_int]
        L.ollin_oracle_maximal_slicing.argtypes = [vp, ctypes.c_void_p]
        L.ollin_oracle_grid.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.ollin_oracle_norms.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p]
        L.ollin_oracle_interp.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p]
        L.ollin_oracle_point_updates.argtypes = [vp]
        L.ollin_oracle_point_updates.restype = ctypes.c_double
        L.ollin_oracle_last_error.restype = ctypes.c_char_p
        L.ollin_oracle_ell_stats.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
        L.ollin_oracle_set_threads.argtypes = [ctypes.c_int]
        L.ollin_oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


class Oracle:
    """One oracle evolution.  Arrays are returned as (Nr+g, Nz+g) numpy arrays
    indexed [i+g-1, j+g-1] for Fortran (i, j)."""

    def __init__(self, params):
        self.L = lib()
        self.p = params
        h = ctypes.c_void_p()
        self._check(self.L.ollin_oracle_create(ctypes.byref(params), ctypes.byref(h)))
        self.h = h

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + self.L.ollin_oracle_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ollin_oracle_destroy(self.h)
            self.h = None

    def initial_data(self):
        self._check(self.L.ollin_oracle_initial_data(self.h))

    def initialize(self):
        self._check(self.L.ollin_oracle_initialize(self.h))

    def step(self):
        t = ctypes.c_double()
        self._check(self.L.ollin_oracle_step(self.h, ctypes.byref(t)))
        return t.value

    def levels(self):
        return range(self.L.ollin_oracle_num_levels(self.h))

    def dims(self, level):
        nr, nz, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self.L.ollin_oracle_dims(self.h, level, ctypes.byref(nr), ctypes.byref(nz), ctypes.byref(g)))
        return nr.value, nz.value, g.value

    def time(self, level):
        return self.L.ollin_oracle_time(self.h, level)

    def get(self, level, name):
        nr, nz, g = self.dims(level)
        a = np.zeros((nz + g, nr + g), dtype=np.float64)  # C-order rows = j
        self._check(self.L.ollin_oracle_get(self.h, level, name.encode(), a.ctypes.data, nr + g))
        return np.ascontiguousarray(a.T)

    def set(self, level, name, arr):
        nr, nz, g = self.dims(level)
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).T)
        self._check(self.L.ollin_oracle_set(self.h, level, name.encode(), a.ctypes.data, nr + g))

    def grid(self, gid):
        """(box, level) of grid ``gid``."""
        b, l = ctypes.c_int(), ctypes.c_int()
        if self.L.ollin_oracle_grid(self.h, gid, ctypes.byref(b), ctypes.byref(l)):
            raise RuntimeError("oracle: bad grid %d" % gid)
        return b.value, l.value

    def aux(self, level):
        self._check(self.L.ollin_oracle_aux(self.h, level))

    def constraints(self, level):
        self._check(self.L.ollin_oracle_constraints(self.h, level))

    def maximal_slicing(self, va_max=None):
        """maximalslicing.f90 on every level; va_max = (r, z) maxima of the
        slicing speeds of the last analysis, or None."""
        if va_max is None:
            self._check(self.L.ollin_oracle_maximal_slicing(self.h, None))
        else:
            v = np.asarray(va_max, dtype=np.float64)
            self._check(self.L.ollin_oracle_maximal_slicing(self.h, v.ctypes.data))

    def norms(self, level, name):
        out = np.zeros(5)
        self._check(self.L.ollin_oracle_norms(self.h, level, name.encode(), out.ctypes.data))
        return out

    def interp(self, level, name, r, z):
        """``name`` at the points (r, z) of grid ``level`` (interp.f90)."""
        r = np.asarray(r, dtype=np.float64).ravel()
        z = np.asarray(z, dtype=np.float64).ravel()
        rz = np.ascontiguousarray(np.stack([r, z], axis=1))
        out = np.zeros(len(r))
        self._check(self.L.ollin_oracle_interp(self.h, level, name.encode(), rz.ctypes.data, len(r),
                                               out.ctypes.data))
        return out

    def point_updates(self):
        return self.L.ollin_oracle_point_updates(self.h)


def ell_stats():
    """(coarse-phase iterations, all-level iterations, phases, final residual)
    of the last elliptic solve of the oracle on this thread."""
    steps = (ctypes.c_int * 2)()
    gres = ctypes.c_double()
    phases = lib().ollin_oracle_ell_stats(steps, ctypes.byref(gres))
    return steps[0], steps[1], phases, gres.value


def set_threads(n):
    """OpenMP threads of the oracle from now on."""
    lib().ollin_oracle_set_threads(int(n))
    return lib().ollin_oracle_max_threads()
