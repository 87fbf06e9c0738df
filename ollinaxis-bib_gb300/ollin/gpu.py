"""ctypes mirror of the C ABI (include/ollin_gpu.h).

``Evolution`` follows the reference's driver (src/base/evolve.f90): create the
level hierarchy, ``initial_data`` (initial.f90), ``initialize`` (symmetries,
auxiliary quantities and Gamma-driver set-up at t=0), then ``step`` =
``call onestep(0)``.  There is no CPU fallback: every call goes to the CUDA
library, and loading fails loudly when it is missing.
"""
import ctypes
import os

import numpy as np

from . import build as _build
from .params import FIELD_ID, DERIVED_ID, Params

_lib = None

ERRORS = {1: "EINVAL", 2: "ECUDA", 3: "ENAN", 4: "ENOMEM", 5: "ESTATE", 6: "ECONV"}


class OllinError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class LevelDesc(ctypes.Structure):
    _fields_ = [("level", ctypes.c_int), ("nr", ctypes.c_int), ("nz", ctypes.c_int), ("ghost", ctypes.c_int),
                ("dr", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
                ("rmin", ctypes.c_double), ("rmax", ctypes.c_double), ("zmin", ctypes.c_double),
                ("zmax", ctypes.c_double), ("time", ctypes.c_double), ("steps", ctypes.c_int),
                ("box", ctypes.c_int), ("rbox", ctypes.c_double), ("zbox", ctypes.c_double)]


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libollin_gpu.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libollin_gpu.so has not been built: run __graft_entry__.build()")
        _build.build()
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    L.ollin_params_default.argtypes = [ctypes.c_void_p]
    L.ollin_gpu_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(vp)]
    L.ollin_gpu_destroy.argtypes = [vp]
    L.ollin_gpu_num_levels.argtypes = [vp]
    L.ollin_gpu_level_desc.argtypes = [vp, ctypes.c_int, ctypes.c_void_p]
    L.ollin_gpu_upload.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    L.ollin_gpu_download.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    L.ollin_gpu_initial_data.argtypes = [vp]
    L.ollin_gpu_initialize.argtypes = [vp]
    L.ollin_gpu_aux.argtypes = [vp, ctypes.c_int]
    L.ollin_gpu_coarse_step.argtypes = [vp, dp]
    L.ollin_gpu_norms.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    L.ollin_gpu_point_updates.argtypes = [vp]
    L.ollin_gpu_point_updates.restype = ctypes.c_double
    L.ollin_gpu_stream.argtypes = [vp]
    L.ollin_gpu_stream.restype = ctypes.c_void_p
    L.ollin_gpu_launch_count.argtypes = [vp]
    L.ollin_gpu_launch_count.restype = ctypes.c_longlong
    L.ollin_gpu_last_error.restype = ctypes.c_char_p
    L.ollin_gpu_kernel_timing.argtypes = [vp, ctypes.c_int]
    L.ollin_gpu_fp64_rate.restype = ctypes.c_double
    L.ollin_gpu_kernel_stats.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_longlong), dp]
    L.ollin_gpu_ell_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int), dp]
    L.ollin_gpu_ell_history.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.ollin_gpu_interp.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp]
    L.ollin_gpu_coords.argtypes = [vp, ctypes.c_int, vp, vp]
    L.ollin_gpu_upload_many.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp]
    L.ollin_gpu_download_many.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp]
    L.ollin_gpu_maximal_slicing.argtypes = [vp, ctypes.c_void_p]
    L.ollin_gpu_coarse_step_many.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.ollin_gpu_coarse_step_fused.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.ollin_gpu_fused_graphs.argtypes = [ctypes.c_int]
    L.ollin_gpu_coarse_step_auto.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_int)]
    L.ollin_gpu_min_lapse.argtypes = [vp, dp]
    L.ollin_gpu_step_begin.argtypes = [vp]
    L.ollin_gpu_step_end.argtypes = [vp, dp]
    sp = ctypes.POINTER(ctypes.c_size_t)
    L.ollin_gpu_footprint.argtypes = [ctypes.c_void_p, sp, sp]
    L.ollin_server_create.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(vp)]
    L.ollin_server_destroy.argtypes = [vp]
    L.ollin_server_submit.argtypes = [vp, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_double]
    L.ollin_server_tick.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.ollin_server_poll.argtypes = [vp, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.ollin_server_usage.argtypes = [vp, sp, sp]
    L.ollin_server_last_error.restype = ctypes.c_char_p
    L.ollin_server_set_graphs.argtypes = [vp, ctypes.c_int]
    L.ollin_server_set_fused.argtypes = [vp, ctypes.c_int]
    L.ollin_gpu_step_graphs.argtypes = [vp, ctypes.c_int, ctypes.c_void_p]
    L.ollin_gpu_step_chaining.argtypes = [vp, ctypes.c_int]
    L.ollin_gpu_download_slot.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    L.ollin_gpu_upload_slot.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    L.ollin_gpu_get_clocks.argtypes = [vp, ctypes.c_int, dp]
    L.ollin_gpu_resume.argtypes = [vp]
    L.ollin_gpu_set_clocks.argtypes = [vp, ctypes.c_int, dp]
    _lib = L
    return L


def field_id(name):
    if name in FIELD_ID:
        return FIELD_ID[name]
    if name in ("KTH",):
        return 10
    if name in DERIVED_ID:
        return DERIVED_ID[name]
    raise KeyError(name)


class Evolution:
    """One evolution on the current CUDA device."""

    def __init__(self, params):
        self.L = load()
        self.p = params
        h = ctypes.c_void_p()
        self._check(self.L.ollin_gpu_create(ctypes.byref(params), ctypes.byref(h)))
        self.h = h

    def _check(self, rc):
        if rc != 0:
            raise OllinError(rc, self.L.ollin_gpu_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.ollin_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # reference driver steps ------------------------------------------------
    def initial_data(self):
        self._check(self.L.ollin_gpu_initial_data(self.h))

    def initialize(self):
        self._check(self.L.ollin_gpu_initialize(self.h))

    def resume(self):
        """After upload_slot/set_clocks of a suspended evolution: continue it
        bit for bit (ollin_gpu_resume), instead of ``initialize``."""
        self._check(self.L.ollin_gpu_resume(self.h))

    def aux(self, level):
        self._check(self.L.ollin_gpu_aux(self.h, level))

    def step(self):
        t = ctypes.c_double()
        self._check(self.L.ollin_gpu_coarse_step(self.h, ctypes.byref(t)))
        return t.value

    # data --------------------------------------------------------------------
    def levels(self):
        return range(self.L.ollin_gpu_num_levels(self.h))

    def desc(self, level):
        d = LevelDesc()
        self._check(self.L.ollin_gpu_level_desc(self.h, level, ctypes.byref(d)))
        return d

    def grid(self, gid):
        """(box, level) of grid ``gid``."""
        d = self.desc(gid)
        return d.box, d.level

    def coords(self, level):
        """(r(1-g..Nr), z(1-g..Nz)) of a grid, as the kernels use them."""
        d = self.desc(level)
        r = np.zeros(d.nr + d.ghost)
        z = np.zeros(d.nz + d.ghost)
        self._check(self.L.ollin_gpu_coords(self.h, level, r.ctypes.data, z.ctypes.data))
        return r, z

    def download(self, level, name):
        """(Nr+g, Nz+g) array indexed [i+g-1, j+g-1] for Fortran (i, j)."""
        d = self.desc(level)
        nr, nz, g = d.nr, d.nz, d.ghost
        a = np.zeros((nz + g, nr + g), dtype=np.float64)
        self._check(self.L.ollin_gpu_download(self.h, level, field_id(name), a.ctypes.data, nr + g))
        return np.ascontiguousarray(a.T)

    def upload(self, level, name, arr):
        d = self.desc(level)
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).T)
        self._check(self.L.ollin_gpu_upload(self.h, level, field_id(name), a.ctypes.data, d.nr + d.ghost))

    # restart data (checkpoint.f90) ---------------------------------------------
    def download_slot(self, level, name, which):
        """Time level ``which`` of an evolved field: 0 the current state, 1
        the start of the level's last step, 2 the start of the step before
        (on the boundary strips: the reference's var_bound_*(..., 0) and
        (..., 1))."""
        d = self.desc(level)
        a = np.zeros((d.nz + d.ghost, d.nr + d.ghost), dtype=np.float64)
        self._check(self.L.ollin_gpu_download_slot(self.h, level, field_id(name), which, a.ctypes.data,
                                                   d.nr + d.ghost))
        return np.ascontiguousarray(a.T)

    def upload_slot(self, level, name, which, arr):
        d = self.desc(level)
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).T)
        self._check(self.L.ollin_gpu_upload_slot(self.h, level, field_id(name), which, a.ctypes.data,
                                                 d.nr + d.ghost))

    def clocks(self, level):
        """(t, t1, t2, s) of a grid."""
        out = np.zeros(4)
        self._check(self.L.ollin_gpu_get_clocks(self.h, level, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def set_clocks(self, level, clocks):
        v = np.ascontiguousarray(np.asarray(clocks, dtype=np.float64))
        self._check(self.L.ollin_gpu_set_clocks(self.h, level, v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def norms(self, level, name):
        out = np.zeros(5)
        self._check(self.L.ollin_gpu_norms(self.h, level, field_id(name), out.ctypes.data))
        return out

    def point_updates(self):
        return self.L.ollin_gpu_point_updates(self.h)

    def stream(self):
        return self.L.ollin_gpu_stream(self.h)

    def launch_count(self):
        return self.L.ollin_gpu_launch_count(self.h)

    def kernel_timing(self, enable=True):
        self._check(self.L.ollin_gpu_kernel_timing(self.h, 1 if enable else 0))

    def step_graphs(self, enable=None):
        """Turn graph-captured steps on/off (None: leave); returns
        (graphs instantiated, graph updates) so far."""
        st = (ctypes.c_longlong * 2)()
        self._check(self.L.ollin_gpu_step_graphs(self.h, -1 if enable is None else int(bool(enable)), st))
        return st[0], st[1]

    def min_lapse(self):
        out = ctypes.c_double()
        self._check(self.L.ollin_gpu_min_lapse(self.h, ctypes.byref(out)))
        return out.value

    def step_chaining(self, enable):
        """Programmatic dependent chaining of a step's kernels (on by default)."""
        self._check(self.L.ollin_gpu_step_chaining(self.h, int(bool(enable))))

    def step_begin(self):
        self._check(self.L.ollin_gpu_step_begin(self.h))

    def step_end(self):
        t = ctypes.c_double()
        self._check(self.L.ollin_gpu_step_end(self.h, ctypes.byref(t)))
        return t.value

    def maximal_slicing(self, va_max=None):
        """maximalslicing.f90 on every level (ollin_gpu_maximal_slicing);
        va_max = (r, z) maxima of the slicing speeds of the host's last
        analysis, or None."""
        if va_max is None:
            self._check(self.L.ollin_gpu_maximal_slicing(self.h, None))
        else:
            v = np.asarray(va_max, dtype=np.float64)
            self._check(self.L.ollin_gpu_maximal_slicing(self.h, v.ctypes.data))

    def ell_stats(self):
        """(coarse-phase iterations, all-level iterations, final residual) of
        the elliptic solve of ``initial_data``."""
        steps = (ctypes.c_int * 2)()
        gres = ctypes.c_double()
        self._check(self.L.ollin_gpu_ell_stats(self.h, steps, ctypes.byref(gres)))
        return steps[0], steps[1], gres.value

    def interp(self, level, name, r, z):
        """``name`` at the points (r, z) of grid ``level`` (interp.f90)."""
        r = np.asarray(r, dtype=np.float64).ravel()
        z = np.asarray(z, dtype=np.float64).ravel()
        rz = np.ascontiguousarray(np.stack([r, z], axis=1))
        out = np.zeros(len(r))
        self._check(self.L.ollin_gpu_interp(self.h, level, field_id(name), rz.ctypes.data, len(r), out.ctypes.data))
        return out

    def ell_history(self, level):
        """RMS residuals of the last mixed / fp64mg solve on ``level``, one per
        FP64 refinement (the first before any correction)."""
        n = ctypes.c_int()
        self._check(self.L.ollin_gpu_ell_history(self.h, level, None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1))
        self._check(self.L.ollin_gpu_ell_history(self.h, level, out.ctypes.data, n.value, ctypes.byref(n)))
        return out[:n.value]

    def kernel_stats(self):
        """(total rhs-kernel ms, rhs launches, grid points x stages) since timing was enabled."""
        ms, n, pts = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
        self._check(self.L.ollin_gpu_kernel_stats(self.h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(pts)))
        return ms.value, n.value, pts.value


def step_many(evolutions):
    """One coarse step of every evolution, queued side by side on their
    streams (ollin_gpu_coarse_step_many); returns each t(0,0)."""
    if not evolutions:
        return []
    L = evolutions[0].L
    hs = (ctypes.c_void_p * len(evolutions))(*[e.h.value for e in evolutions])
    t = np.zeros(len(evolutions))
    rc = L.ollin_gpu_coarse_step_many(hs, len(evolutions), t.ctypes.data)
    if rc != 0:
        raise OllinError(rc, L.ollin_gpu_last_error().decode())
    return list(t)


def step_fused(evolutions):
    """One coarse step of every evolution with each kernel of the step issued
    once for all of them (ollin_gpu_coarse_step_fused); returns each t(0,0)."""
    if not evolutions:
        return []
    L = evolutions[0].L
    hs = (ctypes.c_void_p * len(evolutions))(*[e.h.value for e in evolutions])
    t = np.zeros(len(evolutions))
    rc = L.ollin_gpu_coarse_step_fused(hs, len(evolutions), t.ctypes.data, None)
    if rc != 0:
        raise OllinError(rc, L.ollin_gpu_last_error().decode())
    return list(t)


SCHEDULES = {0: "fused, graphs", 1: "fused, direct launches", 2: "one stream per evolution"}


def step_auto(evolutions):
    """One coarse step of every evolution under the schedule the autotuner
    chose for this batch (ollin_gpu_coarse_step_auto); returns (t(0,0) of
    each, the schedule used)."""
    L = evolutions[0].L
    hs = (ctypes.c_void_p * len(evolutions))(*[e.h.value for e in evolutions])
    t = np.zeros(len(evolutions))
    sched = ctypes.c_int()
    rc = L.ollin_gpu_coarse_step_auto(hs, len(evolutions), t.ctypes.data, ctypes.byref(sched))
    if rc != 0:
        raise OllinError(rc, L.ollin_gpu_last_error().decode())
    return list(t), sched.value


def fused_graphs(on):
    """Replay the fused steps' launch sequences as CUDA graphs (default) or
    issue them directly (ollin_gpu_fused_graphs)."""
    load().ollin_gpu_fused_graphs(1 if on else 0)


def footprint(params):
    """(resident, transient) device bytes of an evolution (ollin_gpu_footprint)."""
    L = load()
    r, t = ctypes.c_size_t(), ctypes.c_size_t()
    rc = L.ollin_gpu_footprint(ctypes.byref(params), ctypes.byref(r), ctypes.byref(t))
    if rc:
        raise OllinError(rc, L.ollin_gpu_last_error().decode())
    return r.value, t.value


RESULT_MAXGRIDS = 8


class Result(ctypes.Structure):
    """ollin_result: the summary of one finished request."""
    _fields_ = [("id", ctypes.c_longlong), ("status", ctypes.c_int), ("collapsed", ctypes.c_int),
                ("steps", ctypes.c_int), ("ngrids", ctypes.c_int), ("t", ctypes.c_double),
                ("min_alpha", ctypes.c_double), ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_ready", ctypes.c_double),
                ("t_done", ctypes.c_double), ("bytes", ctypes.c_size_t),
                ("l2", (ctypes.c_double * 4) * RESULT_MAXGRIDS), ("point_updates", ctypes.c_double)]

    def norms(self):
        """(ngrids, 4) array: L2 norms of alpha, phi, trK, ham per grid."""
        n = min(self.ngrids, RESULT_MAXGRIDS)
        return np.array([[self.l2[g][k] for k in range(4)] for g in range(n)])


class Server:
    """The request loop of the C ABI (ollin_server_*): continuous batching of
    evolutions on the current device, admitted against a byte budget."""

    def __init__(self, budget_bytes, max_active=64, graphs=True, fused=False):
        self.L = load()
        h = ctypes.c_void_p()
        self._check(self.L.ollin_server_create(int(budget_bytes), int(max_active), ctypes.byref(h)))
        self.h = h
        self._check(self.L.ollin_server_set_graphs(self.h, 1 if graphs else 0))
        self._check(self.L.ollin_server_set_fused(self.h, 1 if fused else 0))

    def _check(self, rc):
        if rc != 0:
            raise OllinError(rc, self.L.ollin_server_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.ollin_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, rid, params, t_end, collapse_alpha=0.0, maximalevery=0):
        self._check(self.L.ollin_server_submit(self.h, int(rid), ctypes.byref(params), int(maximalevery),
                                               float(t_end), float(collapse_alpha)))

    def tick(self):
        """One round; returns (running, waiting)."""
        a, w = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.ollin_server_tick(self.h, ctypes.byref(a), ctypes.byref(w)))
        return a.value, w.value

    def poll(self, max_results=256):
        buf = (Result * max_results)()
        n = ctypes.c_int()
        self._check(self.L.ollin_server_poll(self.h, buf, max_results, ctypes.byref(n)))
        return [buf[k] for k in range(n.value)]

    def usage(self):
        u, p = ctypes.c_size_t(), ctypes.c_size_t()
        self._check(self.L.ollin_server_usage(self.h, ctypes.byref(u), ctypes.byref(p)))
        return u.value, p.value

    def drain(self):
        """Tick until nothing runs or waits; return every result."""
        out = []
        while True:
            a, w = self.tick()
            out += self.poll()
            if a == 0 and w == 0:
                return out + self.poll()
