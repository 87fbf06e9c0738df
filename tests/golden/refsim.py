"""Runs the reference Fortran evolution path (translated by ``ftn_subset``)
on a small box-0 grid hierarchy, serially.

The bookkeeping that the reference does in ``main.f90``, ``setupboxes.f90``,
``domaindecomp.f90`` (single process branch) and ``evolve.f90:42-219`` is
restated here in a few lines; everything that touches field values --
``initial``, ``auxiliary`` and the whole of ``onestep`` with the
Perl-generated ``saveold``/``accumulate``/``update``/``symmetries_*`` and the
``bound_interp.inc``/``restrict_interp.inc`` includes -- is the reference's
own Fortran, executed.  Used only by ``make_golden.py``, in a container that
has the reference sources.
"""
import os
import re
import shutil
import subprocess
import tempfile

import numpy as np

import ftn_subset as fs

PARAM_LINE = re.compile(
    r"^\s*(integer|real\s*\(\s*8\s*\)|logical|character\s*\(\s*\d+\s*\))\s*::\s*(\w+)\s*(\([^)]*\))?\s*=\s*([^!]+?)\s*(!.*)?$",
    re.I)

SOURCES = [
    "src/base/onestep.f90", "src/base/auxiliary.f90", "src/base/derivatives.f90",
    "src/base/derivadvect.f90", "src/base/dissipation.f90", "src/base/radbound.f90",
    "src/base/finebound.f90", "src/base/restrict.f90", "src/base/interp.f90",
    "src/base/initial.f90",
    "src/geometry/auxiliary_geometry.f90", "src/geometry/calc_conformalRicci1.f90",
    "src/geometry/calc_conformalRicci2.f90", "src/geometry/calc_conformalRicci3.f90",
    "src/geometry/calc_conformalRicci4.f90", "src/geometry/calc_DIVKTA.f90",
    "src/geometry/factordet.f90", "src/geometry/detrace_KT.f90",
    "src/geometry/sources_geometry.f90", "src/geometry/sources_lapse.f90",
    "src/geometry/sources_shift.f90", "src/geometry/radiative_geometry.f90",
    "src/geometry/constraints.f90",
    "src/matter/auxiliary_matter.f90", "src/matter/potential.f90",
    "src/matter/stressenergy.f90", "src/matter/sources_matter.f90",
    "src/matter/scalar.f90",
    "src/elliptic/wave_elliptic.f90", "src/elliptic/sor_elliptic.f90",
    "src/matter/idata_scalarpulse.f90", "src/geometry/idata_brillwave.f90",
    "src/geometry/maximalslicing.f90", "src/base/syncboxes.f90",
]
GENERATED = ["saveold.f90", "accumulate.f90", "update.f90", "symmetries_r.f90",
             "symmetries_z.f90", "simpleboundary.f90"]


def _param_value(typ, val):
    val = val.strip()
    t = typ.lower().replace(" ", "")
    if t == "integer":
        return int(val)
    if t == "logical":
        return val.lower() == ".true."
    if t.startswith("character"):
        return val.strip("\"'")
    # real(8): a literal without a d-exponent is a default (single) real
    v = val.lower()
    if "d" in v:
        return np.float64(float(v.replace("d", "e")))
    return np.float64(np.float32(float(v)))


class GridFuncs:
    """One (box, level) grid: arrays allocated lazily with the reference's bounds."""

    def __init__(self, ghost, nrmax, nzmax):
        self._g = ghost
        self._nr = nrmax
        self._nz = nzmax

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        g, nr, nz = self._g, self._nr, self._nz
        if name.endswith("_bound_rl") or name.endswith("_bound_rr"):
            a = fs.falloc((0, 1 - g, 0), (g - 1, nz, 2))
        elif name.endswith("_bound_zl") or name.endswith("_bound_zr"):
            a = fs.falloc((1 - g, 0, 0), (nr, g - 1, 2))
        else:
            a = fs.falloc((1 - g, 1 - g), (nr, nz))
        object.__setattr__(self, name, a)
        return a


class ModuleNS:
    """The union of the reference's modules (param, arrays, procinfo)."""

    def __init__(self):
        object.__setattr__(self, "_types", {})
        object.__setattr__(self, "_grid", None)

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        gr = object.__getattribute__(self, "_grid")
        if gr is None:
            raise AttributeError(name)
        return getattr(gr, name)


def _int_array(lbs, ubs, fill=0):
    shape = tuple(u - l + 1 for l, u in zip(lbs, ubs))
    a = np.full(shape, fill, dtype=np.int64).view(fs.FArray)
    a.lb = tuple(lbs)
    return a


def _obj_array(lbs, ubs):
    shape = tuple(u - l + 1 for l, u in zip(lbs, ubs))
    a = np.empty(shape, dtype=object).view(fs.FArray)
    a.lb = tuple(lbs)
    return a


def generate_auto(refdir, workdir):
    """Copy the reference and run its Perl generators; return the auto dir."""
    dst = os.path.join(workdir, "ref")
    shutil.copytree(refdir, dst)
    subprocess.run(["perl", "prl/assign.pl"], cwd=dst, check=False,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    subprocess.run(["perl", "prl/arrays.pl"], cwd=dst, check=False,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return os.path.join(dst, "src", "auto")


class RefSim:
    def __init__(self, refdir, params, workdir=None):
        self.refdir = refdir
        self.workdir = workdir or tempfile.mkdtemp(prefix="ollin_ref_")
        self.auto = generate_auto(refdir, self.workdir)
        M = self.M = ModuleNS()
        # parameter defaults from the reference's param module
        with open(os.path.join(refdir, "src/base/param.f90")) as f:
            for line in f:
                mm = PARAM_LINE.match(line)
                if not mm or mm.group(3):
                    continue
                typ, name, val = mm.group(1), mm.group(2).lower(), mm.group(4)
                object.__setattr__(M, name, _param_value(typ, val))
                t = typ.lower().replace(" ", "")
                M._types[name] = "real8" if t.startswith("real") else (
                    "integer" if t == "integer" else t)
        for k, v in params.items():
            k = k.lower()
            t = M._types.get(k)
            if t == "real8":
                v = np.float64(v)
            elif t == "integer":
                v = int(v)
            object.__setattr__(M, k, v)
        self._setup()
        prog = self.prog = fs.Program(M, include_dir=self.auto)
        texts = []
        for s in SOURCES:
            with open(os.path.join(refdir, s)) as f:
                texts.append(f.read())
        for s in GENERATED:
            with open(os.path.join(self.auto, s)) as f:
                texts.append(f.read())
        prog.load(texts, extra_functions=("interp",))
        prog.define("currentgrid", self._currentgrid)
        prog.define("syncall", lambda: None)
        prog.define("save1dvariable", lambda *a: None)
        prog.define("save2dvariable", lambda *a: None)
        prog.define("sync", lambda *a: None)
        for nm in ("idata_kerr", "idata_complexpulse",
                   "idata_bosonstarcf", "idata_rotboson", "checkpointrestart",
                   "sources_complex", "constraintbound"):
            prog.define(nm, self._unsupported(nm))
        prog.define("grabarray", lambda *a: None)

    @staticmethod
    def _unsupported(name):
        def f(*a):
            raise NotImplementedError("%s is outside the golden-vector scope" % name)
        return f

    # ------------------------------------------------------------------
    # bookkeeping (main.f90, setupboxes.f90, domaindecomp.f90, evolve.f90)
    # ------------------------------------------------------------------
    def _setup(self):
        M = self.M
        s = lambda k, v: object.__setattr__(M, k, v)
        s("rank", 0)
        s("size", 1)
        s("nprocr", 1)
        s("nprocz", 1)
        if M.ghost == 0:
            s("ghost", 2 if M.order == "two" else 3)
        g = M.ghost
        nb = int(M.nb)
        if nb < 0 or nb > 3:
            raise ValueError("The number of refinement boxes must be between 0 and 3")
        nl = _int_array((0,), (3,))
        nl[0], nl[1], nl[2], nl[3] = M.nl0, M.nl1, M.nl2, M.nl3
        s("nl", nl)
        s("nlmax", int(max(nl[b] for b in range(nb + 1))))
        L = M.nlmax
        s("dt0", np.float64(M.dtfac * min(M.dr0, M.dz0)))
        drl = fs.falloc((0,), (L,))
        dzl = fs.falloc((0,), (L,))
        dtl = fs.falloc((0,), (L,))
        for lev in range(L + 1):
            dtl[lev] = M.dt0 / 2 ** lev
            drl[lev] = M.dr0 / 2 ** lev
            dzl[lev] = M.dz0 / 2 ** lev
        s("drl", drl)
        s("dzl", dzl)
        s("dtl", dtl)
        if not M.eqsym and (M.nztotal + g) % 2 == 0:
            s("nztotal", M.nztotal + 1)
        # box sizes and centres, setupboxes.f90:143-206
        nrbox = _int_array((0,), (3,), 1)
        nzbox = _int_array((0,), (3,), 1)
        nrbox[0] = M.nrtotal
        nzbox[0] = M.nztotal
        rbox = fs.falloc((0,), (3,))
        zbox = fs.falloc((0,), (3,))
        for b in range(1, 4):
            nrbox[b] = getattr(M, "nrbox%d" % b)
            nzbox[b] = getattr(M, "nzbox%d" % b)
            rbox[b] = np.float64(getattr(M, "rbox%d" % b))
            zbox[b] = np.float64(getattr(M, "zbox%d" % b))
        for b in range(1, nb + 1):
            if rbox[b] != 0.0:
                rbox[b] = (np.float64(int(rbox[b] / drl[1])) + 0.5) * drl[1]
            if zbox[b] != 0.0:
                if M.eqsym:
                    zbox[b] = (np.float64(int(zbox[b] / dzl[1])) + 0.5) * dzl[1]
                else:
                    zbox[b] = np.float64(int(zbox[b] / dzl[1])) * dzl[1]
        s("nrbox", nrbox)
        s("nzbox", nzbox)
        s("rbox", rbox)
        s("zbox", zbox)
        for nm in ("s",):
            s(nm, _int_array((0, 0), (nb, L)))
        for nm in ("t", "t1", "t2", "rminl", "rmaxl", "zminl", "zmaxl"):
            s(nm, fs.falloc((0, 0), (nb, L)))
        nrl = _int_array((0, 0), (nb, 0))
        nzl = _int_array((0, 0), (nb, 0))
        for b in range(nb + 1):
            nrl[b, 0] = nrbox[b]
            nzl[b, 0] = nzbox[b]
        s("nrl", nrl)
        s("nzl", nzl)
        nrmaxl = _int_array((0,), (nb,))
        nzmaxl = _int_array((0,), (nb,))
        for b in range(nb + 1):
            nrmaxl[b] = nrbox[b]
            nzmaxl[b] = nzbox[b]
        s("nrmaxl", nrmaxl)
        s("nzmaxl", nzmaxl)
        s("nminl_r", _int_array((0, 0), (nb, 0)))
        s("nminl_z", _int_array((0, 0), (nb, 0)))
        # main.f90:380-460: the axis belongs to boxes with rbox = 0, the
        # equator to boxes with zbox = 0
        axis = _int_array((0, 0), (nb, 0), -1)
        eqz = _int_array((0, 0), (nb, 0), -1)
        origin = _int_array((0, 0), (nb, 0), -1)
        for b in range(nb + 1):
            if rbox[b] == 0.0:
                axis[b, 0] = 1
            if zbox[b] == 0.0:
                if M.eqsym:
                    eqz[b, 0] = 1
                    origin[b, 0] = 1
                else:
                    for j in range(1, nzbox[b] - g + 1):
                        aux = (float(j) - 0.5 * float(nzbox[b] - g + 1)) * M.dz0
                        if aux == 0.0 or aux == 0.5 * M.dz0:
                            eqz[b, 0] = j
                            origin[b, 0] = j
                            break
        s("axis", axis)
        s("eqz", eqz)
        s("origin", origin)
        grid = _obj_array((0, 0), (nb, L))
        self.grids = []
        for b in range(nb + 1):
            for lev in range(min(1, b), int(nl[b]) + 1):
                grid[b, lev] = GridFuncs(g, int(nrbox[b]), int(nzbox[b]))
                self.grids.append((b, lev))
        # grid order of the library and the oracle: box 0, then boxes 1..Nb
        self.grids.sort(key=lambda bl: (bl[0] != 0, bl[0], bl[1]))
        s("grid", grid)
        # coordinates (evolve.f90:42-97), single process
        for b, lev in self.grids:
            gf = grid[b, lev]
            dr, dz = drl[lev], dzl[lev]
            r = gf.r
            z = gf.z
            nrb, nzb = int(nrbox[b]), int(nzbox[b])
            for i in range(1 - g, nrb + 1):
                if rbox[b] == 0.0:
                    v = (np.float64(0 + i) - 0.5) * dr
                else:
                    v = rbox[b] + (np.float64(0 + i) - 0.5 * np.float64(nrb - g + 1)) * dr
                fs.fset(r, (i, slice(None, None)), v)
            for j in range(1 - g, nzb + 1):
                if M.eqsym and zbox[b] == 0.0:
                    v = (np.float64(0 + j) - 0.5) * dz
                else:
                    v = zbox[b] + (np.float64(0 + j) - 0.5 * np.float64(nzb - g + 1)) * dz
                fs.fset(z, (slice(None, None), j), v)
            gf.rr[...] = np.sqrt(r ** 2 + z ** 2)
            self.M.rminl[b, lev] = fs.fget(r, (1 - g, 0))
            self.M.rmaxl[b, lev] = fs.fget(r, (nrb, 0))
            self.M.zminl[b, lev] = fs.fget(z, (0, 1 - g))
            self.M.zmaxl[b, lev] = fs.fget(z, (0, nzb))

    def _currentgrid(self, box, level, localgrid):
        M = self.M
        s = lambda k, v: object.__setattr__(M, k, v)
        s("ownaxis", fs.fget(M.axis, (box, M.rank)) != -1)
        s("ownequator", fs.fget(M.eqz, (box, M.rank)) != -1)
        s("ownorigin", fs.fget(M.origin, (box, M.rank)) != -1)
        s("nr", int(fs.fget(M.nrl, (box, M.rank))))
        s("nz", int(fs.fget(M.nzl, (box, M.rank))))
        s("nrmax", int(fs.fget(M.nrmaxl, (box,))))
        s("nzmax", int(fs.fget(M.nzmaxl, (box,))))
        s("time", np.float64(fs.fget(M.t, (box, level))))
        s("dt", np.float64(fs.fget(M.dtl, (level,))))
        s("dr", np.float64(fs.fget(M.drl, (level,))))
        s("dz", np.float64(fs.fget(M.dzl, (level,))))
        object.__setattr__(M, "_grid", localgrid)

    # ------------------------------------------------------------------
    # driver (evolve.f90:104-219 and the main loop :357-381)
    # ------------------------------------------------------------------
    def levels(self):
        """Grid indices: box 0's levels, then the levels of boxes 1..Nb."""
        return range(len(self.grids))

    def box_level(self, gid):
        return self.grids[gid]

    def use(self, gid):
        b, lev = self.grids[gid]
        self._currentgrid(b, lev, self.M.grid[b, lev])

    def time(self, gid):
        b, lev = self.grids[gid]
        return float(self.M.t[b, lev])

    def initial(self):
        """call initial (evolve.f90:124)."""
        M, F = self.M, self.prog.F
        object.__setattr__(M, "s", _int_array((0, 0), (int(M.nb), M.nlmax)))
        F.initial()

    def set_field(self, gid, name, values):
        b, lev = self.grids[gid]
        a = getattr(self.M.grid[b, lev], fs.pyname(name.lower()))
        a.view(np.ndarray)[...] = values

    def initialize(self):
        """evolve.f90:128-195: symmetries, auxiliary at t=0, Gamma driver."""
        M, F = self.M, self.prog.F
        for lev in self.levels():
            self.use(lev)
            if M.ownaxis:
                F.symmetries_r()
            if M.eqsym and M.ownequator:
                F.symmetries_z()
        for lev in self.levels():
            self.use(lev)
            F.auxiliary()
        if M.shift in ("Gammadriver2", "Gammadrivershock2") and not M.driverd0:
            for lev in self.levels():
                self.use(lev)
                M.dtbeta_r[...] = M.drivercsi * M.delta_r
                M.dtbeta_z[...] = M.drivercsi * M.delta_z
        # evolve.f90:211-219: boxes that overlap on a level synchronise
        for level in range(1, int(M.nlmax) + 1):
            for b1 in range(int(M.nb) + 1):
                for b2 in range(int(M.nb) + 1):
                    if b1 != b2 and M.nl[b1] >= level and M.nl[b2] >= level:
                        F.syncboxes(b1, b2, level, True)
        # evolve.f90:228-230; no analysis has run, so va_rp/va_zp are zero
        if M.slicing == "maximal" or M.ilapse == "maximal" or M.maximalevery != 0:
            F.maximalslicing()

    def step(self):
        self.prog.F.onestep(0)

    def maximal_slicing(self):
        """call maximalslicing, as evolve.f90:388-393 does after a coarse step."""
        self.prog.F.maximalslicing()

    def field(self, level, name):
        """Interior+ghost copy of a grid array (Fortran (i,j) -> [i+g-1, j+g-1])."""
        b, lev = self.grids[level]
        a = getattr(self.M.grid[b, lev], fs.pyname(name.lower()))
        return np.array(a.view(np.ndarray), copy=True)

    def analysis(self, gid):
        self.use(gid)
        b, lev = self.grids[gid]
        self.prog.F.constraints(b, lev)
