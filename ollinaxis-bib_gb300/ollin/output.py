"""The reference's output files from the device's state.

* 0-D: ``save0Dvariable`` (src/base/save0Ddata.f90:297-403) appends, per
  variable, box and level, one line ``write(u, "(2ES20.8E3)") t, value`` to
  each of the files ``<var>_b<box>l<level>_{max,min,nm1,nm2}.tl`` and, for
  box 0 only, ``..._origin.tl``.  A new file starts with the list-directed
  header ``comment//varname//'_<kind>.tl'`` (the origin file's header says
  ``_max.tl``, :363).  ``Save0D`` writes them from ``Evolution.norms``.
* 1-D: ``save1Dvariable`` (save1Ddata.f90:156-750, one process) writes a
  ``"Time = `` record ``(A8,ES14.6)`` and then ``(2ES20.8E3)`` pairs along
  the equator row (``.rl``, the row eqz of main.f90:405-470: z = dz/2 with
  equatorial symmetry, else the row at z = 0 or dz0/2), the axis column
  i = 1 (``.zl``, grids on the axis) and, for box 0, the domain diagonal
  interpolated at NN+1 points (``.dl``; without equatorial symmetry the two
  diagonals ``.d1l`` and ``.d2l``), each block closed by an empty record.
  ``Save1D`` writes them from ``Evolution.download`` and ``Evolution.interp``.
* 2-D: ``save2Dvariable`` (save2Ddata.f90:150-280, one process) writes a
  ``#Time = `` record ``(A8,ES23.15)`` and then r, z, value + 1e-30 for every
  point, r fastest, an empty record after each z-row and one more after the
  block: ``(3ES23.15)`` while the file is new and ``(3ES16.8)`` when
  appending (:227-231).  ``Save2D`` writes them.

A host that reads the reference's output finds the same lines.
"""
import math
import os

KINDS = ("max", "min", "nm1", "nm2", "origin")


def fortran_es(v, w=20, d=8, e=3):
    """Fortran ``ESw.dEe`` edit descriptor: one non-zero digit before the
    point, ``d`` after, an exponent of ``e`` digits with its sign, right
    justified in ``w`` columns (the value rounded to nearest, as gfortran
    and ifort do).  ``e=None`` is ``ESw.d``: the exponent as ``E+dd``, or
    ``+ddd`` without the letter when it needs three digits."""
    v = float(v)
    if math.isnan(v):
        return "NaN".rjust(w)
    if math.isinf(v):
        return ("-Infinity" if v < 0 else "Infinity").rjust(w)
    mant, _, exp = ("%.*E" % (d, v)).partition("E")
    k = int(exp)
    sign = "-" if k < 0 else "+"
    if e is None:
        s = ("%sE%s%02d" % (mant, sign, abs(k))) if abs(k) <= 99 else ("%s%s%03d" % (mant, sign, abs(k)))
    else:
        s = "%sE%s%0*d" % (mant, sign, e, abs(k))
    if len(s) > w:
        return "*" * w
    return s.rjust(w)


def tl_line(t, value):
    """One ``(2ES20.8E3)`` record."""
    return fortran_es(t) + fortran_es(value)


def header(varname, kind, comment='"'):
    """List-directed header record of a new file (leading blank)."""
    name = "max" if kind == "origin" else kind
    return " " + comment + varname + "_" + name + ".tl"


def lines(t, stats, box=0):
    """The records of one save0Dvariable call: ``stats`` = (max, min, nm1,
    nm2, origin) as ollin_gpu_norms returns them; no origin record off box 0."""
    out = {k: tl_line(t, v) for k, v in zip(KINDS[:4], stats[:4])}
    if box == 0:
        out["origin"] = tl_line(t, stats[4])
    return out


class Save0D:
    """Appends the 0-D records of ``names`` on every grid of an evolution to
    ``outdir`` as the reference's files (filestatus 'new' on the first call,
    'old' afterwards)."""

    def __init__(self, outdir, names, comment='"'):
        self.outdir = outdir
        self.names = list(names)
        self.comment = comment
        self.first = True
        os.makedirs(outdir, exist_ok=True)

    def write(self, evolution):
        for gid in evolution.levels():
            box, level = evolution.grid(gid)
            t = evolution.clocks(gid)[0]
            for nm in self.names:
                for kind, rec in lines(t, evolution.norms(gid, nm), box).items():
                    path = os.path.join(self.outdir, "%s_b%dl%d_%s.tl" % (nm, box, level, kind))
                    with open(path, "w" if self.first else "a") as f:
                        if self.first:
                            f.write(header(nm, kind, self.comment) + "\n")
                        f.write(rec + "\n")
        self.first = False


# ---- 1-D and 2-D output -----------------------------------------------------

def time_record_1d(t):
    """``write(u, "(A8,ES14.6)") '"Time = ', t``."""
    return '"Time = ' + fortran_es(t, 14, 6, None)


def time_record_2d(t):
    """``write(u, "(A8,ES23.15)") '#Time = ', t``."""
    return "#Time = " + fortran_es(t, 23, 15, None)


def pair(x, y):
    """One ``(2ES20.8E3)`` record."""
    return fortran_es(x) + fortran_es(y)


def equator_row(desc, eqsym):
    """eqz of main.f90:405-470 for a grid (Fortran j), or None when the grid's
    box does not own the equator: j = 1 with equatorial symmetry, otherwise
    the first interior row whose level-0 height is 0 or dz0/2; only boxes with
    zbox = 0 own it."""
    if desc.zbox != 0.0:
        return None
    if eqsym:
        return 1
    g, nz = desc.ghost, desc.nz
    dz0 = desc.dz * float(2 ** desc.level)
    for j in range(1, nz - g + 1):
        aux = (float(j) - 0.5 * float(nz - g + 1)) * dz0
        if aux == 0.0 or aux == 0.5 * dz0:
            return j
    return None


def diagonal_points(desc):
    """save1Ddata.f90:640-660: NN+1 points (r0, z0) along the diagonal of box
    0's grid and their distances rr0 from the origin."""
    rmax, zmax = desc.rmax, desc.zmax
    rrmax = math.sqrt(rmax * rmax + zmax * zmax)
    delta = math.sqrt(desc.dr * desc.dr + desc.dz * desc.dz)
    nn = int(rrmax / delta + 0.5)
    delta = 1.0 / float(nn)
    aux = [(float(i) - 0.5) * delta for i in range(nn + 1)]
    return [a * rmax for a in aux], [a * zmax for a in aux], [a * rrmax for a in aux]


def lines_1d(evolution, gid, name, eqsym):
    """{extension: [records]} of one save1Dvariable call for one grid."""
    d = evolution.desc(gid)
    g = d.ghost
    r, z = evolution.coords(gid)
    a = evolution.download(gid, name)
    t = time_record_1d(d.time)
    out = {}
    eqz = equator_row(d, eqsym)
    if eqz is not None:
        out["rl"] = [t] + [pair(r[k], a[k, eqz + g - 1]) for k in range(d.nr + g)] + [""]
    if d.rbox == 0.0:
        out["zl"] = [t] + [pair(z[k], a[g, k]) for k in range(d.nz + g)] + [""]
    if d.box == 0:
        r0, z0, rr0 = diagonal_points(d)
        v = evolution.interp(gid, name, r0, z0)
        if eqsym:
            out["dl"] = [t] + [pair(x, y) for x, y in zip(rr0, v)] + [""]
        else:
            v2 = evolution.interp(gid, name, r0, [-x for x in z0])
            out["d1l"] = [t] + [pair(x, y) for x, y in zip(rr0, v)] + [""]
            out["d2l"] = [t] + [pair(x, y) for x, y in zip(rr0, v2)] + [""]
    return out


def lines_2d(evolution, gid, name, new):
    """The records of one save2Dvariable call for one grid; ``new`` is the
    file status (the number format depends on it)."""
    d = evolution.desc(gid)
    g = d.ghost
    r, z = evolution.coords(gid)
    a = evolution.download(gid, name)
    w, p = (23, 15) if new else (16, 8)
    out = [time_record_2d(d.time)]
    for j in range(d.nz + g):
        zj = fortran_es(z[j], w, p, None)
        for i in range(d.nr + g):
            out.append(fortran_es(r[i], w, p, None) + zj + fortran_es(a[i, j] + 1.0e-30, w, p, None))
        out.append("")
    out.append("")
    return out


class _Writer:
    def __init__(self, outdir, names):
        self.outdir = outdir
        self.names = list(names)
        self.first = True
        os.makedirs(outdir, exist_ok=True)

    def _append(self, path, records):
        with open(path, "w" if self.first else "a") as f:
            for rec in records:
                f.write(rec + "\n")


class Save1D(_Writer):
    """Appends the 1-D records of ``names`` on every grid of an evolution to
    ``outdir`` as the reference's ``<var>_b<box>l<level>.{rl,zl,dl}`` files
    (``.d1l``/``.d2l`` without equatorial symmetry)."""

    def __init__(self, outdir, names, eqsym):
        super().__init__(outdir, names)
        self.eqsym = bool(eqsym)

    def write(self, evolution):
        for gid in evolution.levels():
            box, level = evolution.grid(gid)
            for nm in self.names:
                for ext, recs in lines_1d(evolution, gid, nm, self.eqsym).items():
                    self._append(os.path.join(self.outdir, "%s_b%dl%d.%s" % (nm, box, level, ext)), recs)
        self.first = False


class Save2D(_Writer):
    """Appends the 2-D records of ``names`` on every grid of an evolution to
    ``outdir`` as the reference's ``<var>_b<box>l<level>.2D`` files."""

    def write(self, evolution):
        for gid in evolution.levels():
            box, level = evolution.grid(gid)
            for nm in self.names:
                self._append(os.path.join(self.outdir, "%s_b%dl%d.2D" % (nm, box, level)),
                             lines_2d(evolution, gid, nm, self.first))
        self.first = False
