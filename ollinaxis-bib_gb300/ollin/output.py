"""The reference's 0-D output lines from the device's statistics.

``save0Dvariable`` (src/base/save0Ddata.f90:297-403) appends, per variable,
box and level, one line ``write(u, "(2ES20.8E3)") t, value`` to each of the
files ``<var>_b<box>l<level>_{max,min,nm1,nm2}.tl`` and, for box 0 only,
``..._origin.tl``.  A new file starts with the list-directed header
``comment//varname//'_<kind>.tl'`` (the origin file's header says
``_max.tl``, :363).  ``Save0D`` writes those files from
``Evolution.norms`` so that a host that reads the reference's output finds
the same lines.
"""
import math
import os

KINDS = ("max", "min", "nm1", "nm2", "origin")


def fortran_es(v, w=20, d=8, e=3):
    """Fortran ``ESw.dEe`` edit descriptor: one non-zero digit before the
    point, ``d`` after, an exponent of ``e`` digits with its sign, right
    justified in ``w`` columns (the value rounded to nearest, as gfortran
    and ifort do)."""
    v = float(v)
    if math.isnan(v):
        return "NaN".rjust(w)
    if math.isinf(v):
        return ("-Infinity" if v < 0 else "Infinity").rjust(w)
    mant, _, exp = ("%.*E" % (d, v)).partition("E")
    k = int(exp)
    sign = "-" if k < 0 else "+"
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
