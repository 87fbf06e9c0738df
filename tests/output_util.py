"""The reference's 0-D records computed straight from a golden fixture's
grid functions (outputs of the reference's own Fortran): the statistics of
save0Dvariable (src/base/save0Ddata.f90:221-288) restated with NumPy, and the
value at the origin by the 4x4 Lagrange interpolation of interp.f90, whose
weights at the origin (half a cell from the axis and the equator on every
box-0 level) are (-1, 9, 9, -1)/16 on i, j = -1..2."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
OUT_NAMES = ("alpha", "phi", "trK", "ham")


def load_fixture(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    cfg = {k: v for k, v in meta.items() if k not in ("steps", "fields", "grids", "oob_beyond_reads")}
    cfg["eqsym"] = 1 if cfg.get("eqsym") else 0
    return d, meta, cfg


def fixture_stats(a, g=3):
    """(max, min, max|f|, RMS, origin) of a[i+g-1, j+g-1] over i = 1..Nr-g,
    j = 1..Nz-g."""
    inner = a[g:-g, g:-g]
    w = np.array([-1.0, 9.0, 9.0, -1.0]) / 16.0
    origin = float(w @ a[g - 2:g + 2, g - 2:g + 2] @ w)
    return (float(inner.max()), float(inner.min()), float(np.abs(inner).max()),
            float(np.sqrt(np.mean(inner ** 2))), origin)


class OracleView:
    """What the 1-D and 2-D writers read (grids, descriptors, coordinates,
    arrays, interpolation), from an oracle evolution with box 0 only."""

    class Desc:
        pass

    def __init__(self, oracle, cfg):
        self.o = oracle
        self.cfg = cfg

    def levels(self):
        return self.o.levels()

    def grid(self, gid):
        return self.o.grid(gid)

    def coords(self, gid):
        r, z = self.o.get(gid, "r"), self.o.get(gid, "z")
        return r[:, 0].copy(), z[0, :].copy()

    def desc(self, gid):
        nr, nz, g = self.o.dims(gid)
        box, level = self.o.grid(gid)
        r, z = self.coords(gid)
        d = OracleView.Desc()
        d.nr, d.nz, d.ghost, d.box, d.level = nr, nz, g, box, level
        d.dr = self.cfg["dr0"] / 2.0 ** level
        d.dz = self.cfg["dz0"] / 2.0 ** level
        d.rmin, d.rmax, d.zmin, d.zmax = r[0], r[-1], z[0], z[-1]
        d.time = self.o.time(gid)
        d.rbox = d.zbox = 0.0
        return d

    def download(self, gid, name):
        return self.o.get(gid, name)

    def interp(self, gid, name, r, z):
        return self.o.interp(gid, name, r, z)
