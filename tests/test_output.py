"""0-D output compatibility (src/base/save0Ddata.f90:297-403): the
``(2ES20.8E3)`` records and file names of save0Dvariable, written by
ollin.output from the statistics of ollin_gpu_norms.  Here, without a GPU:
the edit descriptor against hand-checked Fortran output, and the records of
the oracle's statistics against the records computed from the
reference-executed fixture c1_small (the same lines, character for
character).  The GPU path is held to the same lines in test_gpu_output.py."""
import numpy as np
import pytest

from ollin.output import Save0D, Save1D, Save2D, fortran_es, header, lines, lines_1d, lines_2d, tl_line
from oracle_bind import Oracle
from output_util import OUT_NAMES, OracleView, fixture_stats, load_fixture
from parity_util import params


@pytest.mark.parametrize("v,text", [
    (1.0, "     1.00000000E+000"),
    (-2.5e-7, "    -2.50000000E-007"),
    (0.0, "     0.00000000E+000"),
    (123456789.5, "     1.23456790E+008"),
    (9.999999999e-101, "     1.00000000E-100"),
    (0.05, "     5.00000000E-002"),
])
def test_es20_8e3_edit_descriptor(v, text):
    assert fortran_es(v) == text
    assert len(fortran_es(v)) == 20


def test_records_and_headers():
    rec = lines(0.5, (2.0, -1.0, 2.0, 0.25, 1.5), box=0)
    assert rec["max"] == "     5.00000000E-001     2.00000000E+000"
    assert rec["origin"] == tl_line(0.5, 1.5)
    assert "origin" not in lines(0.5, (2.0, -1.0, 2.0, 0.25, 1.5), box=1)
    assert header("alpha", "nm2") == ' "alpha_nm2.tl'
    assert header("alpha", "origin") == ' "alpha_max.tl'  # save0Ddata.f90:363


def test_oracle_records_match_reference_fixture(tmp_path):
    d, meta, cfg = load_fixture("c1_small")
    o = Oracle(params(cfg))
    o.initial_data()
    o.initialize()
    done = 0
    for target in meta["steps"]:
        while done < target:
            o.step()
            done += 1
        for lev in o.levels():
            o.constraints(lev)
            t = float(d["s%d_L%d_time" % (done, lev)])
            for nm in OUT_NAMES:
                key = "s%d_L%d_%s" % (done, lev, nm)
                if key not in d:  # the constraints are stored at the first and last snapshot
                    continue
                ref = lines(t, fixture_stats(d[key]))
                got = lines(o.time(lev), o.norms(lev, nm))
                assert got == ref, (done, lev, nm, got, ref)


class _FakeEvolution:
    """Just what Save0D reads: grids, clocks and norms."""

    def __init__(self, t):
        self.t = t

    def levels(self):
        return range(2)

    def grid(self, gid):
        return (0, gid)

    def clocks(self, gid):
        return np.array([self.t, 0.0, 0.0, 0.0])

    def norms(self, gid, name):
        return np.array([1.0 + gid, -1.0, 1.0 + gid, 0.5, 0.75])


def test_save0d_files(tmp_path):
    s = Save0D(str(tmp_path), ["alpha"])
    s.write(_FakeEvolution(0.0))
    s.write(_FakeEvolution(0.25))
    text = (tmp_path / "alpha_b0l1_nm1.tl").read_text().splitlines()
    assert text == [' "alpha_nm1.tl', tl_line(0.0, 2.0), tl_line(0.25, 2.0)]
    assert (tmp_path / "alpha_b0l0_origin.tl").read_text().splitlines()[0] == ' "alpha_max.tl'


@pytest.mark.parametrize("v,w,d,text", [
    (1.0, 14, 6, "  1.000000E+00"),
    (0.03125, 14, 6, "  3.125000E-02"),
    (-2.5, 23, 15, " -2.500000000000000E+00"),
    (1.0e-30, 16, 8, "  1.00000000E-30"),
    (2.5e-150, 14, 6, "  2.500000-150"),
])
def test_es_edit_descriptors_without_exponent_width(v, w, d, text):
    """ESw.d: a two-digit exponent after E, or three digits with the letter
    dropped beyond 99."""
    assert fortran_es(v, w, d, None) == text


def _es(v, w, d, e):
    """An independent ESw.dEe formatter (NumPy) for the records below."""
    m = np.format_float_scientific(v, precision=d, unique=False, exp_digits=e).upper()
    return m.rjust(w)


def _fixture_view(name, step):
    """The writers' view of a reference-executed fixture at one snapshot: its
    arrays set into an oracle of the same configuration (for the
    coordinates and interp.f90 along the diagonal)."""
    d, meta, cfg = load_fixture(name)
    o = Oracle(params(cfg))
    o.initial_data()
    for lev in o.levels():
        for nm in ("alpha", "trK"):
            o.set(lev, nm, d["s%d_L%d_%s" % (step, lev, nm)])
    v = OracleView(o, cfg)
    v.time = {lev: float(d["s%d_L%d_time" % (step, lev)]) for lev in o.levels()}
    base_desc = v.desc

    def desc(gid):
        x = base_desc(gid)
        x.time = v.time[gid]
        return x
    v.desc = desc
    return v, d, cfg


def test_1d_and_2d_records_of_a_reference_fixture():
    """save1Dvariable / save2Dvariable records of the fields of the
    reference-executed fixture c1_small after two steps, against records
    built independently here: the equator row j = 1 (.rl), the axis column
    i = 1 (.zl), the diagonal through interp.f90 (.dl), every point with
    +1e-30 (.2D); the time records; the empty records."""
    v, d, cfg = _fixture_view("c1_small", 2)
    g = 3
    for lev in v.levels():
        a = d["s2_L%d_alpha" % lev]
        r, z = v.coords(lev)
        t = float(d["s2_L%d_time" % lev])
        got = lines_1d(v, lev, "alpha", True)
        head = '"Time = ' + _es(t, 14, 6, 2)
        assert got["rl"] == [head] + [_es(r[k], 20, 8, 3) + _es(a[k, g], 20, 8, 3) for k in range(len(r))] + [""]
        assert got["zl"] == [head] + [_es(z[k], 20, 8, 3) + _es(a[g, k], 20, 8, 3) for k in range(len(z))] + [""]
        desc = v.desc(lev)
        rrmax = np.sqrt(desc.rmax ** 2 + desc.zmax ** 2)
        nn = int(rrmax / np.sqrt(desc.dr ** 2 + desc.dz ** 2) + 0.5)
        assert len(got["dl"]) == nn + 3
        aux = (np.arange(nn + 1) - 0.5) / nn
        vals = v.o.interp(lev, "alpha", aux * desc.rmax, aux * desc.zmax)
        assert got["dl"][1:-1] == [_es(x, 20, 8, 3) + _es(y, 20, 8, 3) for x, y in zip(aux * rrmax, vals)]
        two = lines_2d(v, lev, "alpha", True)
        assert two[0] == "#Time = " + _es(t, 23, 15, 2)
        body = []
        for j in range(len(z)):
            body += [_es(r[i], 23, 15, 2) + _es(z[j], 23, 15, 2) + _es(a[i, j] + 1e-30, 23, 15, 2)
                     for i in range(len(r))] + [""]
        assert two[1:] == body + [""]
        again = lines_2d(v, lev, "alpha", False)
        assert again[1] == _es(r[0], 16, 8, 2) + _es(z[0], 16, 8, 2) + _es(a[0, 0] + 1e-30, 16, 8, 2)


def test_1d_2d_files(tmp_path):
    """File names and appending: two calls, the 2-D file's second block in
    the shorter format; without equatorial symmetry the two diagonals and
    the equator row at z = 0."""
    cfg = dict(eqsym=0, nrtotal=16, nztotal=16, nl0=1, dr0=0.25, dz0=0.25, order="four", idata="schwarzschild",
               ilapse="psiminus2")
    o = Oracle(params(cfg))
    o.initial_data()
    o.initialize()
    v = OracleView(o, cfg)
    s1, s2 = Save1D(tmp_path, ["alpha"], eqsym=False), Save2D(tmp_path, ["alpha"])
    s1.write(v)
    s2.write(v)
    s1.write(v)
    s2.write(v)
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["alpha_b0l0.2D", "alpha_b0l0.d1l", "alpha_b0l0.d2l", "alpha_b0l0.rl", "alpha_b0l0.zl",
                     "alpha_b0l1.2D", "alpha_b0l1.d1l", "alpha_b0l1.d2l", "alpha_b0l1.rl", "alpha_b0l1.zl"]
    rl = (tmp_path / "alpha_b0l0.rl").read_text().split("\n")
    nr, nz, g = o.dims(0)
    assert rl[0].startswith('"Time = ') and len(rl) == 2 * (nr + g + 2) + 1
    # the equator row: z = 0 on an odd number of rows
    z = o.get(0, "z")[0, :]
    r_row = [float(x[20:]) for x in rl[1:nr + g + 1]]
    jq = int(np.argmin(np.abs(z)))
    assert z[jq] == 0.0 and np.allclose(r_row, o.get(0, "alpha")[:, jq], rtol=1e-8)
    two = (tmp_path / "alpha_b0l1.2D").read_text().split("\n")
    n1, m1, g1 = o.dims(1)
    block = 1 + (n1 + g1 + 1) * (m1 + g1) + 1
    assert len(two[1]) == 69 and len(two[block + 1]) == 48
    d1 = (tmp_path / "alpha_b0l0.d1l").read_text().split("\n")
    d2 = (tmp_path / "alpha_b0l0.d2l").read_text().split("\n")
    # the Schwarzschild lapse is even in z: the two diagonals agree
    assert [x[20:] for x in d1] == [x[20:] for x in d2]
