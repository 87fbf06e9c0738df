"""0-D output compatibility (src/base/save0Ddata.f90:297-403): the
``(2ES20.8E3)`` records and file names of save0Dvariable, written by
ollin.output from the statistics of ollin_gpu_norms.  Here, without a GPU:
the edit descriptor against hand-checked Fortran output, and the records of
the oracle's statistics against the records computed from the
reference-executed fixture c1_small (the same lines, character for
character).  The GPU path is held to the same lines in test_gpu_output.py."""
import numpy as np
import pytest

from ollin.output import Save0D, fortran_es, header, lines, tl_line
from oracle_bind import Oracle
from output_util import OUT_NAMES, fixture_stats, load_fixture
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
