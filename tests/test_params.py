"""Par-file parsing with the reference's conventions (src/base/parse.f90)."""
import pytest

from ollin.params import SHIFT, SLICING, params_from_par


PAR = """
! Schwarzschild with Gamma driver (comment)
Nrtotal = 64
Nztotal = 64
Nl0 = 2
dr0 = 0.2
dz0 = 0.2
eqsym = .true.
order = four
integrator = rk4
slicing = 1+log
gauge_f = 2.0
shift = Gammadriver2
drivereta = 2.0
geodiss = 0.02
idata = schwarzschild
ilapse = psiminus2
Nt = 200
"""


def test_par_file_values():
    p = params_from_par(PAR)
    assert (p.nrtotal, p.nztotal, p.nl0) == (64, 64, 2)
    assert p.order == 4 and p.eqsym == 1
    assert p.slicing == SLICING["1+log"] and p.shift == SHIFT["Gammadriver2"]
    assert p.geodiss == 0.02 and p.drivereta == 2.0
    assert p.dr0 == 0.2


def test_unknown_values_are_refused():
    with pytest.raises(ValueError):
        params_from_par("shift = Gammadriver3\n")
    with pytest.raises(ValueError):
        params_from_par("nosuchparameter = 3\n")


def test_refinement_box_parameters():
    """Nb, Nl1..3, Nrbox1..3, Nzbox1..3, rbox1..3, zbox1..3 (param.f90:114-139)."""
    p = params_from_par("Nb = 2\nNl1 = 2\nNrbox1 = 12\nNzbox1 = 14\nzbox1 = 6.0\nNl2 = 1\nrbox2 = 8.d0\n"
                        "slicing = maximal\nilapse = maximal\nmaximalevery = 4\n")
    assert p.nb == 2
    assert list(p.nl) == [2, 1, 0]
    assert list(p.nrbox) == [12, 1, 1] and list(p.nzbox) == [14, 1, 1]
    assert list(p.rbox) == [0.0, 8.0, 0.0] and list(p.zbox) == [6.0, 0.0, 0.0]
    assert p.slicing == SLICING["maximal"]


def test_gamma_driver_names():
    """shift = Gammadriver0 / 1 / 2, the shock-avoiding drivers, zero and
    static (param.f90:344 names, sources_shift.f90); driverD0, shiftafter."""
    for name, code in (("Gammadriver0", 5), ("Gammadriver1", 4), ("Gammadriver2", 3), ("Gammadrivershock1", 6),
                       ("Gammadrivershock2", 7), ("zero", 1), ("static", 2)):
        assert params_from_par("shift = %s\n" % name).shift == code
    p = params_from_par("shift = Gammadrivershock2\ndriverD0 = .true.\nshiftafter = 1.5\n")
    assert p.driverD0 == 1 and p.shiftafter == 1.5
