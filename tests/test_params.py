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
        params_from_par("shift = Gammadriver1\n")
    with pytest.raises(ValueError):
        params_from_par("nosuchparameter = 3\n")
