"""The GPU evolution reproduces the convergence of the reference scheme: at
three resolutions its origin values give the same self-convergence factors
as the oracle's (fourth order for trK, phi and the scalar field; the lapse
and the metric are pre-asymptotic here, and with matter the lapse and phi
converge at second order in the reference scheme itself)."""
import numpy as np
import pytest

from convergence_util import RESOLUTIONS, T_END, config, factors, prepare
from parity_util import params
from test_convergence import oracle_origin_values

pytestmark = pytest.mark.gpu

FIELDS = ["alpha", "trK", "phi", "A"]


def gpu_origin_values(matter, fields, order="four"):
    from ollin.gpu import Evolution
    out = []
    for n, h in RESOLUTIONS:
        e = Evolution(params(config(n, h, matter, order)))
        e.initial_data()
        prepare(e, matter, lambda nm: _coord(e, nm), lambda nm, v: e.upload(0, nm, v))
        e.initialize()
        for _ in range(int(round(T_END / (0.25 * h)))):
            e.step()
        out.append([e.norms(0, f)[4] for f in fields])
    return out


def _coord(e, name):
    d = e.desc(0)
    g = d.ghost
    r = (np.arange(1 - g, d.nr + 1, dtype=np.float64) - 0.5) * d.dr
    z = (np.arange(1 - g, d.nz + 1, dtype=np.float64) - 0.5) * d.dz
    R, Z = np.meshgrid(r, z, indexing="ij")
    return R if name == "r" else Z


@pytest.mark.parametrize("matter", [False, True], ids=["gauge_pulse", "scalar_pulse"])
def test_gpu_reproduces_reference_convergence(matter):
    fields = FIELDS + (["scalar_phi"] if matter else [])
    og = gpu_origin_values(matter, fields)
    oo = oracle_origin_values(matter, fields)
    for k, f in enumerate(fields):
        cg, co = factors([v[k] for v in og]), factors([v[k] for v in oo])
        assert abs(cg - co) <= 1e-4 * abs(co), "%s: gpu factor %.6f oracle %.6f" % (f, cg, co)
        if f in ("trK", "scalar_phi") or (f == "phi" and not matter):
            assert 13.0 < cg < 20.0, "%s: convergence factor %.2f" % (f, cg)


def test_gpu_reproduces_order_two_convergence():
    """order = two: the device's factors equal the oracle's (second order in
    trK and KTA; the lapse and phi are pre-asymptotic at these resolutions)."""
    fields = ["alpha", "trK", "phi", "KTA"]
    og = gpu_origin_values(False, fields, order="two")
    oo = oracle_origin_values(False, fields, order="two")
    for k, f in enumerate(fields):
        cg, co = factors([v[k] for v in og]), factors([v[k] for v in oo])
        assert abs(cg - co) <= 1e-4 * abs(co), "%s: gpu factor %.6f oracle %.6f" % (f, cg, co)
        if f in ("trK", "KTA"):
            assert 3.5 < cg < 6.0, "%s: convergence factor %.2f" % (f, cg)
