"""Coarse steps recorded by stream capture and launched as one CUDA graph
(ollin_gpu_step_graphs): the same kernels, arguments and order as direct
launches, so every field is the same bit for bit, through the first steps,
maximal-slicing solves and syncboxes copies, whose launch structure differs
from the step before."""
import numpy as np
import pytest

from parity_util import C1, field_list, params

pytestmark = pytest.mark.gpu

CASES = {
    "puncture_3_levels": (dict(C1, nrtotal=32, nztotal=32, nl0=2), 0),
    "shift_advect": (dict(C1, nrtotal=40, nztotal=24, nl0=1, shift="Gammadriver2", drivercsi=0.75, drivereta=2.0), 0),
    "scalar_pulse": (dict(eqsym=1, order="four", integrator="rk4", ilapse="one", slicing="1+log", gauge_f=2.0,
                          geodiss=0.02, dtfac=0.25, boundtype="radiative", nrtotal=32, nztotal=32, nl0=1, dr0=0.4,
                          dz0=0.4, idata="scalarpulse", mattertype="scalar", scalar_a0=0.05, scalar_r0=3.0,
                          scalar_z0=3.0, scalardiss=0.02, we_maxiter=200), 0),
    "overlapping_boxes": (dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, Nb=1, Nl1=1, Nrbox1=16,
                               Nzbox1=16, zbox1=2.0), 0),
    "maximal_every_step": (dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, we_maxiter=150), 1),
    "icn_no_eqsym": (dict(C1, nrtotal=24, nztotal=24, nl0=1, eqsym=0, integrator="icn", icniter=3), 0),
}


@pytest.mark.parametrize("name", list(CASES))
def test_graph_steps_equal_direct_steps(name):
    from ollin.gpu import Evolution
    cfg, every = CASES[name]
    ev = []
    for graphs in (False, True):
        e = Evolution(params(cfg))
        e.initial_data()
        e.initialize()
        e.step_graphs(graphs)
        if every:
            e.maximal_slicing()
        ev.append(e)
    direct, graph = ev
    for k in range(1, 7):
        ts = []
        for e in ev:
            e.step_begin()
            ts.append(e.step_end())
            if every and k % every == 0:
                e.maximal_slicing()
        assert ts[0] == ts[1]
    for lev in direct.levels():
        for nm in field_list(cfg):
            assert np.array_equal(direct.download(lev, nm), graph.download(lev, nm)), (lev, nm)
    inst, upd = graph.step_graphs()
    assert inst + upd == 6 and inst >= 1
    if not every:
        assert upd >= 3  # steady steps reuse the executable graph
    assert direct.step_graphs() == (0, 0)


def test_coarse_step_honours_graph_mode():
    """ollin_gpu_coarse_step launches the captured graph too."""
    from ollin.gpu import Evolution
    cfg = CASES["puncture_3_levels"][0]
    ev = []
    for graphs in (False, True):
        e = Evolution(params(cfg))
        e.initial_data()
        e.initialize()
        e.step_graphs(graphs)
        ev.append(e)
    for _ in range(5):
        assert ev[0].step() == ev[1].step()
    for lev in ev[0].levels():
        for nm in field_list(cfg):
            assert np.array_equal(ev[0].download(lev, nm), ev[1].download(lev, nm)), (lev, nm)
    assert sum(ev[1].step_graphs()) == 5


@pytest.mark.parametrize("name", ["puncture_3_levels", "overlapping_boxes"])
def test_chained_launches_equal_ordinary_launches(name):
    """The kernels of a step as a programmatic dependent chain (each waits on
    the device for its predecessor) give the fields of ordinary launches."""
    from ollin.gpu import Evolution
    cfg, _ = CASES[name]
    ev = []
    for chain in (False, True):
        e = Evolution(params(cfg))
        e.initial_data()
        e.initialize()
        e.step_chaining(chain)
        ev.append(e)
    for _ in range(4):
        assert ev[0].step() == ev[1].step()
    for lev in ev[0].levels():
        for nm in field_list(cfg):
            assert np.array_equal(ev[0].download(lev, nm), ev[1].download(lev, nm)), (lev, nm)
