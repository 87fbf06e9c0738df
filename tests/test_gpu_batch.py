"""Several independent evolutions stepped together
(ollin_gpu_coarse_step_many): each gives, bit for bit, what it gives when
stepped alone, and a non-finite value in one of them is reported."""
import numpy as np
import pytest

from parity_util import C1, field_list, params

pytestmark = pytest.mark.gpu

CFGS = [
    dict(C1, nrtotal=32, nztotal=32, nl0=1),
    dict(C1, nrtotal=24, nztotal=40, nl0=2, shift="Gammadriver2", drivercsi=0.75, drivereta=2.0),
    dict(C1, nrtotal=40, nztotal=24, nl0=0, integrator="icn", icniter=3, slicing="harmonic", gauge_f=1.0),
]


def make(cfg):
    from ollin.gpu import Evolution
    e = Evolution(params(cfg))
    e.initial_data()
    e.initialize()
    return e


def test_batched_steps_equal_single_steps():
    from ollin.gpu import step_many
    alone = [make(c) for c in CFGS]
    batch = [make(c) for c in CFGS]
    for _ in range(3):
        t_alone = [e.step() for e in alone]
        t_batch = step_many(batch)
        assert t_alone == t_batch
    for cfg, a, b in zip(CFGS, alone, batch):
        for lev in a.levels():
            for nm in field_list(cfg):
                assert np.array_equal(a.download(lev, nm), b.download(lev, nm)), (lev, nm)


def test_batched_step_reports_nan():
    from ollin.gpu import OllinError, step_many
    es = [make(c) for c in CFGS[:2]]
    a = es[1].download(0, "alpha")
    a[5, 5] = np.nan
    es[1].upload(0, "alpha", a)
    with pytest.raises(OllinError) as ex:
        step_many(es)
    assert ex.value.code == 3
