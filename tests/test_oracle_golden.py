"""The oracle against golden vectors produced by executing the reference's
own Fortran (tests/golden/make_golden.py): every stored grid function, every
level, every snapshot, including ghosts and the derived constraint arrays."""
import json
import os

import numpy as np
import pytest

from oracle_bind import Oracle
from parity_util import params, scalar_pulse

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["c1_small", "c2_small", "icn_harmonic", "scalar_shift"]

# The oracle restates the reference statement by statement; the remaining
# differences come from libm (exp/log/pow) last-bit differences amplified by
# the cancellation in nested derivatives.
TOL = 1e-9


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    return d, meta


def cfg_of(meta):
    skip = {"steps", "fields"}
    cfg = {k: v for k, v in meta.items() if k not in skip}
    cfg["eqsym"] = 1 if cfg.get("eqsym") else 0
    return cfg


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fortran(name):
    d, meta = load(name)
    cfg = cfg_of(meta)
    o = Oracle(params(cfg))
    o.initial_data()
    if cfg.get("mattertype") == "scalar":
        for lev in o.levels():
            nr, nz, g = o.dims(lev)
            r, z = o.get(lev, "r"), o.get(lev, "z")
            for nm, v in zip(["scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi"], scalar_pulse(r, z)):
                o.set(lev, nm, v)
    o.initialize()
    done = 0
    worst = 0.0
    for target in meta["steps"]:
        while done < target:
            o.step()
            done += 1
        for lev in o.levels():
            assert o.time(lev) == float(d["s%d_L%d_time" % (done, lev)])
            for nm in meta["fields"]:
                ref = d["s%d_L%d_%s" % (done, lev, nm)]
                got = o.get(lev, nm)
                scale = max(np.abs(ref).max(), 1e-300)
                err = np.abs(got - ref).max() / scale
                worst = max(worst, err)
                assert err <= TOL, "%s step %d level %d %s: rel %.3e" % (name, done, lev, nm, err)
            key = "s%d_L%d_ham" % (done, lev)
            if key in d:
                o.constraints(lev)
                for nm in ["ham", "mom_r", "mom_z", "RSCAL", "KT2", "Lapla_alpha"]:
                    ref = d["s%d_L%d_%s" % (done, lev, nm)]
                    got = o.get(lev, nm)
                    # interior points: the reference leaves the ghosts of
                    # mom_r/mom_z as computed, the comparison covers i,j >= 1
                    g = 3
                    ref_i, got_i = ref[g:, g:], got[g:, g:]
                    scale = max(np.abs(ref_i).max(), 1e-300)
                    err = np.abs(got_i - ref_i).max() / scale
                    assert err <= TOL, "%s step %d level %d %s: rel %.3e" % (name, done, lev, nm, err)
    print("%s: worst relative difference %.2e" % (name, worst))


def test_golden_fixture_inventory():
    for name in CASES:
        d, meta = load(name)
        assert meta["steps"][0] == 0 and len(meta["fields"]) >= 16
        assert "s0_L0_alpha" in d
