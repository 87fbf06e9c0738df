"""Host side of the request loop (ollin_server_*, ollin_gpu_footprint): the
footprint bound and admission bookkeeping need no device, and the result
record's ctypes mirror matches the C layout."""
import ctypes
import os
import subprocess

import pytest

from parity_util import C1, params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_footprint_grows_with_the_hierarchy():
    from ollin.gpu import footprint
    r1, t1 = footprint(params(dict(C1, nrtotal=64, nztotal=64, nl0=1)))
    r2, _ = footprint(params(dict(C1, nrtotal=128, nztotal=128, nl0=1)))
    r3, _ = footprint(params(dict(C1, nrtotal=64, nztotal=64, nl0=3)))
    assert r1 < r2 and r1 < r3
    # an elliptic initial-data solve needs its arrays while it runs
    _, tp = footprint(params(dict(C1, idata="scalarpulse", mattertype="scalar", scalar_a0=0.05)))
    assert tp > 0
    # 4 slots + accumulator of every evolved slot and the auxiliary arrays
    # of a 1024^2 level are above 1 GB
    big, _ = footprint(params(dict(C1, nrtotal=1024, nztotal=1024, nl0=0)))
    assert big > 1 << 30


def test_footprint_takes_the_reference_ghost_and_boundary_choices():
    """main.f90:286-318 keeps a par-file ghost larger than the order needs
    (fewer is raised to the order's own), and boundtype takes none, static
    and flat beside radiative; more than 8 ghost zones is refused."""
    from ollin.gpu import OllinError, footprint
    from ollin.params import BOUND, params_from_par
    base, _ = footprint(params(C1))
    assert footprint(params(dict(C1, ghost=1)))[0] == base
    assert footprint(params(dict(C1, ghost=4)))[0] > base
    for b in ("none", "static", "flat"):
        footprint(params(dict(C1, boundtype=b)))
    p = params_from_par("boundtype = flat\nghost = 5\n")
    assert p.boundtype == BOUND["flat"] and p.ghost == 5
    with pytest.raises(OllinError):
        footprint(params(dict(C1, ghost=9)))


def test_footprint_rejects_what_create_rejects():
    from ollin.gpu import OllinError, footprint
    with pytest.raises(OllinError) as e:
        footprint(params(dict(C1, ghost=-1)))
    assert e.value.code == 1
    with pytest.raises(OllinError):
        footprint(params(dict(C1, Nb=1, Nl1=1, Nrbox1=200, Nzbox1=16, rbox1=1.0)))


def test_submit_checks_the_budget():
    from ollin.gpu import OllinError, Server, footprint
    p = params(C1)
    r, t = footprint(p)
    s = Server(r + t - 1)
    with pytest.raises(OllinError) as e:
        s.submit(1, p, 1.0)
    assert e.value.code == 4
    s2 = Server(r + t)
    s2.submit(1, p, 1.0)
    with pytest.raises(OllinError):
        s2.submit(2, p, -1.0)
    s2.close()


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="host has a GPU")
def test_request_without_a_device_fails_into_its_result():
    from ollin.gpu import Server
    s = Server(1 << 40, max_active=4)
    s.submit(7, params(C1), 0.5)
    res = s.drain()
    assert len(res) == 1 and res[0].id == 7 and res[0].status == 2 and res[0].steps == 0
    assert s.usage()[0] == 0


def test_result_layout_matches_header(tmp_path):
    from ollin.gpu import Result
    fields = [f for f, _ in Result._fields_]
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "ollin_gpu.h"', "int main(void){",
           'printf("%zu\\n", sizeof(ollin_result));']
    for f in fields:
        src.append('printf("%%zu\\n", offsetof(ollin_result, %s));' % f)
    src.append("return 0;}")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(Result)
    for f, off in zip(fields, out[1:]):
        assert getattr(Result, f).offset == off, f
