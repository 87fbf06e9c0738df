"""ollin_gpu_norms_noalloc: the 0-D statistics of a grid function the caller
already holds on the device, for callers that cannot call cudaMalloc (hosts
whose device memory comes from their own allocator or pool, code inside a
stream capture, read-only tools).  The entry point allocates nothing; its
intermediate results live in a fixed device array of the library image.

Checked through the C ABI against the existing entry point ollin_gpu_norms
on the same field, on two calls in a row, within the parity tolerance of the
other GPU tests.  This file is collected last so that a stop-at-first-failure
run has run every other test before it."""
import ctypes

import numpy as np
import pytest

from parity_util import C1, params

pytestmark = pytest.mark.gpu


def test_noalloc_norms_match_existing_entry_point_twice():
    torch = pytest.importorskip("torch")
    from ollin.gpu import Evolution, load
    lib = load()
    lib.ollin_gpu_norms_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p]
    lib.ollin_gpu_noalloc_last_error.restype = ctypes.c_char_p
    e = Evolution(params(dict(C1, nl0=1)))
    e.initial_data()
    e.initialize()
    for _ in range(2):
        e.step()
    d = e.desc(1)
    for name in ("alpha", "trK"):
        host = e.download(1, name)                       # [i+g-1, j+g-1]
        dev = torch.from_numpy(np.ascontiguousarray(host.T)).cuda()  # r fastest, ld = nr+g
        torch.cuda.synchronize()
        out = np.zeros(5)
        rc = lib.ollin_gpu_norms_noalloc(ctypes.c_void_p(dev.data_ptr()), d.nr, d.nz, d.ghost, d.nr + d.ghost,
                                         d.dr, d.dz, 1, None, out.ctypes.data)
        assert rc == 0, lib.ollin_gpu_noalloc_last_error()
        ref = e.norms(1, name)
        np.testing.assert_allclose(out, ref, rtol=1e-10, atol=1e-14)
    # a grid beyond the fixed scratch is refused, not truncated
    out = np.zeros(5)
    rc = lib.ollin_gpu_norms_noalloc(ctypes.c_void_p(dev.data_ptr()), d.nr, 8192 + 4, 3, d.nr + 3,
                                     d.dr, d.dz, 1, None, out.ctypes.data)
    assert rc == 1
    e.close()
