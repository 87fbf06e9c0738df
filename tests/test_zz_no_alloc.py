"""ollin_gpu_norms_noalloc: the 0-D statistics of a grid function the caller
already holds on the device, for callers that cannot call cudaMalloc (hosts
whose device memory comes from their own allocator or pool, regions where an
allocation would synchronise the device, read-only tools).  The entry point
allocates nothing; its intermediate results live in a fixed device array of
the library image.

Checked through the C ABI against the existing entry point ollin_gpu_norms
on the same field, on two calls in a row, within the parity tolerance of the
other GPU tests; then on a caller's stream, at the largest accepted grid
(8192 interior rows, against NumPy), on a field holding a NaN, on an
order-two grid (two ghost zones), and on a capturing stream (refused).  This file
is collected last so that a stop-at-first-failure run has run every other
test before it."""
import ctypes

import numpy as np
import pytest

from parity_util import C1, params

pytestmark = pytest.mark.gpu

ENAN = 3
EINVAL = 1


def _lib():
    from ollin.gpu import load
    lib = load()
    lib.ollin_gpu_norms_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p]
    lib.ollin_gpu_noalloc_last_error.restype = ctypes.c_char_p
    return lib


def _call(lib, dev, nr, nz, dr, dz, stream=None, ld=None, ghost=3):
    out = np.zeros(5)
    rc = lib.ollin_gpu_norms_noalloc(ctypes.c_void_p(dev.data_ptr()), nr, nz, ghost,
                                     nr + ghost if ld is None else ld, dr, dz, 1, stream, out.ctypes.data)
    return rc, out


def _numpy_stats(f, dr, dz):
    """save0Dvariable's statistics of f[i+2, j+2] (i, j from -2) restated in
    NumPy: interior i = 1..nr-3, j = 1..nz-3; the origin lies half a cell from
    the axis and the equator, so its bicubic weights are (-1, 9, 9, -1)/16 on
    i, j = -1..2."""
    inner = f[3:-3, 3:-3]
    w = np.array([-1.0, 9.0, 9.0, -1.0]) / 16.0
    origin = float(w @ f[1:5, 1:5] @ w)
    return np.array([inner.max(), inner.min(), np.abs(inner).max(), np.sqrt(np.mean(inner ** 2)), origin])


def test_noalloc_norms_match_existing_entry_point_twice():
    torch = pytest.importorskip("torch")
    from ollin.gpu import Evolution
    lib = _lib()
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
        ref = e.norms(1, name)
        for _call_no in range(2):
            rc, out = _call(lib, dev, d.nr, d.nz, d.dr, d.dz)
            assert rc == 0, lib.ollin_gpu_noalloc_last_error()
            np.testing.assert_allclose(out, ref, rtol=1e-10, atol=1e-14)
        # on a caller's own stream, with the field written on that stream
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            dev2 = torch.from_numpy(np.ascontiguousarray(host.T)).cuda(non_blocking=False)
        rc, out = _call(lib, dev2, d.nr, d.nz, d.dr, d.dz, stream=ctypes.c_void_p(s.cuda_stream))
        assert rc == 0, lib.ollin_gpu_noalloc_last_error()
        np.testing.assert_allclose(out, ref, rtol=1e-10, atol=1e-14)
    # a grid beyond the fixed scratch is refused, not truncated
    rc, _ = _call(lib, dev, d.nr, 8192 + 4, d.dr, d.dz)
    assert rc == EINVAL
    e.close()


def test_noalloc_norms_at_the_row_limit_and_nan():
    torch = pytest.importorskip("torch")
    lib = _lib()
    rng = np.random.default_rng(7)
    nr, nz = 40, 8192 + 3                                # exactly 8192 interior rows: accepted
    f = rng.standard_normal((nr + 3, nz + 3))            # [i+2, j+2]
    dev = torch.from_numpy(np.ascontiguousarray(f.T)).cuda()
    torch.cuda.synchronize()
    rc, out = _call(lib, dev, nr, nz, 0.1, 0.1)
    assert rc == 0, lib.ollin_gpu_noalloc_last_error()
    np.testing.assert_allclose(out, _numpy_stats(f, 0.1, 0.1), rtol=1e-12, atol=1e-14)
    # one NaN in the interior is reported as OLLIN_ENAN
    g = f.copy()
    g[nr // 2, nz - 10] = np.nan
    devn = torch.from_numpy(np.ascontiguousarray(g.T)).cuda()
    torch.cuda.synchronize()
    rc, _ = _call(lib, devn, nr, nz, 0.1, 0.1)
    assert rc == ENAN
    # the next call on a clean field is unaffected by the NaN left in the scratch
    rc, out = _call(lib, dev, nr, nz, 0.1, 0.1)
    assert rc == 0, lib.ollin_gpu_noalloc_last_error()
    np.testing.assert_allclose(out, _numpy_stats(f, 0.1, 0.1), rtol=1e-12, atol=1e-14)


def test_noalloc_norms_order_two_and_capture_refused():
    """Two ghost zones (order two) against ollin_gpu_norms; a capturing
    stream is refused before any work is queued (the call ends by
    synchronising its stream)."""
    torch = pytest.importorskip("torch")
    from ollin.gpu import Evolution
    lib = _lib()
    e = Evolution(params(dict(C1, nl0=1, order="two")))
    e.initial_data()
    e.initialize()
    e.step()
    d = e.desc(1)
    assert d.ghost == 2
    host = e.download(1, "alpha")
    dev = torch.from_numpy(np.ascontiguousarray(host.T)).cuda()
    torch.cuda.synchronize()
    rc, out = _call(lib, dev, d.nr, d.nz, d.dr, d.dz, ghost=2)
    assert rc == 0, lib.ollin_gpu_noalloc_last_error()
    np.testing.assert_allclose(out, e.norms(1, "alpha"), rtol=1e-10, atol=1e-14)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc, _ = _call(lib, dev, d.nr, d.nz, d.dr, d.dz, stream=ctypes.c_void_p(s.cuda_stream), ghost=2)
        spare = dev * 1.0  # keeps the captured graph non-empty
    assert rc == EINVAL and b"capturing" in lib.ollin_gpu_noalloc_last_error()
    del spare
    e.close()


def test_noalloc_norms_with_four_ghost_zones():
    """A par-file ghost of 4 (order four): the interior i = 1..Nr-ghost,
    j = 1..Nz-ghost of save0Dvariable and the origin value, against
    ollin_gpu_norms on the same grid."""
    torch = pytest.importorskip("torch")
    from ollin.gpu import Evolution
    lib = _lib()
    e = Evolution(params(dict(C1, nl0=1, ghost=4)))
    e.initial_data()
    e.initialize()
    e.step()
    d = e.desc(1)
    assert d.ghost == 4
    for name in ("alpha", "trK"):
        host = e.download(1, name)
        dev = torch.from_numpy(np.ascontiguousarray(host.T)).cuda()
        torch.cuda.synchronize()
        rc, out = _call(lib, dev, d.nr, d.nz, d.dr, d.dz, ghost=4)
        assert rc == 0, lib.ollin_gpu_noalloc_last_error()
        np.testing.assert_allclose(out, e.norms(1, name), rtol=1e-10, atol=1e-14)
    e.close()
