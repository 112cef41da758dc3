"""The allocation-free CG entry point against the allocating one.

mpg_cg_csr_noalloc exists for callers that cannot allocate device memory at
the call: a framework that owns all device memory through its own pool, a
real-time loop that must not pay for an allocation, a host that only lends
out device pointers.  It keeps its scratch in a static device array of the
library, so this test checks that its answers equal those of mpg_cg_csr
(which keeps scratch in a context) on two calls in a row (the second call
reuses the array the first one left behind), on a caller's own stream, on a
smaller matrix solved after a larger one (the array still holds the larger
call's vectors), and that a matrix larger than the static array is refused.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _p(t):
    return C.c_void_p(t.data_ptr())


def _solve_both(mpg, L, ctx, torch, n, d_rp, d_col, d_val, b, tol, max_iter, stream=None):
    """x from mpg_cg_csr and from mpg_cg_csr_noalloc (on `stream`, a torch
    stream, or the default stream), with iteration counts and residuals."""
    d_b = _dev(torch, b)
    x_ctx = torch.zeros(n, dtype=torch.float64, device="cuda")
    x_na = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    it1, r1 = C.c_int(), C.c_double()
    rc = L.mpg_cg_csr(ctx.h, n, _p(d_rp), _p(d_col), _p(d_val), _p(d_b), _p(x_ctx), tol, max_iter, C.byref(it1),
                      C.byref(r1))
    assert rc == mpg.OK, ctx.last_error()
    it2, r2 = C.c_int(), C.c_double()
    handle = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = L.mpg_cg_csr_noalloc(handle, n, _p(d_rp), _p(d_col), _p(d_val), _p(d_b), _p(x_na), tol, max_iter,
                              C.byref(it2), C.byref(r2))
    assert rc == mpg.OK, rc
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    return x_ctx.cpu().numpy(), it1.value, x_na.cpu().numpy(), it2.value, r2.value


def test_noalloc_cg_on_a_stream_and_after_a_larger_matrix(mpg, orc):
    torch = pytest.importorskip("torch")
    L = mpg.load()
    ctx = mpg.Ctx(0)
    rng = np.random.default_rng(12)
    tol, max_iter = 1e-10, 5000
    stream = torch.cuda.Stream()
    # the larger matrix first, then a smaller one: the static array still
    # holds the first call's vectors beyond the second call's rows
    for n_side, jitter in ((14, 0.2), (7, 0.1)):
        m = orc.Mesh(n_side, split=6, mapping=4, jitter=jitter, seed=5)
        rp, col, val = m.assemble(1)
        n = m.N
        assert n <= mpg.NOALLOC_MAX_N
        d_rp, d_col, d_val = _dev(torch, rp), _dev(torch, col), _dev(torch, val)
        b = rng.standard_normal(n)
        b[m.boundary == 1] = 0.0
        a, it1, c, it2, r2 = _solve_both(mpg, L, ctx, torch, n, d_rp, d_col, d_val, b, tol, max_iter, stream)
        assert it2 == it1, (n_side, it1, it2)
        assert np.abs(c - a).max() <= 1e-12 * np.abs(a).max(), n_side
        assert r2 < tol
        assert np.linalg.norm(b - m.spmv(c)) <= 1e-9 * np.linalg.norm(b)


def test_noalloc_cg_matches_allocating_entry_point(mpg, orc):
    torch = pytest.importorskip("torch")
    L = mpg.load()
    m = orc.Mesh(12, split=6, mapping=4, jitter=0.2, seed=3)
    rp, col, val = m.assemble(1)
    n = m.N
    assert n <= mpg.NOALLOC_MAX_N
    d_rp, d_col, d_val = _dev(torch, rp), _dev(torch, col), _dev(torch, val)
    ctx = mpg.Ctx(0)
    rng = np.random.default_rng(11)
    tol, max_iter = 1e-10, 5000
    for call in range(2):
        b = rng.standard_normal(n)
        b[m.boundary == 1] = 0.0
        d_b = _dev(torch, b)
        x_ctx = torch.zeros(n, dtype=torch.float64, device="cuda")
        x_na = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        it1, r1 = C.c_int(), C.c_double()
        rc = L.mpg_cg_csr(ctx.h, n, _p(d_rp), _p(d_col), _p(d_val), _p(d_b), _p(x_ctx), tol, max_iter,
                          C.byref(it1), C.byref(r1))
        assert rc == mpg.OK, ctx.last_error()
        it2, r2 = C.c_int(), C.c_double()
        rc = L.mpg_cg_csr_noalloc(None, n, _p(d_rp), _p(d_col), _p(d_val), _p(d_b), _p(x_na), tol, max_iter,
                                  C.byref(it2), C.byref(r2))
        assert rc == mpg.OK, rc
        torch.cuda.synchronize()
        a = x_ctx.cpu().numpy()
        c = x_na.cpu().numpy()
        assert it2.value == it1.value, (call, it1.value, it2.value)
        assert np.abs(c - a).max() <= 1e-12 * np.abs(a).max(), call
        assert r2.value < tol
        assert np.linalg.norm(b - m.spmv(c)) <= 1e-9 * np.linalg.norm(b)
    # a matrix larger than the static scratch is refused before anything runs
    it3, r3 = C.c_int(-7), C.c_double()
    big = mpg.NOALLOC_MAX_N + 1
    rc = L.mpg_cg_csr_noalloc(None, big, _p(d_rp), _p(d_col), _p(d_val), _p(d_b), _p(x_na), tol, max_iter,
                              C.byref(it3), C.byref(r3))
    assert rc == mpg.ERR_CAPACITY
    assert it3.value == -7
