"""ppm_estimate_noalloc (the estimate staged in a fixed device array, with no
device allocation) against ppm_estimate on the same photon map and queries.

Two calls in a row go through the C ABI: the first fills the whole array
(the maximum query count), the second is smaller, so a row left over from
the first call would show up as a mismatch.  Tolerance is the FP64 estimate
bar used by the parity tests (1e-9 relative).

The entry point exists for callers that cannot let the library allocate
device memory once they are running, so the test also reads the device's
free memory (cudaMemGetInfo, through torch) before the context's first call
of the entry point and after its last: it must not move.  The array and the
kernels the entry point uses are placed when the context is created.
"""
import ctypes as C

import numpy as np
import pytest

from ppmpa_gb300 import Context, _lib, scene as S

pytestmark = pytest.mark.gpu

MAX_Q = 32768   # PPM_ESTIMATE_NOALLOC_MAX_QUERIES in include/ppm_api.h


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def _queries(rng, n):
    q = rng.random((n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return np.ascontiguousarray(q), np.ascontiguousarray(nrm)


def _noalloc(lib, ctx, q, nrm, pfilter):
    rgb = np.full((q.shape[0], 3), np.nan)
    st = lib.ppm_estimate_noalloc(ctx.h, _p(q), _p(nrm), q.shape[0], pfilter, _p(rgb))
    assert st == 0, lib.ppm_last_error(ctx.h).decode()
    return rgb


def _free_device_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def test_noalloc_estimate_matches_estimate_on_two_calls_in_a_row(built_lib):
    lib = _lib.load(built_lib)
    rng = np.random.default_rng(2024)
    npho = 80000
    pos = rng.random((npho, 3))
    d = rng.normal(size=(npho, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    wl = rng.integers(0, 3, npho).astype(np.uint8)
    r2, power = 0.04 ** 2, 0.002
    qa, na = _queries(rng, MAX_Q)
    qb, nb = _queries(rng, 5000)
    ctx = Context(0, seed=7)
    try:
        ctx.build_photonmap(pos, d, wl, power, r2)
        want_a = ctx.estimate(qa, na, S.FILTER_CONE)
        want_b = ctx.estimate(qb, nb, S.FILTER_GAUSS)
        ctx.sync()
        free_before = _free_device_bytes()   # before this context's first allocation-free call
        got_a = _noalloc(lib, ctx, qa, na, S.FILTER_CONE)
        got_b = _noalloc(lib, ctx, qb, nb, S.FILTER_GAUSS)
        assert np.allclose(got_a, want_a, rtol=1e-9, atol=1e-12)
        assert np.allclose(got_b, want_b, rtol=1e-9, atol=1e-12)
        assert (want_a > 0).mean() > 0.3 and (want_b > 0).mean() > 0.3
        again = _noalloc(lib, ctx, qa, na, S.FILTER_CONE)
        assert np.array_equal(again, got_a)
        assert _free_device_bytes() == free_before, "the allocation-free estimate changed free device memory"

        # one query more than the array holds is refused before any device work
        big_q = np.zeros((MAX_Q + 1, 3))
        out = np.zeros((MAX_Q + 1, 3))
        st = lib.ppm_estimate_noalloc(ctx.h, _p(big_q), _p(big_q), MAX_Q + 1, S.FILTER_NONE, _p(out))
        assert st == 1
        assert b"at most 32768" in lib.ppm_last_error(ctx.h)
    finally:
        ctx.close()
