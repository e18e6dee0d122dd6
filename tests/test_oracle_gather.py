"""orc_gather_sums (the oracle of the render gather's per-hit-point export)
against the oracle's pinned estimate and in-radius set: the flux sums times
pw / (pi r2) are estimate_radiance, the counts are the kdtree `within` set
sizes, and the checksums are the sums of SplitMix64's output function over
those sets (computed here in numpy from orc_within's indices)."""
import numpy as np
import pytest

from oracle.binding import Oracle
from ppmpa_gb300 import scene as S


def slot_mix(i):
    z = (i.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


@pytest.mark.parametrize("pfilter", [S.FILTER_NONE, S.FILTER_CONE, S.FILTER_GAUSS])
def test_gather_sums_agree_with_estimate_and_within(pfilter):
    rng = np.random.default_rng(8)
    n, nq, r2, pw = 20000, 400, 0.06 ** 2, 0.003
    pos = rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    wl = rng.integers(0, 3, n).astype(np.uint8)
    q = rng.random((nq, 3))
    nrm = rng.normal(size=(nq, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    orc = Oracle(S.Scene(), threads=2)
    count, check, sums = orc.gather_sums(pos, d, wl, q, nrm, r2, pfilter)
    rgb = orc.estimate(pos, d, wl, q, nrm, r2, pw, pfilter)
    assert np.allclose(sums * (pw / (np.pi * r2)), rgb, rtol=1e-12, atol=0)
    off, idx = orc.within(pos, q, r2)
    assert np.array_equal(count, np.diff(off))
    want = np.zeros(nq, np.uint64)
    mixes = slot_mix(idx.astype(np.uint64))
    for i in range(nq):
        want[i] = np.sum(mixes[off[i]:off[i + 1]], dtype=np.uint64)
    assert np.array_equal(check, want)
    assert count.mean() > 10
