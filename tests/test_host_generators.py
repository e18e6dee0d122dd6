"""Host-side generators of the synthetic workloads (CPU): the icosphere
mesh, the seeded photon / query sets of the gather sweep, and the numpy
restatement of the FP32 map's packed directions."""
import numpy as np

from ppmpa_gb300 import mesh as M, workloads as W


def test_icosphere_counts_orientation_and_radius():
    for level in range(4):
        v, f = M.icosphere(level)
        assert len(f) == 20 * 4 ** level
        assert len(v) == 10 * 4 ** level + 2                       # Euler: V = F/2 + 2
        assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
        n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
        assert (np.einsum("ij,ij->i", n, v[f].sum(1)) > 0).all()    # counter-clockwise seen from outside
        edges = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
        _, counts = np.unique(edges, axis=0, return_counts=True)
        assert (counts == 2).all()                                   # closed: every edge shared by two faces


def test_displaced_icosphere_stays_within_its_amplitude():
    v, f = M.displaced_icosphere(3, (0.0, 0.75, 1.0), 0.55, amplitude=0.05, seed=1)
    r = np.linalg.norm(v - np.array([0.0, 0.75, 1.0]), axis=1)
    assert r.min() >= 0.55 * 0.95 - 1e-12 and r.max() <= 0.55 * 1.05 + 1e-12
    assert r.std() > 1e-4                                            # the noise does displace
    v2, _ = M.displaced_icosphere(3, (0.0, 0.75, 1.0), 0.55, amplitude=0.05, seed=1)
    assert np.array_equal(v, v2)                                     # seeded


def test_mesh_scene_size_and_materials():
    sc = M.mesh_scene(level=2)
    assert sc.n_objects == 5 + 20 * 4 ** 2
    assert len(sc.lights) == 1


def test_sweep_photons_and_queries_are_seeded_and_in_range():
    for kind in ("uniform", "clustered"):
        p1, d1, w1 = W.photons(50000, kind)
        p2, d2, w2 = W.photons(50000, kind)
        assert np.array_equal(p1, p2) and np.array_equal(d1, d2) and np.array_equal(w1, w2)
        assert p1.dtype == np.float32 and d1.dtype == np.float32 and w1.dtype == np.uint8
        assert np.allclose(np.linalg.norm(d1.astype(np.float64), axis=1), 1.0, atol=1e-6)
        assert set(np.unique(w1)) <= {0, 1, 2}
        q, n, r2 = W.queries(20000, kind)
        r = np.sqrt(r2)
        assert r.min() >= W.R_MIN * (1 - 1e-12) and r.max() <= W.R_MAX * (1 + 1e-12)
        assert np.allclose(np.linalg.norm(n.astype(np.float64), axis=1), 1.0, atol=1e-6)
    # clustered: about 90 % of the photons lie within a few sigma of a blob centre
    p, _, _ = W.photons(20000, "clustered")
    c = W._centres(W.PHOTON_SEED).astype(np.float64)
    d2 = ((p.astype(np.float64)[:, None, :] - c[None, :, :]) ** 2).sum(-1).min(1)
    near = np.sqrt(d2) < 5 * W.BLOB_SIGMA
    assert 0.88 < near.mean() < 0.93


def test_oct_roundtrip_error_is_small():
    rng = np.random.default_rng(3)
    d = rng.normal(size=(100000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    e = W.oct_roundtrip(d)
    assert np.allclose(np.linalg.norm(e, axis=1), 1.0)
    ang = np.arccos(np.clip(np.einsum("ij,ij->i", d, e), -1.0, 1.0))
    assert ang.max() < 2e-4                                          # 15+15-bit octahedral codes
