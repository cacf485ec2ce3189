"""Seeded workload generators: shapes, zero mean, determinism, periodicity."""
import numpy as np

import workloads


def test_uniform_rhs():
    b = workloads.uniform_rhs(16, 0)
    assert b.shape == (16, 16, 16)
    assert abs(b.mean()) < 1e-15
    assert np.array_equal(b, workloads.uniform_rhs(16, 0))
    assert b.max() <= 0.5 + 0.02 and b.min() >= -0.5 - 0.02  # U[-0.5,0.5] minus its sample mean
    assert workloads.uniform_rhs((5, 6, 7), 1).shape == (7, 6, 5)


def test_blob_rhs_is_periodic_sum_of_gaussians():
    n = 32
    b = workloads.blob_rhs(n, seed=3, blobs=4, width=0.05)
    assert abs(b.mean()) < 1e-12
    # direct evaluation of one configuration
    rng = np.random.default_rng(3)
    c = rng.uniform(0, 1, size=(4, 3))
    s = rng.choice(np.array([-1.0, 1.0]), size=4)
    x = np.arange(n) / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    ref = np.zeros((n, n, n))
    for k in range(4):
        d = [np.minimum(np.abs(G - c[k, a]), 1 - np.abs(G - c[k, a])) for a, G in ((0, X), (1, Y), (2, Z))]
        ref += s[k] * np.exp(-(d[0] ** 2 + d[1] ** 2 + d[2] ** 2) / (2 * 0.05 ** 2))
    ref -= ref.mean()
    assert np.allclose(b, ref, atol=1e-12)


def test_batches():
    hb = workloads.helmholtz_batch(count=5)
    assert len(hb) == 5
    for n, sigma, b in hb:
        assert n in (32, 48, 64, 96, 128, 160)
        assert 0 <= sigma.real <= 50 and 1 <= sigma.imag <= 50
        assert b.shape == (n, n, n) and np.iscomplexobj(b)
    db = workloads.differentiable_batch(count=2, n=8)
    assert len(db) == 2 and db[0][1].shape == (8, 8, 8)
