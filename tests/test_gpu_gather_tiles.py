"""Tiling of the canonical gather (k_gather_tiled.cu).

Each warp stages its cell's 3x3x3 neighbourhood in shared-memory tiles,
queries are sorted by cell and sub-cell, and staged photons farther than r
from the box of a warp's queries are dropped. The result of a query must
not depend on which queries share its warp or on how a neighbourhood is cut
into tiles. The cases are dense clusters (thousands of photons per
neighbourhood, many tiles per cell), sparse photons over many cells (warps
spanning cells), and queries out of reach of every photon. They are checked
against the float64 restatement query by query (every difference explained
by a photon on the sphere or a perpendicular normal) and, bit for bit, under
a permutation of the queries.
"""
import numpy as np
import pytest

from test_gpu_stages import check_canonical_gather, pack_normals

pytestmark = pytest.mark.gpu


def _unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _photons(rng, n, centers, spread):
    pos = centers[rng.integers(0, len(centers), n)] + rng.normal(size=(n, 3)) * spread
    nrm = rng.normal(size=(n, 3))
    nrm[: n // 2] = [0, 1, 0]
    nrm = _unit(nrm)
    ph8 = np.zeros((n, 8), np.float32)
    ph8[:, :3] = pos
    ph8[:, 3:6] = rng.uniform(0.1, 1.0, (n, 3))
    ph8[:, 6] = pack_normals(nrm)
    return ph8, nrm


def _queries(rng, m, centers, spread):
    pos = centers[rng.integers(0, len(centers), m)] + rng.normal(size=(m, 3)) * spread
    nrm = rng.normal(size=(m, 3))
    nrm[: m // 2] = [0, 1, 0]
    return np.concatenate([pos, _unit(nrm), rng.uniform(0.2, 0.9, (m, 3)), rng.uniform(0.5, 2.0, (m, 3))],
                          1).astype(np.float32)


def test_dense_clusters(ctx):
    rng = np.random.default_rng(11)
    centers = np.array([[0.0, 0.0, 0.0], [3.0, 1.0, -2.0], [-4.0, 2.5, 1.0]])
    ph8, nrm = _photons(rng, 30000, centers, 0.6)
    q = _queries(rng, 1500, centers, 0.6)
    r = 0.45
    out = ctx.gather(1, ph8, q, r)
    assert (out.sum(1) > 0).mean() > 0.9  # most queries gather many photons
    check_canonical_gather(out, ph8, nrm, q, r, "dense clusters")


def test_sparse_many_cells(ctx):
    rng = np.random.default_rng(12)
    ph8, nrm = _photons(rng, 20000, np.zeros((1, 3)), 6.0)
    q = _queries(rng, 3000, np.zeros((1, 3)), 6.0)
    r = 0.9
    out = ctx.gather(1, ph8, q, r)
    check_canonical_gather(out, ph8, nrm, q, r, "sparse cells")


def test_permutation_is_bit_identical(ctx):
    rng = np.random.default_rng(13)
    centers = np.array([[0.0, 0.0, 0.0], [1.2, 0.0, 0.4]])
    ph8, _ = _photons(rng, 25000, centers, 0.8)
    # fluxes that are small powers of two: every partial sum is exact, so the
    # result does not depend on the order of the photons within a bucket
    # (the grid build scatters them with atomics) but only on which photons
    # each query gathers
    ph8[:, 3:6] = rng.choice(np.float32([0.25, 0.5, 1.0, 2.0]), (len(ph8), 3))
    q = _queries(rng, 4000, centers, 0.9)
    r = 0.35
    out = ctx.gather(1, ph8, q, r)
    assert (out.sum(1) > 0).mean() > 0.9
    for seed in (1, 2):
        perm = np.random.default_rng(seed).permutation(len(q))
        outp = ctx.gather(1, ph8, q[perm], r)
        np.testing.assert_array_equal(outp, out[perm])


def test_queries_out_of_reach(ctx):
    rng = np.random.default_rng(14)
    ph8, _ = _photons(rng, 5000, np.zeros((1, 3)), 0.5)
    # inside the photons' box but more than r from all of them, and far outside it
    q = _queries(rng, 200, np.array([[40.0, 0.0, 0.0], [0.0, -30.0, 5.0]]), 0.1)
    out = ctx.gather(1, ph8, q, 0.3)
    assert np.all(out == 0.0)
