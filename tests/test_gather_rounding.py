"""Rounding of the canonical gather's distance test (k_gather_tiled.cu).

The kernel tests a photon p against a query q in coordinates relative to
the centre c of the query's grid cell: the tile holds p' = p - c and
|p'|^2, each lane -2 q' and r^2 - |q'|^2, and the photon counts when
fma(-2q'z, p'z, fma(-2q'y, p'y, fma(-2q'x, p'x, |p'|^2))) < r^2 - |q'|^2.
This restates that FP32 arithmetic in numpy (an FMA as the float64 sum of
the exact product, rounded once) and checks that the error of d^2 - r^2
stays inside the band in which the float64 restatement of the gather
counts a photon as on the sphere (1e-5 r^2): the only photons whose
classification may differ from the restatement's are listed as ambiguous
by the parity tests.
"""
import numpy as np
import pytest

f32 = np.float32
BAND = 1e-5  # relative in r^2, as the gather parity bounds


def _fma(a, b, c):
    # a * b of two floats is exact in float64; one rounding to float32
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def _sq(v, contract):
    # x*x + y*y + z*z in FP32: as fma(z, z, fma(y, y, x*x)) when the device
    # compiler contracts the products into the sums (its default), else
    # with a rounding after every operation; the bound holds for both
    if contract:
        return _fma(v[:, 2], v[:, 2], _fma(v[:, 1], v[:, 1], (v[:, 0] * v[:, 0]).astype(f32)))
    s = (v[:, 0] * v[:, 0]).astype(f32) + (v[:, 1] * v[:, 1]).astype(f32)
    return (s.astype(f32) + (v[:, 2] * v[:, 2]).astype(f32)).astype(f32)


@pytest.mark.parametrize("contract", [True, False])
@pytest.mark.parametrize("cell_factor,bound", [(1.0, 2e-6), (1.5, 2e-6), (2.0, 2.5e-6), (4.0, 5e-6)])
def test_cell_centred_test_stays_inside_the_band(cell_factor, bound, contract):
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(12):
        r = f32(10.0 ** rng.uniform(-3, 1))
        cell = f32(cell_factor * r)
        org = f32(rng.uniform(-500, 500))
        lc = rng.integers(0, 200, 3).astype(f32)
        cc = (org + (lc + f32(0.5)) * cell).astype(f32)
        n = 100_000
        q = (org + (lc + rng.uniform(0, 1, (n, 3))) * cell).astype(f32)
        # photons around the sphere's surface (|p - q| within 10 % of r)
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        p = (q.astype(np.float64) + u * float(r) * rng.uniform(0.9, 1.1, (n, 1))).astype(f32)
        qp = (q - cc).astype(f32)
        pp = (p - cc).astype(f32)
        m = (f32(-2.0) * qp).astype(f32)
        lhs = _fma(m[:, 2], pp[:, 2], _fma(m[:, 1], pp[:, 1], _fma(m[:, 0], pp[:, 0], _sq(pp, contract))))
        thr = (f32(r) * f32(r) - _sq(qp, contract)).astype(f32)
        exact = ((p.astype(np.float64) - q.astype(np.float64)) ** 2).sum(1) - float(r) ** 2
        err = np.abs((lhs.astype(np.float64) - thr.astype(np.float64)) - exact) / float(r) ** 2
        worst = max(worst, float(err.max()))
    assert worst < bound <= BAND, worst


@pytest.mark.parametrize("contract", [True, False])
def test_classification_differs_only_inside_the_band(contract):
    """Photons the FP32 test classifies differently from the exact
    distance all lie within the band around the sphere."""
    rng = np.random.default_rng(12)
    r, cell = f32(0.37), f32(0.37)
    org = f32(-3.0)
    lc = np.array([4, 9, 2], np.float32)
    cc = (org + (lc + f32(0.5)) * cell).astype(f32)
    n = 400_000
    q = (org + (lc + rng.uniform(0, 1, (n, 3))) * cell).astype(f32)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    p = (q.astype(np.float64) + u * float(r) * (1.0 + rng.uniform(-1e-5, 1e-5, (n, 1)))).astype(f32)
    qp, pp = (q - cc).astype(f32), (p - cc).astype(f32)
    m = (f32(-2.0) * qp).astype(f32)
    inside32 = _fma(m[:, 2], pp[:, 2], _fma(m[:, 1], pp[:, 1], _fma(m[:, 0], pp[:, 0], _sq(pp, contract)))) < \
        (f32(r) * f32(r) - _sq(qp, contract)).astype(f32)
    d2 = ((p.astype(np.float64) - q.astype(np.float64)) ** 2).sum(1)
    inside64 = d2 < float(r) ** 2
    differ = inside32 != inside64
    assert differ.any()  # the sample does reach the rounding
    assert np.all(np.abs(d2[differ] - float(r) ** 2) <= BAND * float(r) ** 2)
