"""Dipole BSSRDF parity: DipoleBSSRDF::operator() and the octree irradiance
sum of SubsurfaceIntegrator against the reference's outputs.

Rd is computed in FP32 except the reference's fast_exp staircase, whose
integer argument is formed exactly, so Rd agrees to 1e-5 relative wherever
it is not vanishingly small. The hierarchical sum takes a node whole when
area/d^2 < max_error; a node whose FP32 ratio lands on the other side of the
threshold than the reference's double one changes the approximation, so such
boundary queries are counted and bounded instead of compared."""
import numpy as np
import pytest

import scenes as S

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def _mat(g, k):
    return g[f"mat{k}"].view(S.MATERIAL_DTYPE)[0]


@pytest.mark.parametrize("k", [0, 1, 2])
def test_dipole_rd(ctx, golden, k):
    g = golden("dipole")
    out = ctx.dipole_rd(_mat(g, k), g["d2"]).astype(np.float64)
    ref = g[f"rd{k}"]
    scale = np.abs(ref).max()
    ok = np.abs(out - ref) <= RTOL * np.abs(ref) + 1e-7 * scale
    assert ok.mean() > 0.999, (ok.mean(), np.argwhere(~ok)[:5])


@pytest.mark.parametrize("k", [0, 1, 2])
@pytest.mark.parametrize("e", [0, 1])
def test_dipole_irradiance(ctx, golden, k, e):
    g = golden("dipole")
    me = (0.05, 0.5)[e]
    out = ctx.dipole_irradiance(_mat(g, k), g["ipts"], me, g["queries"]).astype(np.float64)
    ref = g[f"irr{k}_{e}"]
    scale = np.abs(ref).max()
    ok = np.all(np.abs(out - ref) <= RTOL * np.abs(ref) + 1e-7 * scale, axis=1)
    assert ok.mean() > 0.99, ok.mean()
    # where a threshold decision flipped, the result is still the same sum to
    # within the approximation the threshold controls
    assert np.all(np.abs(out - ref) <= 0.05 * np.abs(ref) + 1e-6 * scale)


def test_fast_exp_integer_form_exhaustive(ctx):
    # every float argument: the integer form used by the render agrees bit
    # for bit with the double form wherever it applies (|y| <= 700)
    covered, differ = ctx.fast_exp_check(0, 1 << 32)
    assert differ == 0
    # 0 and the floats of (0, 700] in both signs
    n_pos = int(np.array([700.0], np.float32).view(np.uint32)[0])
    assert covered == 2 * (n_pos + 1)

