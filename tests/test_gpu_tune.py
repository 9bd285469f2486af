"""Launch-shape knobs (pppm_render_tune_ex): each setting renders the same
passes as the defaults. The photon paths, their deposits and the eye paths
are the same (counts equal); only the order in which deposits are appended,
and so the order of the gather's floating-point sums, may change: pixels
agree within 1e-4 relative (an FP32 sum of n terms reordered moves by at
most about n u, u = 2^-24, with n up to a few thousand photons)."""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu

DEFAULTS = dict(cell_factor=1.0, bounce_blocks_per_sm=64, eye_blocks_per_sm=128, refill=24, exact_batch=12,
                gather_stage=128, query_sub_bits=1)


def _render(ctx, sc, par, passes, knobs=None, graph=False):
    ctx.render_begin(sc.camera, par)
    if knobs:
        ctx.render_tune(**knobs)
    if graph:
        st = ctx.render_graph(passes)
    else:
        st = [ctx.render_pass(t) for t in range(1, passes + 1)]
    return ctx.render_read().astype(np.float64), st


def _close(img, ref):
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return float(np.max(np.abs(img - ref) / scale))


@pytest.mark.parametrize("mode", [P.MODE_CANONICAL, P.MODE_COMPAT])
def test_knobs_change_no_result(ctx, mode):
    sc = S.small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20_000)
    ctx.set_scene(sc)
    par = P.Context.make_params(mode=mode, photons=20_000, max_bounce_photon=16, max_bounce_eye=16,
                                radius_scale=1 / 32 if mode == P.MODE_CANONICAL else 0.1, seed=5, num_streams=8)
    ref, st0 = _render(ctx, sc, par, 4)
    assert ctx.get_tune() == pytest.approx(DEFAULTS)
    settings = [dict(refill=8, exact_batch=1), dict(refill=32, exact_batch=32, bounce_blocks_per_sm=2, eye_blocks_per_sm=3)]
    if mode == P.MODE_CANONICAL:
        settings += [dict(gather_stage=32, query_sub_bits=0), dict(gather_stage=256, query_sub_bits=3, cell_factor=1.5)]
    for knobs in settings:
        img, st = _render(ctx, sc, par, 4, knobs)
        got = ctx.get_tune()
        assert all(got[k] == pytest.approx(v) for k, v in knobs.items()), (knobs, got)
        for a, b in zip(st, st0):
            assert (a.photons_stored, a.photon_rays, a.eye_rays, a.gather_queries) == \
                   (b.photons_stored, b.photon_rays, b.eye_rays, b.gather_queries), knobs
        err = _close(img, ref)
        print(f"mode {mode} knobs {knobs}: max relative pixel difference {err:.2e}")
        assert err < 1e-4, (knobs, err)


def test_knobs_apply_inside_a_graph(ctx):
    sc = S.small_test_scene(seed=4, subdiv=3, width=64, height=48, photons=20_000)
    ctx.set_scene(sc)
    par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=20_000, max_bounce_photon=16, max_bounce_eye=16,
                                radius_scale=1 / 32, seed=6)
    ref, _ = _render(ctx, sc, par, 5)
    img, _ = _render(ctx, sc, par, 5, dict(gather_stage=64, query_sub_bits=2, refill=16, exact_batch=4), graph=True)
    assert _close(img, ref) < 1e-4


def test_knob_ranges(ctx):
    sc = S.small_test_scene(seed=3, subdiv=2, width=16, height=16, photons=2_000)
    ctx.set_scene(sc)
    par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=2_000, radius_scale=1 / 32)
    with pytest.raises(P.PppmError) as e:
        ctx.render_tune(refill=4)  # no render yet
    assert e.value.code in (P.E_STATE,)
    ctx.render_begin(sc.camera, par)
    for bad in (dict(refill=33), dict(exact_batch=0), dict(gather_stage=48), dict(gather_stage=288),
                dict(query_sub_bits=4), dict(cell_factor=0.5), dict(bounce_blocks_per_sm=65),
                dict(eye_blocks_per_sm=129)):
        with pytest.raises(P.PppmError) as e:
            ctx.render_tune(**bad)
        assert e.value.code == P.E_ARG, bad
    # a rejected call changes nothing
    assert ctx.get_tune() == pytest.approx(DEFAULTS)
