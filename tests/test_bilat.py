"""Filter-only mode "BDPTSC Bilaterial" (src/cudaRTBDPTStreamBilat.cu): the
oracle's frame-limit, filter-pass and debug-view semantics on the CPU, and
GPU parity of every plane the mode produces."""
import numpy as np
import pytest

from cudapt_gb300 import layouts
from helpers import assert_bits_equal, scene_arrays

W = H = 48
BILAT = layouts.MODE_BDPT_SC_BILAT


def _params(**kw):
    base = dict(eye_depth_max=6, light_depth_max=6, render_iterations=4, filter_iterations=2, bilat_radius=3)
    base.update(kw)
    return layouts.default_params(**base)


def _oracle(orc, frames, debug=0, **kw):
    (v, t, m), cam = scene_arrays("cornell")
    r = orc.Renderer(W, H, BILAT, _params(**kw), threads=4)
    r.set_debug(debug)
    sc = orc.Scene(v, t, m)
    r.render(sc, cam, frames)
    return r, sc, cam


def test_defaults_match_reference():
    p = layouts.default_params()
    assert (p["bilat_color_eud"], p["bilat_pos_eud"], p["bilat_norm_eud"]) == (1.0, 1.0, 1.0)
    assert (p["bilat_emit_eud"], p["bilat_diff_eud"]) == (0.5, 0.5)
    assert (p["bilat_radius"], p["filter_iterations"], p["render_iterations"]) == (5, 1, 5)


def test_oracle_frame_limit_and_filter_passes(orc):
    r, sc, cam = _oracle(orc, 4)
    res4, n4 = r.get(0).copy(), r.sample_counts()[0].copy()
    assert r.stats()["paths"] == W * H and n4.min() >= 4
    r.render(sc, cam, 2)  # frames 4 and 5: past "Render Iteration" -> filter only
    assert r.stats()["paths"] == 0 and r.frame == 5
    assert np.array_equal(r.get(0), res4) and np.array_equal(r.sample_counts()[0], n4)
    # two filter passes with the diffuse plane as the third feature (:1418-1432)
    p = r.params
    g = orc.gaussian(float(p["bilat_color_eud"]), int(p["bilat_radius"]))
    pos, norm, diff = r.get(1), r.get(2), r.get(3)
    f1 = orc.bilateral(res4, pos, norm, diff, W, H, 1.0, 1.0, 1.0, 0.5, 3, g)
    f2 = orc.bilateral(f1, pos, norm, diff, W, H, 1.0, 1.0, 1.0, 0.5, 3, g)
    assert np.array_equal(r.get(4), f2) and np.array_equal(r.get(11), f2)


def test_oracle_debug_views(orc):
    views = {}
    for dm in (4, 5, 6, 7, 2, 3):
        r, _, _ = _oracle(orc, 3, debug=dm, min_trace_prob=0.25)
        views[dm] = (r, r.get(11))
    r = views[4][0]
    assert np.array_equal(views[4][1], r.get(8))   # direct light
    assert np.array_equal(views[5][1], r.get(1))   # position
    assert np.array_equal(views[6][1], r.get(2))   # normal
    assert np.array_equal(views[7][1], r.get(0))   # unfiltered result
    # "Prob" (2) and "Prob With Limit" (3): filter of max(minProb, mean potential), result untouched
    pot = r.get(10)
    assert pot.min() >= 0.0 and np.all(np.isfinite(pot))
    g = orc.gaussian(1.0, 3)
    for dm, mp in ((2, 0.0), (3, 0.25)):
        rr = views[dm][0]
        view = np.repeat(np.maximum(mp, rr.get(10)), 3).astype(np.float32)
        f = orc.bilateral(view, rr.get(1), rr.get(2), rr.get(3), W, H, 1.0, 1.0, 1.0, 0.5, 3, g)
        f = orc.bilateral(f, rr.get(1), rr.get(2), rr.get(3), W, H, 1.0, 1.0, 1.0, 0.5, 3, g)
        assert np.array_equal(views[dm][1], f)
        assert np.array_equal(rr.get(0), r.get(0))


def test_oracle_direct_light_and_gbuffer(orc):
    """First-hit emissive is the material's; direct light is non-negative
    where the camera sees the lamp; the G-buffer planes are the last frame's."""
    r, _, _ = _oracle(orc, 2)
    emis, direct = r.get(9).reshape(-1, 3), r.get(8).reshape(-1, 3)
    lamp = emis.max(1) > 0
    assert lamp.any() and (~lamp).any()
    assert np.all(direct[lamp] > 0)
    nrm = r.get(2).reshape(-1, 3)
    hit = np.linalg.norm(nrm, axis=1) > 0
    np.testing.assert_allclose(np.linalg.norm(nrm[hit], axis=1), 1.0, atol=1e-3)


# ---------------------------------------------------------------------------
# GPU parity: every plane of the mode against the oracle, bit for bit on
# almost every pixel (the plain-mode bar), over frames that trace and frames
# that only filter, for every debug view.

def _gpu(gb, frames, debug=0, **kw):
    (v, t, m), cam = scene_arrays("cornell")
    s = gb.RTScene(v, t, m).build_bvh()
    r = gb.RTRenderer(W, H, BILAT, _params(**kw))
    if debug:
        r.attr_set("Debug Mode", debug)
    out = None
    for _ in range(frames):
        out = r.render(s, cam).copy()
    return r, out


@pytest.mark.gpu
def test_gpu_bilat_planes_bitexact(gbdev, orc):
    frames = 6  # 4 traced + 2 filter-only
    r, out = _gpu(gbdev, frames)
    ref, _, _ = _oracle(orc, frames)
    assert r.last_stats["paths"] == 0 and r.last_stats["frame"] == frames - 1
    for gid, oid in ((0, 0), (1, 1), (2, 2), (3, 3), (8, 8), (9, 9), (10, 10), (4, 4)):
        assert_bits_equal(r.read_buffer(gid), ref.get(oid), f"plane {gid}")
    assert np.array_equal(out, r.read_buffer(4))
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")


@pytest.mark.gpu
@pytest.mark.parametrize("debug", [2, 3, 4, 5, 6, 7])
def test_gpu_bilat_debug_views(gbdev, orc, debug):
    r, out = _gpu(gbdev, 3, debug=debug, min_trace_prob=0.25)
    ref, _, _ = _oracle(orc, 3, debug=debug, min_trace_prob=0.25)
    assert_bits_equal(out, ref.get(11), f"debug view {debug}")


@pytest.mark.gpu
def test_gpu_bilat_attributes(gbdev):
    (v, t, m), cam = scene_arrays("cornell")
    r = gbdev.RTRenderer(16, 16, BILAT, gbdev.default_params())
    names = r.attr_names()
    assert names[:9] == ["Filter Color E Delta", "Filter Pos E Delta", "Filter Norm E Delta", "Filter Emit E Delta",
                         "Filter Diff E Delta", "Filter Radius", "Filter Iteration", "Debug Mode", "Render Iteration"]
    assert r.attr_get("Filter Color E Delta") == 1.0 and r.attr_get("Render Iteration") == 5.0
    r.attr_set("Filter Iteration", 3)
    assert r.params["filter_iterations"] == 3
    with pytest.raises(gbdev.GbptError):
        r.attr_set("Debug Mode", 9)
    r.SetRendererMode(layouts.MODE_BDPT_SC_ADAP_BILAT)
    assert "Filter Color EuD" in r.attr_names()
