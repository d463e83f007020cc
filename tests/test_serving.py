"""Batched render serving (gbpt_server_*): concurrent requests of uneven
size give the same images as the same requests rendered alone, the
scheduling knobs the autotuner picks change no pixel, admission refuses
what cannot fit, and the serving configuration's workload is drawn as
specified."""
import numpy as np
import pytest

from helpers import scene_arrays


def test_poisson_workload_draws():
    from cudapt_gb300 import serving
    a = serving.poisson_workload(64, 200.0, seed=3)
    b = serving.poisson_workload(64, 200.0, seed=3)
    assert a == b and len(a) == 64
    t = np.array([r[0] for r in a])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    assert 0.1 < t[-1] < 1.0  # 63 gaps of mean 5 ms
    for _, name, w, h, spp, depth in a:
        assert name in ("cornell", "interior", "hall")
        assert (w, h) in serving.RESOLUTIONS and spp in serving.SPP and depth in serving.DEPTHS


def test_server_structs_match_header(gb):
    import ctypes
    from cudapt_gb300._native import Request, RequestStatus
    assert ctypes.sizeof(Request) == 80 and ctypes.sizeof(RequestStatus) == 56
    assert Request.params.offset == 64 and RequestStatus.paths.offset == 40


def _alone(gb, scene, cam, w, h, frames, mode, params):
    r = gb.RTRenderer(w, h, mode, params)
    r.render_frames(scene, cam, frames - 1, stats=False)
    img = r.render(scene, cam, stats=False).copy()
    r.close()
    return img


@pytest.mark.gpu
@pytest.mark.parametrize("policy,graphs", [(1, False), (0, True)])
def test_server_images_equal_single_renders(gbdev, policy, graphs):
    from cudapt_gb300 import serving
    (v, t, m), cam = scene_arrays("cornell")
    cornell = gbdev.RTScene(v, t, m).build_bvh()
    (v2, t2, m2), cam2 = scene_arrays("interior")
    interior = gbdev.RTScene(v2, t2, m2).build_bvh()
    jobs = [(cornell, cam, 64, 48, 3, 0, 8), (interior, cam2, 96, 64, 4, 0, 10), (cornell, cam, 32, 32, 7, 1, 6),
            (interior, cam2, 80, 60, 2, 4, 8), (cornell, cam, 64, 48, 3, 0, 8), (interior, cam2, 96, 64, 5, 3, 6)]
    outs = [np.zeros(w * h * 3, np.float32) for (_, _, w, h, _, _, _) in jobs]
    with serving.Server(workers=3, policy=policy, graphs=graphs) as srv:
        ids = []
        for (s, c, w, h, f, mode, d), o in zip(jobs, outs):
            p = gbdev.default_params(eye_depth_max=d, light_depth_max=d, pt_depth_max=d, warmup_frames=2)
            ids.append(srv.submit(s, c, w, h, f, mode=mode, params=p, out=o))
        st = [srv.wait(i) for i in ids]
    for (s, c, w, h, f, mode, d), o, r in zip(jobs, outs, st):
        assert r["done"] == 1 and r["status"] == 0, r
        assert r["paths"] == w * h * f and r["latency_ms"] >= r["run_ms"] > 0
        p = gbdev.default_params(eye_depth_max=d, light_depth_max=d, pt_depth_max=d, warmup_frames=2)
        want = _alone(gbdev, s, c, w, h, f, mode, p)
        assert np.array_equal(o.view(np.uint32), want.view(np.uint32)), (w, h, mode, r)


@pytest.mark.gpu
def test_scheduling_knobs_change_no_pixel(gbdev):
    """Refill threshold, the tail kernel's first bounce and the persistent
    grids' CTAs per SM reorder work between lanes only: every setting gives
    the same image."""
    (v, t, m), cam = scene_arrays("interior")
    s = gbdev.RTScene(v, t, m).build_bvh()
    imgs = []
    for refill, tail, ctas in ((0, -1, 0), (12, -1, 1), (28, 7, 2), (20, 10, 3), (5, 2, 0), (8, -1, 32)):
        p = gbdev.default_params(eye_depth_max=10, light_depth_max=10, walk_refill=refill, tail_from=tail,
                                 walk_ctas=ctas)
        imgs.append(_alone(gbdev, s, cam, 96, 72, 2, 0, p))
    for im in imgs[1:]:
        assert np.array_equal(im.view(np.uint32), imgs[0].view(np.uint32))


@pytest.mark.gpu
def test_server_autotuner_and_admission(gbdev):
    from cudapt_gb300 import serving
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    with serving.Server(workers=2) as srv:
        ids = [srv.submit(s, cam, 64, 64, 2) for _ in range(16)]
        st = [srv.wait(i) for i in ids]
        assert all(r["status"] == 0 for r in st)
        refill, tail, n = srv.tuned(0, 5, 64, 64)
        assert n == 16 and refill in (2, 4, 8) and tail in (-1, 2, 5)
        assert len({(r["walk_refill"], r["tail_from"]) for r in st}) >= 3  # candidates were explored
        k = srv.tuned_knobs(0, 5, 64, 64)
        assert k["samples"] == 16 and k["bands"] == 1 and k["walk_ctas"] in (0, 2, 3)
        assert (k["walk_refill"], k["tail_from"]) == (refill, tail)
    # a released status is gone
    with serving.Server(workers=1) as srv:
        rid = srv.submit(s, cam, 32, 32, 1)
        assert srv.wait(rid)["status"] == 0
        with pytest.raises(gbdev.GbptError):
            srv.wait(rid, timeout_ms=0)
    # a reserve larger than the device: nothing can be admitted, and nothing else runs
    with serving.Server(workers=1, hbm_reserve=1 << 50) as srv:
        r = srv.wait(srv.submit(s, cam, 64, 64, 1))
        assert r["done"] == 1 and r["status"] == 2  # GBPT_ERR_OOM
