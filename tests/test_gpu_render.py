"""GPU parity of whole frames: plain streaming BDPT and the adaptive +
bilateral variant against the oracle's per-path restatement."""
import numpy as np
import pytest

from helpers import assert_bits_equal, block_means, scene_arrays

pytestmark = pytest.mark.gpu


def _render_both(gb, orc, name, W, H, frames, mode=0, **pk):
    (v, t, m), cam = scene_arrays(name)
    params = gb.default_params(**pk)
    s = gb.RTScene(v, t, m).build_bvh()
    r = gb.RTRenderer(W, H, mode, params)
    stats = []
    for _ in range(frames):
        img = r.render(s, cam).copy()
        stats.append(r.last_stats)
    osc = orc.Scene(v, t, m)
    ref = orc.Renderer(W, H, mode, params)
    ref.render(osc, cam, frames)
    return r, ref, img, ref.get(0), stats


def test_cornell_light_cache_bitexact(gbdev, orc):
    (v, t, m), cam = scene_arrays("cornell")
    params = gbdev.default_params(eye_depth_max=8, light_depth_max=8)
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(32, 32, 0, params)
    r.render(s, cam)
    n = r.last_stats["light_vertices"]
    ref = orc.Renderer(32, 32, 0, params)
    ref.render(orc.Scene(v, t, m), cam, 1)
    want = ref.light_cache()
    assert n == len(want) and n > 128
    got = r.light_cache(n)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_cornell_plain_bitexact(gbdev, orc):
    r, ref, img, want, stats = _render_both(gbdev, orc, "cornell", 64, 64, 7, eye_depth_max=8, light_depth_max=8)
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")
    assert stats[-1]["frame"] == 6 and stats[-1]["paths"] == 64 * 64


def test_cornell_statistics_independent_seeds(gbdev, orc):
    """Different Philox keys: 8x8-block means agree within 3 sigma."""
    (v, t, m), cam = scene_arrays("cornell")
    W = H = 64
    frames = 24
    pa = gbdev.default_params(eye_depth_max=8, light_depth_max=8, seed=1234)
    pb = gbdev.default_params(eye_depth_max=8, light_depth_max=8, seed=98765)
    s = gbdev.RTScene(v, t, m).build_bvh()
    runs = []
    for p, dev in ((pa, True), (pb, False), (gbdev.default_params(eye_depth_max=8, light_depth_max=8, seed=555), True)):
        per = []
        if dev:
            r = gbdev.RTRenderer(W, H, 0, p)
            prevS, prevN = np.zeros(W * H * 3), np.zeros(W * H)
            for f in range(frames):
                img = r.render(s, cam).astype(np.float64)
                N = r.read_buffer(6).astype(np.float64)
                S = img * np.repeat(N, 3)
                per.append(block_means(S - prevS, W, H) / np.maximum(
                    block_means(np.repeat(N - prevN, 3), W, H), 1e-9))
                prevS, prevN = S, N
        else:
            ref = orc.Renderer(W, H, 0, p)
            osc = orc.Scene(v, t, m)
            prevS, prevN = np.zeros(W * H * 3), np.zeros(W * H)
            for f in range(frames):
                ref.render(osc, cam, 1)
                img = ref.get(0).astype(np.float64)
                N = ref.sample_counts()[0].astype(np.float64)
                S = img * np.repeat(N, 3)
                per.append(block_means(S - prevS, W, H) / np.maximum(
                    block_means(np.repeat(N - prevN, 3), W, H), 1e-9))
                prevS, prevN = S, N
        per = np.array(per)
        runs.append((per.mean(0), per.std(0, ddof=1) / np.sqrt(frames)))
    (m1, s1), (m2, s2), (m3, s3) = runs
    z12 = np.abs(m1 - m2) / np.sqrt(s1 ** 2 + s2 ** 2 + 1e-12)
    z13 = np.abs(m1 - m3) / np.sqrt(s1 ** 2 + s3 ** 2 + 1e-12)
    assert np.mean(z12 < 3) >= 0.97, np.mean(z12 < 3)
    assert np.mean(z13 < 3) >= 0.97, np.mean(z13 < 3)


def test_interior_plain_matches(gbdev, orc):
    r, ref, img, want, stats = _render_both(gbdev, orc, "interior", 96, 72, 4, eye_depth_max=10, light_depth_max=10)
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")


def test_walk_counters_match_oracle(gbdev, orc):
    """Closest-hit rays, node visits and triangle tests of a whole frame
    (wavefront and tail kernels) equal the oracle's counts for the same
    paths exactly: the persistent walks visit nodes in TracePrimitive's
    order.  The kernels skip connection rays whose contribution is zero
    whatever their visibility, so their any-hit work is at most the
    oracle's."""
    (v, t, m), cam = scene_arrays("interior")
    W, H = 80, 60
    params = gbdev.default_params(eye_depth_max=10, light_depth_max=10)
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(W, H, 0, params)
    r.set_counting(True)
    r.render(s, cam)
    st = r.render_frames(s, cam, 1)
    ref = orc.Renderer(W, H, 0, params)
    ref.render(orc.Scene(v, t, m), cam, 2)
    rs = ref.stats()
    assert st["paths"] == rs["paths"] == W * H
    for got, want in ((st["rays"] - st["shadow_rays"], rs["ext_rays"]), (st["nodes"], rs["ext_nodes"]),
                      (st["tris"], rs["ext_tris"])):
        assert int(got) == int(want), (got, want)
    assert st["shadow_rays"] <= rs["rays"] - rs["ext_rays"]
    assert st["shadow_nodes"] <= rs["nodes"] - rs["ext_nodes"]


def test_env_term(gbdev, orc):
    """Constant environment on a miss (scene open at z=1: Cornell)."""
    r, ref, img, want, _ = _render_both(gbdev, orc, "cornell", 48, 48, 3, eye_depth_max=8, light_depth_max=8,
                                        env=(0.1, 0.1, 0.1))
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")


def test_adaptive_matches(gbdev, orc):
    r, ref, img, want, stats = _render_both(gbdev, orc, "cornell", 64, 48, 5, mode=1, eye_depth_max=8,
                                            light_depth_max=8, warmup_frames=2, filter_radius=4)
    cnt_ref = ref.sample_counts()[1]
    assert cnt_ref.sum() > 0
    for b in (1, 2, 3, 4, 5):  # G-buffer position, normal, diffuse; filtered image; error
        assert_bits_equal(r.read_buffer(b), ref.get(b), f"buffer {b}")
    assert_bits_equal(img, want, "image")
    sn_ref, cnt_ref = ref.sample_counts()
    assert_bits_equal(r.read_buffer(6), sn_ref, "sampleN")


def test_adaptive_accumulation_tiers(gbdev, orc):
    """The per-pixel sums of budgeted frames use 8, 32 or 1024 partials by
    sample count (kernels k_accum / k_accum_mid / k_accum_huge); the oracle
    sums in the same order, so frames stay bit-identical across the tiers."""
    r, ref, img, want, stats = _render_both(gbdev, orc, "cornell", 192, 160, 4, mode=1, eye_depth_max=8,
                                            light_depth_max=8, warmup_frames=2, filter_radius=4)
    cnt = ref.sample_counts()[1]
    assert cnt.max() > 64  # the warp-per-pixel tier ran
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")
    # the hall's fireflies draw most of a frame's budget onto single pixels: the CTA-per-pixel tier
    # (512x288: the first budgeted frame gives one pixel about 5000 samples)
    r, ref, img, want, stats = _render_both(gbdev, orc, "hall_small", 512, 288, 6, mode=1, eye_depth_max=5,
                                            light_depth_max=5, warmup_frames=5, filter_radius=4)
    assert ref.sample_counts()[1].max() > 4096, ref.sample_counts()[1].max()
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")


def test_adaptive_binary_matches(gbdev, orc):
    """'BDPTSC Adap Bilat Binary': window search passes, leftover fill, per-pass apply."""
    r, ref, img, want, stats = _render_both(gbdev, orc, "cornell", 64, 48, 5, mode=2, eye_depth_max=8,
                                            light_depth_max=8, warmup_frames=2, filter_radius=4)
    assert_bits_equal(img, want, "image")
    sn_gpu = r.read_buffer(6)
    assert_bits_equal(sn_gpu, ref.sample_counts()[0], "sampleN")
    assert sn_gpu.sum() > 64 * 48 * 4  # the budgeted frames added W*H paths each
    for b in (1, 2, 3, 4):
        assert_bits_equal(r.read_buffer(b), ref.get(b), f"buffer {b}")


def test_bilateral_kernel_bitexact(gbdev, orc):
    rng = np.random.Generator(np.random.PCG64(21))
    W, H = 77, 45
    planes = [rng.random(W * H * 3).astype(np.float32) for _ in range(4)]
    # many equal neighbours (zero distances) and a few far outliers in the normal plane
    planes[2] = np.round(planes[2] * 2.0).astype(np.float32) / np.float32(2.0)
    planes[2][rng.integers(0, W * H * 3, 64)] = np.float32(1e6)
    L = gbdev._native.load()
    # radii 4 and 5 run the compile-time-radius tile kernels, 2/3/24 the run-time-radius one,
    # 25 (window above the shared-memory limit) the direct kernel
    for radius, emit, delta in ((4, False, 3.0), (5, True, 50.0), (2, False, 1.0), (4, True, 2.0), (5, False, 4.0),
                                (3, True, 1.5), (24, False, 9.0), (25, True, 9.0)):
        g = np.zeros(64, np.float32)
        gbdev._native.check(L.gbpt_gaussian_table(delta, radius, g.ctypes.data))
        gref = orc.gaussian(delta, radius)
        assert np.array_equal(g[: 2 * radius + 1], gref[: 2 * radius + 1])
        out = np.zeros(W * H * 3, np.float32)
        e = planes[3] if emit else None
        gbdev._native.check(L.gbpt_bilateral(planes[0].ctypes.data, planes[1].ctypes.data, planes[2].ctypes.data,
                                             e.ctypes.data if emit else None, W, H, 0.5, 1.0, 0.25, 0.1, radius,
                                             g.ctypes.data, out.ctypes.data, 0))
        want = orc.bilateral(planes[0], planes[1], planes[2], e, W, H, 0.5, 1.0, 0.25, 0.1, radius, gref)
        assert np.array_equal(out.view(np.uint32), want.view(np.uint32)), (radius, emit)


def test_errors_are_reported(gbdev):
    import cudapt_gb300 as gb
    (v, t, m), cam = scene_arrays("cornell")
    bad = t.copy()
    bad["v0"][0] = 10 ** 6
    with pytest.raises(gb.GbptError):
        gb.RTScene(v, bad, m)
    s = gb.RTScene(v, t, m)
    r = gb.RTRenderer(16, 16)
    with pytest.raises(gb.GbptError, match="BVH"):
        r.render(s, cam)
    with pytest.raises(gb.GbptError):
        gb.RTRenderer(16, 16, params=gb.default_params(light_paths=5000))
    for below in (-0.5, 1.5, float("nan")):
        with pytest.raises(gb.GbptError, match="tail_below"):
            gb.RTRenderer(16, 16, params=gb.default_params(tail_below=below))
    with pytest.raises(gb.GbptError, match="carry_steps"):
        gb.RTRenderer(16, 16, params=gb.default_params(carry_steps=(1 << 20) + 1))
    with pytest.raises(gb.GbptError):
        r.attr_set("No Such Attribute", 1.0)


def test_fp32_converges_to_fp64_reference(gbdev, orc):
    """RMSE against the FP64 host render of the same estimator: the GPU's FP32
    image after F frames is far closer to the FP64 image of the same F frames
    (same random numbers) than two independent F-frame images are to each
    other, and the error of independent runs shrinks as frames grow."""
    (v, t, m), cam = scene_arrays("cornell")
    W = H = 32
    params = gbdev.default_params(eye_depth_max=8, light_depth_max=8)
    s = gbdev.RTScene(v, t, m).build_bvh()
    osc = orc.Scene(v, t, m)
    ref64 = {}
    for F in (8, 32):
        r = gbdev.RTRenderer(W, H, 0, params)
        for _ in range(F):
            img = r.render(s, cam).astype(np.float64)
        ref64[F] = orc.render_fp64(osc, params, W, H, cam, F)
        rmse_same = np.sqrt(np.mean((img - ref64[F]) ** 2))
        other = gbdev.RTRenderer(W, H, 0, gbdev.default_params(eye_depth_max=8, light_depth_max=8, seed=4321))
        for _ in range(F):
            img2 = other.render(s, cam).astype(np.float64)
        rmse_indep = np.sqrt(np.mean((img2 - ref64[F]) ** 2))
        assert rmse_same < 0.15 * rmse_indep, (F, rmse_same, rmse_indep)
        ref64[F, "indep"] = rmse_indep
    assert ref64[32, "indep"] < ref64[8, "indep"]


def test_mode_switch_and_result_buffers(gbdev):
    """SetRendererMode reaches every registered renderer; the image gbpt_render
    copies into the caller's page-locked buffer equals GetResult's copy."""
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(32, 32, 0, gbdev.default_params(eye_depth_max=4, light_depth_max=4))
    assert r._pinned is not None
    L = gbdev._native.load()
    for mode in (0, 3, 4, 1, 2):
        r.SetRendererMode(mode)
        img = r.render(s, cam)
        got = np.ctypeslib.as_array(L.gbpt_result(r.handle), shape=(32 * 32 * 3,))
        assert np.array_equal(img.view(np.uint32), got.view(np.uint32)), mode
        assert np.isfinite(img).all() and img.max() > 0
    with pytest.raises(gbdev.GbptError) as e:
        r.SetRendererMode(5)
    assert e.value.status == 1
    r.close()
    assert r._pinned is None
    img[:] = 0  # still valid memory after the release


@pytest.mark.parametrize("name,W,H,depth,mode,extra", [
    ("interior", 1024, 768, 10, 0, {}),
    ("interior", 1024, 768, 10, 0, dict(level=3, env=(0.1, 0.1, 0.1))),  # the benchmark interior as stated
    ("hall", 1280, 720, 5, 0, {}),
    ("hall", 1280, 720, 8, 4, {}),  # unidirectional PTSC on the hall
])
def test_full_size_frame_bands_match_oracle(gbdev, orc, name, W, H, depth, mode, extra):
    """The benchmark workloads at full size: one GPU frame against the
    oracle's rendering of three 4-row bands of the same frame (every path's
    random numbers follow from its global pixel id and the frame's light
    cache, so a window of the image renders alone)."""
    from cudapt_gb300 import scenes
    extra = dict(extra)
    env = extra.pop("env", None)
    (v, t, m), cam = getattr(scenes, name)(**extra)
    pk = dict(eye_depth_max=depth, light_depth_max=depth, pt_depth_max=depth)
    if env is not None:
        pk["env"] = env
    params = gbdev.default_params(**pk)
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(W, H, mode, params)
    img = r.render(s, cam).reshape(H, W, 3).copy()
    assert r.last_stats["paths"] == W * H
    osc = orc.Scene(v, t, m)
    for y0 in (0, H // 2, H - 4):
        ref = orc.Renderer(W, 4, mode, params)
        ref.set_window(0, y0, W, H)
        ref.render(osc, cam, 1)
        want = ref.get(0).reshape(4, W, 3)
        got = img[y0:y0 + 4]
        assert_bits_equal(got, want, f"rows {y0}..{y0 + 3}")
        assert_bits_equal(r.read_buffer(6).reshape(H, W)[y0:y0 + 4], ref.sample_counts()[0].reshape(4, W),
                          f"sampleN rows {y0}..{y0 + 3}")


def test_cornell_box_config_full_size(gbdev, orc):
    """The Cornell box benchmark configuration as stated: 256x256, depth 8,
    16 progressive frames (16 camera samples per pixel), Philox seed 1234;
    the whole image and every sample count equal the oracle's."""
    r, ref, img, want, stats = _render_both(gbdev, orc, "cornell", 256, 256, 16, eye_depth_max=8,
                                            light_depth_max=8, seed=1234)
    assert stats[-1]["frame"] == 15 and stats[-1]["paths"] == 256 * 256
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")


def test_full_size_hall_adaptive_bilateral(gbdev, orc):
    """The adaptive + bilateral benchmark configuration at full size: the
    332K-triangle hall at 1280x720, 8 uniform frames then budgeted frames
    (the PLL allocator spends W*H paths per frame by the filtered-minus-raw
    error), bilateral radius 4.  The budget couples every pixel through the
    frame's error sum, so the oracle renders the whole frame; image, sample
    counts, G-buffer, filtered image and error plane equal the oracle's."""
    from cudapt_gb300 import scenes
    (v, t, m), cam = scenes.hall()
    W, H = 1280, 720
    params = gbdev.default_params(eye_depth_max=5, light_depth_max=5, warmup_frames=8, filter_radius=4)
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(W, H, 1, params)
    frames = 10
    for _ in range(frames):
        img = r.render(s, cam).copy()
    ref = orc.Renderer(W, H, 1, params)
    ref.render(orc.Scene(v, t, m), cam, frames)
    sn_ref, cnt_ref = ref.sample_counts()
    assert cnt_ref.sum() > 0 and cnt_ref.max() > 8  # the budgeted frames ran
    assert_bits_equal(img, ref.get(0), "image")
    assert_bits_equal(r.read_buffer(6), sn_ref, "sampleN")
    for b in (1, 2, 3, 4, 5):
        assert_bits_equal(r.read_buffer(b), ref.get(b), f"buffer {b}")


@pytest.mark.parametrize("mode,depth", [(0, 10), (4, 8)])
def test_graph_frames_equal_direct_launches(gbdev, mode, depth):
    """Frames issued as CUDA graphs (plain and PTSC) give the images of direct
    launches: across light-pass frames, a camera change and knob changes that
    alter the graph's shape (tail kernel or not)."""
    (v, t, m), cam = scene_arrays("interior")
    s = gbdev.RTScene(v, t, m).build_bvh()
    cam2 = dict(cam)
    cam2["pos"] = [float(x) + 0.25 for x in cam["pos"]]
    p = gbdev.default_params(eye_depth_max=depth, light_depth_max=depth, pt_depth_max=depth)
    runs = []
    for graphs in (False, True):
        r = gbdev.RTRenderer(80, 60, mode, p)
        r.set_graphs(graphs)
        imgs = []
        for f in range(9):
            c = cam if f < 5 else cam2
            if f == 6:  # restarts accumulation with knobs that change the graph's shape
                r.params = gbdev.default_params(eye_depth_max=depth, light_depth_max=depth, pt_depth_max=depth,
                                                tail_from=depth, walk_refill=12)
            imgs.append(r.render(s, c, stats=(f == 8)).copy())
        runs.append(imgs)
        if graphs:
            assert r.last_stats["ms_total"] > 0
        r.close()
    for f, (a, b) in enumerate(zip(*runs)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f


@pytest.mark.parametrize("mode", [0, 3, 4])
def test_bands_change_no_pixel(gbdev, orc, mode):
    """A frame split into bands (one wavefront per band, each on its own
    stream) gives the image of a single wavefront, with and without CUDA
    graphs; the stats count every band's paths and rays."""
    (v, t, m), cam = scene_arrays("interior")
    s = gbdev.RTScene(v, t, m).build_bvh()
    W, H = 97, 61  # bands of unequal size
    imgs, stats = {}, {}
    for bands in (1, 2, 3, 8):
        for graphs in (False, True):
            p = gbdev.default_params(eye_depth_max=10, light_depth_max=10, pt_depth_max=8, bands=bands,
                                     render_iterations=3)
            r = gbdev.RTRenderer(W, H, mode, p)
            r.set_graphs(graphs)
            for _ in range(4):
                img = r.render(s, cam).copy()
            imgs[bands, graphs] = (r.read_buffer(0), r.read_buffer(6))
            stats[bands, graphs] = r.last_stats
            r.close()
    base = imgs[1, False]
    for key, (res, sn) in imgs.items():
        assert_bits_equal(res, base[0], f"image, bands/graphs {key}")
        assert_bits_equal(sn, base[1], f"sampleN, bands/graphs {key}")
    for key, st in stats.items():
        if mode != 3:  # the filter-only mode's fourth frame only filters
            assert st["paths"] == W * H, (key, st["paths"])
            assert st["rays"] == stats[1, False]["rays"], key
    ref = orc.Renderer(W, H, mode, gbdev.default_params(eye_depth_max=10, light_depth_max=10, pt_depth_max=8,
                                                         render_iterations=3))
    ref.render(orc.Scene(v, t, m), cam, 4)
    assert_bits_equal(base[0], ref.get(0), "image against the oracle")


@pytest.mark.parametrize("mode,depth", [(0, 10), (1, 6), (4, 8)])
def test_carry_and_tail_switch_change_no_pixel(gbdev, mode, depth):
    """Walks carried mid-walk from the bounce launches to the tail kernel
    (carry_steps; at 1 step the carry buffer fills and the other walks finish
    in their launch) and the switch to the tail kernel decided on the device
    (tail_below) move work between kernels only: image, sample counts and ray
    counts equal those of per-bounce launches throughout, in both traversal
    orders (the wide walk carries nothing)."""
    (v, t, m), cam = scene_arrays("interior")
    W, H = 96, 72
    runs = {}
    for order in ("reference", "wide"):
        s = gbdev.RTScene(v, t, m).build_bvh()
        s.set_traversal(order)
        for cs, below, tail in ((0, 0.0, depth), (96, 0.0, depth), (1, 0.0, depth), (0, 0.5, depth),
                                (96, 0.3, -1), (1, 0.95, -1), (4, 1.0, 2)):
            p = gbdev.default_params(eye_depth_max=depth, light_depth_max=depth, pt_depth_max=depth, carry_steps=cs,
                                     tail_below=below, tail_from=tail, warmup_frames=2)
            r = gbdev.RTRenderer(W, H, mode, p)
            rays = 0
            for _ in range(4):
                r.render(s, cam, stats=True)
                rays += r.last_stats["rays"]
            runs[order, cs, below, tail] = (r.read_buffer(0), r.read_buffer(6), rays)
            r.close()
    base = runs["reference", 0, 0.0, depth]
    for key, (img, sn, rays) in runs.items():
        assert_bits_equal(img, base[0], f"image {key}")
        assert_bits_equal(sn, base[1], f"sampleN {key}")
        assert rays == base[2], (key, rays, base[2])


@pytest.mark.parametrize("mode", [0, 3, 4])
def test_windows_assemble_the_image(gbdev, mode):
    """Windows of one image rendered by separate renderers (ragged row bands,
    as cudapt_gb300.sharding assigns them, and 2x2 tiles) give the whole
    image's running means and sample counts to the bit (the filter-only
    mode's unfiltered planes)."""
    from cudapt_gb300 import sharding
    (v, t, m), cam = scene_arrays("interior")
    s = gbdev.RTScene(v, t, m).build_bvh()
    W, H, frames = 90, 71, 3
    p = gbdev.default_params(eye_depth_max=10, light_depth_max=10, pt_depth_max=8, render_iterations=5)
    full = gbdev.RTRenderer(W, H, mode, p)
    for _ in range(frames):
        full.render_frames(s, cam, 1, stats=False)
    want_img, want_n = full.read_buffer(0), full.read_buffer(6)
    full.close()
    bands = [sharding.render_band(gbdev, s, cam, W, H, 3, k, frames, mode, p) for k in range(3)]
    assert [b[1] for b in bands] == [24, 24, 23]
    assert_bits_equal(sharding.assemble([b[2] for b in bands], W), want_img, "row bands")
    assert_bits_equal(sharding.assemble([b[3] for b in bands], W, 1), want_n, "row-band sample counts")
    img = np.zeros((H, W, 3), np.float32)
    for x0, y0, w, h in ((0, 0, 45, 35), (45, 0, 45, 35), (0, 35, 45, 36), (45, 35, 45, 36)):
        r = gbdev.RTRenderer(w, h, mode, p).set_window(x0, y0, W, H)
        for _ in range(frames):
            r.render_frames(s, cam, 1, stats=False)
        img[y0:y0 + h, x0:x0 + w] = r.read_buffer(0).reshape(h, w, 3)
        r.close()
    assert_bits_equal(img.reshape(-1), want_img, "2x2 tiles")


def test_window_refused_in_adaptive_mode(gbdev):
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(16, 8, 1, gbdev.default_params()).set_window(0, 8, 16, 16)
    with pytest.raises(gbdev.GbptError) as e:
        r.render(s, cam)
    assert e.value.status == 6
    with pytest.raises(gbdev.GbptError):
        r.set_window(4, 0, 16, 16)  # 16 columns do not fit from x = 4
    r.set_window(0, 0, 16, 8)  # the whole image again
    assert np.isfinite(r.render(s, cam)).all()
