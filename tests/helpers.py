"""Shared helpers of the test suite (scene setup, ray generation, statistics)."""
import numpy as np

from cudapt_gb300 import layouts, scenes

SCENES = {"cornell": scenes.cornell, "interior": scenes.interior}


def scene_arrays(name, **kw):
    if name == "hall_small":
        return scenes.hall(boxes=200)
    return SCENES[name](**kw)


def random_rays(v, n, seed, pad=0.1):
    """Origins uniform in the scene box (slightly enlarged), directions uniform on the sphere."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = v["pos"]
    lo, hi = p.min(0) - pad, p.max(0) + pad
    o = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


def camera_rays(cam, w, h, seed):
    """Pinhole rays of a w x h grid with jitter (host numpy, any rounding)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos, d, up = (np.array(cam[k], np.float64) for k in ("pos", "dir", "up"))
    right = np.cross(d, up)
    right /= np.linalg.norm(right)
    up2 = np.cross(right, d)
    up2 /= np.linalg.norm(up2)
    th = np.tan(cam["fov"] / 2)
    ys, xs = np.mgrid[0:h, 0:w]
    u = (2 * (xs + rng.random(xs.shape)) / w - 1) * th * w / h
    vv = (2 * (ys + rng.random(ys.shape)) / h - 1) * th
    dirs = right * u[..., None] + up2 * vv[..., None] + d
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    o = np.broadcast_to(pos, dirs.shape)
    return np.concatenate([o.reshape(-1, 3), dirs.reshape(-1, 3)], 1).astype(np.float32)


def block_means(img, w, h, b=8):
    a = img.reshape(h, w, 3)[: h // b * b, : w // b * b]
    return a.reshape(h // b, b, w // b, b, 3).mean(axis=(1, 3))


def assert_bits_equal(got, want, what=""):
    """Exact equality of two float (or integer) arrays, word for word; the
    message names how many words differ and the first few indices."""
    g = np.ascontiguousarray(got)
    w = np.ascontiguousarray(want)
    assert g.shape == w.shape, (what, g.shape, w.shape)
    gv = g.view(np.uint32) if g.dtype == np.float32 else g
    wv = w.view(np.uint32) if w.dtype == np.float32 else w
    bad = np.nonzero(gv.ravel() != wv.ravel())[0]
    assert len(bad) == 0, (f"{what}: {len(bad)} of {gv.size} words differ; first at "
                           f"{bad[:5].tolist()}: got {g.ravel()[bad[:5]].tolist()} want {w.ravel()[bad[:5]].tolist()}")
