"""Checkpoint / resume of a renderer: a renderer restored from a checkpoint
continues the interrupted progressive sequence to the bit (every random
number follows from seed, request id, frame, pixel and sample), including a
checkpoint taken inside a light-pass group, whose light cache the restored
renderer makes again."""
import numpy as np
import pytest

from helpers import scene_arrays

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_resume_continues_bit_for_bit(gbdev, mode):
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    p = gbdev.default_params(eye_depth_max=6, light_depth_max=6, pt_depth_max=6, warmup_frames=2,
                             render_iterations=0)
    W, H, total, cut = 48, 40, 9, 5  # frames 0..4 before the checkpoint: frame 5 is inside a group of 3
    a = gbdev.RTRenderer(W, H, mode, p)
    want = [a.render(s, cam, stats=False).copy() for _ in range(total)]
    a.close()
    b = gbdev.RTRenderer(W, H, mode, p)
    for _ in range(cut):
        b.render(s, cam, stats=False)
    data = b.checkpoint()
    b.close()
    s2 = gbdev.RTScene(v, t, m).build_bvh()  # a new handle of the same scene, as in a new process
    c = gbdev.RTRenderer(W, H, 0, gbdev.default_params())
    c.restore(data)
    assert c.mode == mode
    for f in range(cut, total):
        got = c.render(s2, cam, stats=False)
        assert np.array_equal(got.view(np.uint32), want[f].view(np.uint32)), (mode, f)
    assert np.array_equal(c.read_buffer(6), c.read_buffer(6))
    c.close()


def test_restore_rejects_other_scene_and_bad_data(gbdev):
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(32, 32, 0, gbdev.default_params())
    r.render(s, cam)
    data = r.checkpoint()
    r.close()
    with pytest.raises(gbdev.GbptError):
        gbdev.RTRenderer(16, 16, 0, gbdev.default_params()).restore(data)  # other size
    with pytest.raises(gbdev.GbptError):
        gbdev.RTRenderer(32, 32, 0, gbdev.default_params()).restore(b"not a checkpoint" * 8)
    (v2, t2, m2), cam2 = scene_arrays("interior")
    other = gbdev.RTScene(v2, t2, m2).build_bvh()
    q = gbdev.RTRenderer(32, 32, 0, gbdev.default_params()).restore(data)
    with pytest.raises(gbdev.GbptError) as e:
        q.render(other, cam)
    assert "another scene" in str(e.value)
