"""Row-band sharding of one image over several renderers (ranks or GPUs).

Pixels are independent and every path's random numbers follow from its
full-image pixel id (``RTRenderer.set_window``), so rank r of n renders the
rows ``shard_rows(H, n, r)`` of the image and ``assemble`` stacks the bands
into the image a single renderer makes, to the bit.  The light-vertex cache
needs no exchange: every rank makes the same one (same key and frame).  The
reference renders one image per process (src/cudaRTBDPTStream.cu:134-169);
this is the host side of splitting it.
"""
import numpy as np


def shard_rows(height, world, rank):
    """(first row, rows) of rank `rank` of `world`: contiguous bands whose
    sizes differ by at most one row, the larger ones first."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in 0..world-1")
    base, extra = divmod(height, world)
    rows = base + (1 if rank < extra else 0)
    y0 = rank * base + min(rank, extra)
    return y0, rows


def assemble(bands, width, channels=3):
    """The whole image from the bands of ranks 0..n-1 (row 0 first, as the
    renderer lays out its image), each a flat array of rows * width * channels."""
    parts = [np.asarray(b).reshape(-1, width * channels) for b in bands]
    return np.concatenate(parts).reshape(-1)


def render_band(gb, scene, cam, width, height, world, rank, frames, mode=0, params=None):
    """Rank `rank`'s band of a width x height image after `frames` progressive
    frames on this process's GPU: (y0, rows, running means, sample counts)."""
    y0, rows = shard_rows(height, world, rank)
    r = gb.RTRenderer(width, rows, mode, params)
    r.set_window(0, y0, width, height)
    for _ in range(frames):
        r.render_frames(scene, cam, 1, stats=False)
    out = (y0, rows, r.read_buffer(0).copy(), r.read_buffer(6).copy())
    r.close()
    return out
