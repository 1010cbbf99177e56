"""The image order of the flat kernels (cbq_query.image_width): work item g goes
to the pixel at place g % 32 of tile g / 32, tiles of 4 x 8 pixels running left
to right along 8-row bands (csrc/cbq_flat.cuh, FlatCtxT::ray_slot).  launch_flat
applies it when the width is a multiple of 4 and the launch's rays fill whole
8-row bands; these tests check, with the same integer arithmetic in numpy, that
it is then a bijection of [0, n), and that a warp's 32 items are one tile."""
import numpy as np
import pytest


def ray_slot(g, w):
    g = np.asarray(g, dtype=np.uint64)
    t = (g >> np.uint64(5)).astype(np.uint32)
    k = (g & np.uint64(31)).astype(np.uint32)
    per_band = np.uint32(w >> 2)
    band = t // per_band
    col = t - band * per_band
    row = (band * np.uint32(8) + (k >> np.uint32(2))).astype(np.uint64)
    return row * np.uint64(w) + (col * np.uint32(4) + (k & np.uint32(3))).astype(np.uint64)


def applies(w, n):
    return w > 0 and w % 4 == 0 and n < (1 << 32) and n % (8 * w) == 0


@pytest.mark.parametrize("w,rows", [(2048, 2048), (1024, 1024), (1920, 1080 * 8), (384, 256), (4, 8), (12, 16),
                                    (12288, 8)])
def test_tile_order_is_a_bijection(w, rows):
    n = w * rows
    assert applies(w, n)
    s = ray_slot(np.arange(n, dtype=np.uint64), w)
    assert s.min() == 0 and s.max() == n - 1
    assert np.unique(s).size == n


def test_a_warp_takes_one_tile():
    w = 1920
    s = ray_slot(np.arange(32 * 1000, dtype=np.uint64), w).reshape(-1, 32)
    x, y = s % w, s // w
    assert np.all(x.max(axis=1) - x.min(axis=1) == 3)
    assert np.all(y.max(axis=1) - y.min(axis=1) == 7)


@pytest.mark.parametrize("w,n", [(383, 383 * 8), (392, 98304), (2048, 2048 * 1000 + 4), (0, 1024)])
def test_other_launches_keep_their_order(w, n):
    assert not applies(w, n)
