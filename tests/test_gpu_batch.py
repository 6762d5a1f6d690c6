"""Batched views: many independent views rendered in one pass, each into its
own tile of an atlas (ps3d_set_viewport_rect), give per tile exactly what the
view gives rendered alone in a pipeline of the view's size; the view alone
matches the oracle (depth bit-exact, colour within 1 LSB)."""
import numpy as np
import pytest

from common import colour_diff
from cpu_backends import OraclePipeline

VIEWS = 24
SIZE = 128


def _scenes():
    from puresoft3d_gb300 import scenes as S
    return S.scene_c4(views=VIEWS, size=SIZE)


def _tile_colour(atlas, ox, oy, size):
    h = atlas.shape[0]  # colour memory is top-down: pixel row y is memory row h-1-y
    return atlas[h - oy - size:h - oy, ox:ox + size]


def _tile_depth(depth, ox, oy, size):
    return depth[oy:oy + size, ox:ox + size]


@pytest.mark.gpu
def test_atlas_tiles_equal_views_alone(gpu_lib):
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    batched, plain = _scenes()
    atlas = PuresoftPipeline(batched.width, batched.height)
    S.replay_setup(batched, atlas)
    S.replay_frame(batched, atlas)
    colour = atlas.readColour().copy()
    depth = atlas.readDepth()[:, :batched.width].copy()
    alone = PuresoftPipeline(SIZE, SIZE)
    S.replay_setup(plain, alone)
    covered = 0
    for v, (ox, oy) in enumerate(batched.info["origins"]):
        S.replay_ops(plain.info["view_frames"][v], alone)
        c = alone.readColour()
        d = alone.readDepth()[:, :SIZE]
        assert np.array_equal(_tile_colour(colour, ox, oy, SIZE), c), "view %d colour" % v
        td = _tile_depth(depth, ox, oy, SIZE)
        assert np.array_equal(td.view(np.uint32), d.view(np.uint32)), "view %d depth" % v
        covered += int((d < 1.0).sum())
    assert covered > VIEWS * 200, "views cover too little to test anything"
    atlas.close()
    alone.close()


@pytest.mark.gpu
def test_atlas_of_many_draws(gpu_lib):
    """600 views of 32x32 in one pass: more draws than the set-up keeps in
    shared memory, so each warp finds its triangles' draws by its search of
    the draw table; every tile equals its view rendered alone."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    views, size = 600, 32
    batched, plain = S.scene_c4(views=views, size=size, tex_size=32, tri_min=20, tri_max=300)
    atlas = PuresoftPipeline(batched.width, batched.height)
    S.replay_setup(batched, atlas)
    S.replay_frame(batched, atlas)
    colour = atlas.readColour().copy()
    depth = atlas.readDepth()[:, :batched.width].copy()
    alone = PuresoftPipeline(size, size)
    S.replay_setup(plain, alone)
    covered = 0
    for v, (ox, oy) in enumerate(batched.info["origins"]):
        S.replay_ops(plain.info["view_frames"][v], alone)
        c = alone.readColour()
        d = alone.readDepth()[:, :size]
        assert np.array_equal(_tile_colour(colour, ox, oy, size), c), "view %d colour" % v
        assert np.array_equal(_tile_depth(depth, ox, oy, size).view(np.uint32), d.view(np.uint32)), "view %d" % v
        covered += int((d < 1.0).sum())
    assert covered > views * 50, "views cover too little to test anything"
    atlas.close()
    alone.close()


@pytest.mark.gpu
def test_views_alone_match_oracle(gpu_lib):
    """Every view alone against the oracle: depth bit-exact, colour within
    1 LSB."""
    from common import assert_depth_exact
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    _, plain = _scenes()
    g = PuresoftPipeline(SIZE, SIZE)
    o = OraclePipeline(SIZE, SIZE)
    S.replay_setup(plain, g)
    S.replay_setup(plain, o)
    for v in range(VIEWS):
        S.replay_ops(plain.info["view_frames"][v], g)
        S.replay_ops(plain.info["view_frames"][v], o)
        assert_depth_exact(g.readDepth()[:, :SIZE], o.readDepth()[:, :SIZE], "view %d" % v)
        mx, mean = colour_diff(g.readColour(), o.readColour())
        assert mx <= 1, "view %d: colour differs by up to %d LSB (mean %.4f)" % (v, mx, mean)
    g.close()
    o.close()


@pytest.mark.gpu
def test_batched_command_buffer_replay(gpu_lib):
    """The batched pass recorded once and replayed as a graph gives the same
    atlas as the immediate path, on every replay."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    batched, _ = _scenes()
    p = PuresoftPipeline(batched.width, batched.height)
    S.replay_setup(batched, p)
    S.replay_frame(batched, p)
    ref = p.readColour().copy()
    p.beginCommands()
    S.replay_frame(batched, p)
    cb = p.endCommands()
    for _ in range(3):
        p.clearColour(0)
        p.finish()
        cb.submit()
        assert np.array_equal(p.readColour(), ref)
    cb.destroy()
    p.close()


def _small_soup(n, w, h, seed=11, size=0.02):
    """n small triangles scattered over the whole target at random depths."""
    from kat_scenes import _scene
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, size=(n, 1, 2))
    d = rng.uniform(-size, size, size=(n, 3, 2))
    z = rng.uniform(-0.9, 0.9, size=(n, 3, 1))
    xy = c + d
    clip = np.concatenate([xy, z, np.ones((n, 3, 1))], axis=2).reshape(-1, 4)
    return _scene("soup_%d_%dx%d" % (n, w, h), w, h, clip, behavior_off=4)


@pytest.mark.gpu
@pytest.mark.parametrize("bin_w,passes", [(16, 2), (8, 3)])
def test_bin_sort_large_grids(gpu_lib, bin_w, passes):
    """6144x4224: 50688 bins of 16 columns (16-bit bin numbers, two radix
    passes) or 101376 bins of 8 columns (17 bits, three passes)."""
    from common import assert_depth_exact, render
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    scene = _small_soup(3000, 6144, 4224)
    bins = -(-6144 // bin_w) * -(-4224 // 32)
    assert (bins - 1).bit_length() > 8 * (passes - 1)
    g = PuresoftPipeline(scene.width, scene.height)
    g.setBinWidth(bin_w)
    gpu = render(g, scene)
    ora = render(OraclePipeline(scene.width, scene.height), scene)
    assert (gpu["depth"] < 1.0).sum() > 100000
    assert_depth_exact(gpu["depth"], ora["depth"], scene.name)
    mx, mean = colour_diff(gpu["colour"], ora["colour"])
    assert mx <= 1, "colour differs by up to %d LSB (mean %.4f)" % (mx, mean)


@pytest.mark.gpu
@pytest.mark.parametrize("bin_w", [8, 32])
def test_single_bin_and_tiny_targets(gpu_lib, bin_w):
    """A 24x20 target: one bin at 32 columns (nothing to sort), three at 8."""
    from common import assert_depth_exact, render
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    scene = _small_soup(40, 24, 20, seed=5, size=0.5)
    g = PuresoftPipeline(scene.width, scene.height)
    g.setBinWidth(bin_w)
    gpu = render(g, scene)
    ora = render(OraclePipeline(scene.width, scene.height), scene)
    assert_depth_exact(gpu["depth"], ora["depth"], scene.name)
    assert colour_diff(gpu["colour"], ora["colour"])[0] <= 1
