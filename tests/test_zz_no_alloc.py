"""ps3d_finish_noalloc (fixed device scratch, no allocation) against
ps3d_finish on the same recorded frames: depth bit-exact and colour within
1 LSB per channel, on two calls in a row; a pass too large for the fixed
scratch is refused before anything runs; a pass whose bin lists overflow it
is completed by ps3d_finish.  Collected last so that it also runs after
every other GPU test in the same process."""
import numpy as np
import pytest

from common import assert_depth_exact, colour_diff
from golden.make_golden import golden_cases
from kat_scenes import _scene, _tri_mesh

COLOUR_TOL = 1  # LSB per channel
CASES = [c for c in golden_cases() if c[0].split("_")[0] in ("c1", "c2") or c[0].startswith("kat_soup_lit")
         or c[0].startswith("kat_alphatest_blend") or c[0].startswith("kat_post")]


def _outputs(pipe, scene):
    out = {"colour": pipe.readColour().copy(),
           "depth": pipe.readDepthTexture(scene.info["depth_texture"]).copy()}
    if "shadow_texture" in scene.info:
        out["shadow"] = pipe.readDepthTexture(scene.info["shadow_texture"]).copy()
    return out


def _reference(scene):
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    p = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, p)
    S.replay_frame(scene, p)
    p.finish()
    out = _outputs(p, scene)
    p.close()
    return out


def _same(a, b, what):
    for k in a:
        if k == "colour":
            mx, mean = colour_diff(a[k], b[k])
            assert mx <= COLOUR_TOL, "%s: colour differs by up to %d LSB (mean %.4f)" % (what, mx, mean)
        else:
            assert_depth_exact(a[k], b[k], "%s %s" % (what, k))


@pytest.mark.gpu
@pytest.mark.parametrize("name,scene", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_finish(name, scene, gpu_lib):
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline, allocation_count
    ref = _reference(scene)
    p = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, p)
    p.finish()
    p.finishNoAlloc()  # first call: looks the scratch address up
    allocs = allocation_count()
    for call in range(2):
        S.replay_frame(scene, p)
        p.finishNoAlloc()
        # the defining property: no device or pinned allocation was made
        assert allocation_count() == allocs, "%s call %d allocated" % (name, call + 1)
        _same(ref, _outputs(p, scene), "%s call %d" % (name, call + 1))
    p.close()


def _quads(n, w, h):
    """n full-viewport quads at scattered depths: many bin pairs per triangle."""
    clip = []
    for k in range(n):
        z = 0.5 + 0.4 * np.sin(k * 1.7)
        a, b, c, d = [-1, -1, z, 1], [1, -1, z, 1], [1, 1, z, 1], [-1, 1, z, 1]
        clip += [a, b, c, a, c, d]
    return _scene("quads_%d_%dx%d" % (n, w, h), w, h, clip, behavior_off=4)


@pytest.mark.gpu
def test_noalloc_refuses_oversized_pass(gpu_lib):
    """A 2048x2048 colour pass needs 32 MiB for its shade list alone."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    scene = _quads(4, 2048, 2048)
    ref = _reference(scene)
    p = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, p)
    p.finish()
    S.replay_frame(scene, p)
    with pytest.raises(IndexError, match="fixed scratch"):
        p.finishNoAlloc()
    p.finish()  # the commands stayed recorded
    _same(ref, _outputs(p, scene), "oversized pass")
    p.close()


@pytest.mark.gpu
def test_noalloc_bin_overflow_completed_by_finish(gpu_lib):
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    scene = _quads(2000, 1024, 1024)
    ref = _reference(scene)
    p = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, p)
    p.finish()
    S.replay_frame(scene, p)
    with pytest.raises(MemoryError, match="bin pairs"):
        p.finishNoAlloc()
    p.finish()
    _same(ref, _outputs(p, scene), "bin overflow")
    # the same pipeline takes the no-allocation path again: the frame with a
    # two-quad VAO in place of the 2000-quad one
    mesh = _tri_mesh(np.asarray([[-1, -1, 0.3, 1], [1, -1, 0.3, 1], [1, 1, 0.3, 1]] * 2, dtype=np.float32))
    vao = p.createVAO()
    for slot, key in ((0, "position"), (3, "normal"), (4, "uv")):
        p.attachVBO(vao, slot, mesh[key])
    small = [op if op[0] != "drawVAO" else ("drawVAO", vao) for op in scene.frame]
    S.replay_ops(small, p)
    p.finishNoAlloc()
    S.replay_ops(small, p)
    p.finish()
    again = _outputs(p, scene)
    S.replay_ops(small, p)
    p.finishNoAlloc()
    _same(again, _outputs(p, scene), "after the overflow")
    p.close()
