"""GPU path against the oracle and the golden fixtures: depth (hence
coverage) bit-exact, colour within 1 LSB per 8-bit channel."""
import numpy as np
import pytest

from common import assert_depth_exact, colour_diff, load_golden, render, sha
from cpu_backends import OraclePipeline
from golden.make_golden import golden_cases, scene_digest

CASES = golden_cases()
COLOUR_TOL = 1  # LSB per channel


@pytest.mark.gpu
@pytest.mark.parametrize("name,scene", CASES, ids=[c[0] for c in CASES])
def test_gpu_matches_oracle(name, scene, gpu_lib):
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    gpu = render(PuresoftPipeline(scene.width, scene.height), scene)
    ora = render(OraclePipeline(scene.width, scene.height), scene)
    assert_depth_exact(gpu["depth"], ora["depth"], name)
    if "shadow" in ora:
        assert_depth_exact(gpu["shadow"], ora["shadow"], name + " shadow map")
    mx, mean = colour_diff(gpu["colour"], ora["colour"])
    assert mx <= COLOUR_TOL, "%s: colour differs by up to %d LSB (mean %.4f)" % (name, mx, mean)
    # pinned to the reference build's own render of the same inputs: the
    # inputs generated on this host must be the fixture's
    g = load_golden(name)
    assert scene_digest(scene) == str(g["digest"]), "%s: scene inputs differ from the fixture's" % name
    assert sha(gpu["depth"]) == str(g["depth_sha"]), name
    if "shadow_sha" in g:
        assert sha(gpu["shadow"]) == str(g["shadow_sha"]), name
    # colour is the reference build's bit for bit (the rcpps / rsqrtss
    # tables included), except that the scene viewer's spotlight uses the
    # device's acosf / cosf where the reference build has glibc's
    if "viewer" not in name:
        assert sha(gpu["colour"]) == str(g["colour_sha"]), name + ": colour differs from the reference build"
    for k in ora:
        if k.startswith("tex"):  # a texture the scene rendered into through setFBO
            assert np.array_equal(gpu[k], ora[k]), name + " " + k
            assert sha(gpu[k]) == str(g[k + "_sha"]), name + " " + k


@pytest.mark.gpu
@pytest.mark.parametrize("name,scene", CASES, ids=[c[0] for c in CASES])
def test_deferred_varyings_match_oracle(name, scene, gpu_lib):
    """The shade computing its winners' vertex varyings (the set-up storing
    none) gives the oracle's frame on every golden case; passes that blend
    or discard keep stored varyings."""
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    g = PuresoftPipeline(scene.width, scene.height)
    g.setLazyVaryings(True)
    gpu = render(g, scene)
    ora = render(OraclePipeline(scene.width, scene.height), scene)
    assert_depth_exact(gpu["depth"], ora["depth"], name)
    mx, mean = colour_diff(gpu["colour"], ora["colour"])
    assert mx <= COLOUR_TOL, "%s: colour differs by up to %d LSB (mean %.4f)" % (name, mx, mean)


@pytest.mark.gpu
def test_fragment_counts_match_oracle(gpu_lib):
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in CASES if c[0].startswith("kat_soup_lit")][0]
    g = PuresoftPipeline(scene.width, scene.height)
    g.setFragmentCounting(True)
    render(g, scene)
    o = OraclePipeline(scene.width, scene.height)
    render(o, scene)
    st = g.stats()
    assert (st["fragments"], st["fragments_passed"]) == o.fragments()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c3_small", "c2_small", "kat_post_add_fog"])
def test_bin_capacity_replay(gpu_lib, monkeypatch, case):
    """A pass whose bin lists overflow the preallocated room is re-run
    transparently with larger buffers; the result is unchanged.  In the
    two-pass case (shadow pass, then the lit pass sampling it, on the two pass
    streams) the first pass overflows while the second may already run.  In
    the post-process case (pass, add, pass, fog, add) every post-process runs
    exactly once although the passes around them replay."""
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in CASES if c[0].startswith(case)][0]
    monkeypatch.setenv("PS3D_PAIR_CAP", "64")
    g = PuresoftPipeline(scene.width, scene.height)
    out = render(g, scene)
    assert g.stats()["replays"] >= 1
    ref = render(OraclePipeline(scene.width, scene.height), scene)
    assert_depth_exact(out["depth"], ref["depth"], name)
    if "shadow" in ref:
        assert_depth_exact(out["shadow"], ref["shadow"], name + " shadow map")
    assert colour_diff(out["colour"], ref["colour"])[0] <= COLOUR_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("split", [1, 2, 4, 8])
@pytest.mark.parametrize("cull", [1, 0])
@pytest.mark.parametrize("occupancy", [0, 8])
@pytest.mark.parametrize("bin_w", [8, 16, 32])
@pytest.mark.parametrize("case", ["kat_soup_depth", "c3_small", "kat_post_add_fog", "kat_alphatest_blend",
                                  "kat_def0_planet_cloud"])
def test_schedules_agree(gpu_lib, bin_w, occupancy, cull, split, case):
    """Every schedule (bin width x raster kernel variants: occupancy, span
    culling, row split) gives the oracle's result."""
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in CASES if c[0].startswith(case)][0]
    g = PuresoftPipeline(scene.width, scene.height)
    g.setBinWidth(bin_w)
    g.setRasterOccupancy(occupancy)
    g.setSpanCulling(cull)
    g.setRowSplit(split)
    assert g.binWidth() == bin_w
    out = render(g, scene)
    ref = render(OraclePipeline(scene.width, scene.height), scene)
    assert_depth_exact(out["depth"], ref["depth"], name)
    mx, mean = colour_diff(out["colour"], ref["colour"])
    assert mx <= COLOUR_TOL, "%s: colour differs by up to %d LSB (mean %.4f)" % (name, mx, mean)


@pytest.mark.gpu
@pytest.mark.parametrize("split", [1, 2, 4, 8])
@pytest.mark.parametrize("cull", [1, 0])
@pytest.mark.parametrize("bin_w", [8, 16])
@pytest.mark.parametrize("case", ["kat_soup_depth", "c3_small", "kat_post_add_fog", "kat_alphatest_blend",
                                  "kat_def0_planet_cloud", "kat_basic_notest", "kat_blend_notest"])
def test_warp_bin_schedules_agree(gpu_lib, bin_w, cull, split, case):
    """The one-warp-per-bin raster (every bin width it serves, span culling
    on and off, every row split) gives the oracle's result; passes that
    blend or discard keep the shared-bin raster and must agree too."""
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in CASES if c[0].startswith(case)][0]
    g = PuresoftPipeline(scene.width, scene.height)
    g.setBinWidth(bin_w)
    g.setWarpBins(True)
    g.setSpanCulling(cull)
    g.setRowSplit(split)
    g.setFragmentCounting(True)
    out = render(g, scene)
    o = OraclePipeline(scene.width, scene.height)
    ref = render(o, scene)
    assert_depth_exact(out["depth"], ref["depth"], name)
    if "shadow" in ref:
        assert_depth_exact(out["shadow"], ref["shadow"], name + " shadow map")
    mx, mean = colour_diff(out["colour"], ref["colour"])
    assert mx <= COLOUR_TOL, "%s: colour differs by up to %d LSB (mean %.4f)" % (name, mx, mean)
    if case in ("kat_soup_depth", "c3_small", "kat_basic_notest"):  # passes without blending or discard
        st = g.stats()
        assert (st["fragments"], st["fragments_passed"]) == o.fragments(), name


@pytest.mark.gpu
@pytest.mark.parametrize("warp", [0, 1])
@pytest.mark.parametrize("split", [1, 4])
@pytest.mark.parametrize("cull", [1, 0])
@pytest.mark.parametrize("bin_w", [8, 16, 32])
@pytest.mark.parametrize("case", ["kat_soup_depth", "kat_soup_lit", "c3_small", "c2_small", "kat_post_add_fog",
                                  "kat_def04_sky_soup", "kat_basic_notest", "c1_640x480"])
def test_span_item_schedules_agree(gpu_lib, bin_w, cull, split, warp, case):
    """Span items (short triangles binned per row span, set up before the
    raster) under every raster shape give the oracle's result and fragment
    counts."""
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in CASES if c[0].startswith(case)][0]
    g = PuresoftPipeline(scene.width, scene.height)
    g.setSpanItems(True)
    g.setBinWidth(bin_w)
    g.setWarpBins(warp)
    g.setSpanCulling(cull)
    g.setRowSplit(split)
    g.setFragmentCounting(True)
    out = render(g, scene)
    o = OraclePipeline(scene.width, scene.height)
    ref = render(o, scene)
    assert_depth_exact(out["depth"], ref["depth"], name)
    if "shadow" in ref:
        assert_depth_exact(out["shadow"], ref["shadow"], name + " shadow map")
    mx, mean = colour_diff(out["colour"], ref["colour"])
    assert mx <= COLOUR_TOL, "%s: colour differs by up to %d LSB (mean %.4f)" % (name, mx, mean)
    if case not in ("kat_post_add_fog", "kat_def04_sky_soup"):
        st = g.stats()
        assert (st["fragments"], st["fragments_passed"]) == o.fragments(), name


@pytest.mark.gpu
def test_repeated_frames_identical(gpu_lib):
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    scene = S.scene_c1()
    g = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, g)
    outs = []
    for _ in range(3):
        S.replay_frame(scene, g)
        g.flush()
        outs.append(g.readColour().copy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])


@pytest.mark.gpu
def test_command_buffer_graph_replay_matches_immediate(gpu_lib):
    """A recorded frame replayed as a CUDA graph renders what the immediate
    path renders, frame after frame."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    scene = S.scene_c2(width=320, height=180, shadow_size=256, meshes=12, tex_size=64, spread=5.0)
    g = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, g)
    S.replay_frame(scene, g)
    ref = (g.readColour().copy(), g.readDepthTexture(scene.info["depth_texture"]).copy())
    g.beginCommands()
    S.replay_frame(scene, g)
    cb = g.endCommands()
    for i in range(4):
        g.clearColour(0)
        g.finish()
        cb.submit(upload_inputs=(i % 2 == 1))
        col = g.readColour()
        dep = g.readDepthTexture(scene.info["depth_texture"])
        assert np.array_equal(col, ref[0]), i
        assert np.array_equal(dep.view(np.uint32), ref[1].view(np.uint32)), i
    cb.destroy()


@pytest.mark.gpu
def test_fast_division_is_correctly_rounded(gpu_lib):
    """The kernels' FMA-corrected reciprocal and quotient equal CUDA's IEEE
    results (every mantissa of exponents -100..100; 2^28 random pairs)."""
    from puresoft3d_gb300.pipeline import selftest_division
    assert selftest_division(1 << 28) == (0, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("repeats", [2, 3, 9])
def test_repeated_multipass_frames_in_one_launch(gpu_lib, repeats):
    """The two-pass frame (shadow map, then the lit pass sampling it)
    recorded `repeats` times before one finish: 4 and 6 passes run on the two
    pass streams -- the second shadow pass must wait for the first lit pass
    that samples the map it overwrites -- and 18 on one stream.  The result
    equals one frame on the oracle."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in CASES if c[0].startswith("c2_small")][0]
    g = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, g)
    for _ in range(repeats):
        S.replay_frame(scene, g)
    g.finish()
    ref = render(OraclePipeline(scene.width, scene.height), scene)
    assert_depth_exact(g.readDepthTexture(scene.info["depth_texture"]), ref["depth"], name)
    assert_depth_exact(g.readDepthTexture(scene.info["shadow_texture"]), ref["shadow"], name + " shadow map")
    assert colour_diff(g.readColour(), ref["colour"])[0] <= COLOUR_TOL


@pytest.mark.gpu
def test_device_wait_runs_out_and_pipeline_recovers(gpu_lib):
    """A bounded device wait on a flag that nothing sets gives up after its
    poll limit; the host reports PS3D_ERR_TIMEOUT and the pipeline then
    renders correctly."""
    import re
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in CASES if c[0].startswith("kat_soup_lit")][0]
    g = PuresoftPipeline(scene.width, scene.height)
    with pytest.raises(TimeoutError) as e:
        g.selftestWait(1 << 14)
    ms = float(re.match(r"([0-9.]+) ms", str(e.value)).group(1))
    assert 0.0 < ms < 2000.0
    out = render(g, scene)
    ref = render(OraclePipeline(scene.width, scene.height), scene)
    assert_depth_exact(out["depth"], ref["depth"], name)
    assert colour_diff(out["colour"], ref["colour"])[0] <= COLOUR_TOL


@pytest.mark.gpu
def test_layered_texture_gpu(gpu_lib):
    """Layered textures on the device: per-layer write and read back, zeroed
    extra layers, out-of-range layers and layer counts refused, and a
    skybox draw refused when its texture is not a six-layer cube map."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    p = PuresoftPipeline(16, 16)
    face = np.arange(6 * 5 * 4, dtype=np.uint8).reshape(6, 5, 4)
    idx = p.createTexture(5, 6, 20, 4, face, 0, extra_layers=5)
    assert np.array_equal(p.readTexture(idx, 0), face.reshape(6, 20))
    assert not p.readTexture(idx, 3).any()
    p.writeTextureLayer(idx, 3, face[::-1])
    assert np.array_equal(p.readTexture(idx, 3), face[::-1].reshape(6, 20))
    with pytest.raises(IndexError):
        p.readTexture(idx, 6)
    with pytest.raises(IndexError):
        p.createTexture(5, 6, 20, 4, face, 0, extra_layers=6)
    flat = p.createTexture(5, 6, 20, 4, face, 0)
    prog = p.createProgramme(p.addProcessor(S.VP_DEF04), p.addProcessor(S.IP_DEF04), p.addProcessor(S.FP_DEF04))
    p.useProgramme(prog)
    vao = p.createVAO()
    p.attachVBO(vao, 0, np.array([[-1, 1, 0, 1], [-1, -1, 0, 1], [1, -1, 0, 1]], dtype=np.float32))
    p.setUniform(1, S.col_major(np.eye(4)))
    p.setUniform(2, np.array([flat], dtype=np.int32))
    with pytest.raises(ValueError):
        p.drawVAO(vao)
    p.setUniform(2, np.array([idx], dtype=np.int32))
    p.drawVAO(vao)
    p.finish()
    p.close()


@pytest.mark.gpu
def test_post_process_arguments(gpu_lib):
    """Unknown post-processors and short parameters are refused at record
    time; the fog needs a depth buffer covering the colour buffer."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    p = PuresoftPipeline(32, 16)
    with pytest.raises(ValueError):
        p.postProcess(0x7777)
    with pytest.raises(ValueError):
        p.postProcess(S.PP_ADD8, b"\x01")
    with pytest.raises(ValueError):
        p.postProcess(S.PP_FOG, None)
    small = p.createTexture(16, 16, 64, 4, None, 0)
    p.setDepth(small)
    with pytest.raises(ValueError):
        p.postProcess(S.PP_FOG, S.fog_params(0, 0.0, 1.0))
    p.setDepth(-1)
    p.clearDepth(1.0)
    p.clearColour(0x01020304)
    p.postProcess(S.PP_FOG, S.fog_params(0xFFFFFFFF, 0.0, 1.0))  # depth cleared to 1.0: full fog
    p.postProcess(S.PP_ADD8, S.add8_params(1, 1, 1, 1))
    img = p.readColour()
    assert (img.reshape(-1, 4) == np.array([0, 0, 0, 2], dtype=np.uint8)).all()  # 255 + 1 wraps; alpha 1 + 1
    p.close()


@pytest.mark.gpu
def test_span_occlusion_is_conservative(gpu_lib):
    """The raster drops a span before computing its depths when no pixel
    can pass the depth test; on random spans with depth bounds at the
    pass/fail boundary it never drops one with a passing pixel, and does
    drop many."""
    from puresoft3d_gb300.pipeline import selftest_occlusion
    wrong, dropped = selftest_occlusion(1 << 22)
    assert wrong == 0
    assert dropped > (1 << 22) // 20


@pytest.mark.gpu
def test_forward_pass_waits_for_earlier_colour_pass(gpu_lib):
    """Two passes on the two pass streams: a lit pass into one depth target,
    then a blended (forward) pass into another, which reads the colour the
    first pass's shade wrote; repeated frames match the oracle every time."""
    from kat_scenes import _alpha_texture, _tri_mesh, random_soup
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    b = S._Builder()
    opaque = b.texture(S.checker_noise_bgra(16, 4, np.random.default_rng(5)))
    alpha = b.texture(_alpha_texture(6))
    d1, d2 = b.empty_texture(96, 64), b.empty_texture(96, 64)
    prog = b.programme(S.VP_DEF01, S.IP_DEF01, S.FP_LIT1)
    va = b.vao(_tri_mesh(random_soup(400, 31)), slots=(0, 3, 4))
    vb = b.vao(_tri_mesh(random_soup(200, 32)), slots=(0, 3, 4))
    eye = np.eye(4)
    b.f("clearColour", 0xFF000000)
    b.f("useProgramme", prog)
    for slot in (3, 4, 5):
        b.f("setUniform", slot, S.col_major(eye))
    b.f("setUniform", 7, S.vec4(0.3, 0.5, 0.81))
    b.f("setUniform", 8, S.vec4(0, 0, 2, 1))
    b.f("setDepth", d1)
    b.f("clearDepth", 1.0)
    b.f("setUniform", 9, np.array([opaque], dtype=np.int32))
    b.f("drawVAO", va)
    b.f("setDepth", d2)
    b.f("clearDepth", 1.0)
    b.f("enable", S.ALPHABLEND)
    b.f("setUniform", 9, np.array([alpha], dtype=np.int32))
    b.f("drawVAO", vb)
    b.f("disable", S.ALPHABLEND)
    scene = S.Scene("fwd_after_colour", 96, 64, b.setup, b.frame, {"triangles": 600, "depth_texture": d2})
    o = OraclePipeline(96, 64)
    S.replay_setup(scene, o)
    S.replay_frame(scene, o)
    want = o.readColour()
    g = PuresoftPipeline(96, 64)
    S.replay_setup(scene, g)
    for _ in range(20):
        S.replay_frame(scene, g)
        got = g.readColour()
        assert colour_diff(got, want)[0] <= COLOUR_TOL


def _tiny_thin_clip(w, h, seed):
    """Triangles in pixel units turned into clip space: sub-pixel ones, slivers
    whose every row is empty, spans clamped away at the left and right
    edges, and thin triangles 30-35 rows tall (around the set-up's exact-span
    limit of 32 rows), in both orientations."""
    rng = np.random.default_rng(seed)
    tris = []
    for _ in range(300):  # sub-pixel and few-pixel
        c = rng.uniform([-2, -2], [w + 2, h + 2])
        tris.append(c + rng.normal(size=(3, 2)) * rng.uniform(0.2, 2.0))
    for _ in range(80):  # horizontal slivers across a row boundary
        y = rng.integers(1, h - 1) + rng.uniform(-0.3, 0.3)
        x = rng.uniform(0, w)
        tris.append(np.array([[x, y], [x + rng.uniform(2, 20), y + rng.uniform(-0.4, 0.4)], [x + 1, y + 0.45]]))
    for _ in range(80):  # vertical needles, under a pixel wide
        x, y = rng.uniform(-1, w + 1), rng.uniform(0, h)
        tris.append(np.array([[x, y], [x + rng.uniform(0.05, 0.9), y], [x + rng.uniform(0, 0.9), y + rng.uniform(3, 40)]]))
    for rows in (30, 31, 32, 33, 34, 35):  # around the exact-span limit
        for _ in range(6):
            x, y = rng.uniform(0, w), rng.uniform(0, h - rows - 1)
            tris.append(np.array([[x, y], [x + rng.uniform(0.5, 6), y + 0.2], [x + rng.uniform(-3, 3), y + rows + 0.5]]))
    out = []
    for t in tris:
        if rng.random() < 0.5:
            t = t[::-1]  # either winding
        z = rng.uniform(-0.9, 0.9)
        for px, py in t:
            wc = rng.uniform(0.7, 1.6)
            out.append([(2 * px / w - 1) * wc, (2 * py / h - 1) * wc, (z + rng.normal() * 0.02) * wc, wc])
    return np.array(out, dtype=np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("bin_w", [8, 16, 32])
def test_tiny_and_thin_triangles(gpu_lib, bin_w):
    """The set-up's exact spans drop triangles with no pixel and trim bins and
    rows to the spans: on triangles built to hit those cases the GPU gives
    the oracle's depth bit for bit, its colour within 1 LSB and the same
    fragment counts."""
    import kat_scenes as K
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    w, h = 96, 80
    scene = K._scene("tiny_thin", w, h, _tiny_thin_clip(w, h, 5), lit=True)
    g = PuresoftPipeline(w, h)
    g.setBinWidth(bin_w)
    g.setFragmentCounting(True)
    out = render(g, scene)
    o = OraclePipeline(w, h)
    ref = render(o, scene)
    assert_depth_exact(out["depth"], ref["depth"], "tiny_thin")
    assert colour_diff(out["colour"], ref["colour"])[0] <= COLOUR_TOL
    st = g.stats()
    assert (st["fragments"], st["fragments_passed"]) == o.fragments()
    assert int((ref["depth"] < 1.0).sum()) > 500  # the scene covers something


def _soup_clip(n, seed, back=False):
    """n small triangles over the target at random depths, in clip space, all
    wound to face the viewer (back: all away from it)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.95, 0.95, size=(n, 1, 2))
    d = rng.uniform(-0.15, 0.15, size=(n, 3, 2))
    z = rng.uniform(-0.9, 0.9, size=(n, 3, 1))
    t = np.concatenate([c + d, z, np.ones((n, 3, 1))], axis=2)
    e1, e2 = t[:, 1, :2] - t[:, 0, :2], t[:, 2, :2] - t[:, 1, :2]
    cz = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]  # z of cross(v1 - v0, v2 - v1)
    flip = (cz < 0) != back
    t[flip] = t[flip][:, ::-1]
    return t.reshape(-1, 4)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 127, 128, 129, 255, 256, 257, 1000, 3000])
def test_setup_group_boundaries(gpu_lib, n):
    """The set-up takes triangles in ticketed groups of 128 and emits a
    group's pairs after setting up its next group: triangle counts around the
    group size (a partial last group, one group, a group and one triangle,
    more groups than blocks at once) give the oracle's depth bit for bit, its
    colour within 1 LSB and the same fragment counts; so does a pass whose
    triangles all face away under culling (no pair at all)."""
    import kat_scenes as K
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    w, h = 96, 64
    for culled in (False, True):
        clip = _soup_clip(n, 100 + n, back=culled)  # culled: every triangle faces away, culling on
        scene = K._scene("groups_%d_%d" % (n, culled), w, h, clip, lit=True,
                         behavior_on=K.S.FACE_CULLING if culled else 0)
        g = PuresoftPipeline(w, h)
        g.setFragmentCounting(True)
        out = render(g, scene)
        o = OraclePipeline(w, h)
        ref = render(o, scene)
        assert_depth_exact(out["depth"], ref["depth"], scene.name)
        assert colour_diff(out["colour"], ref["colour"])[0] <= COLOUR_TOL
        st = g.stats()
        assert (st["fragments"], st["fragments_passed"]) == o.fragments(), scene.name
        g.close()
