"""Known-answer scenes for the rasteriser, interpolator and depth test.

Each scene feeds clip-space positions straight through (PV = M = identity),
so a case states exactly which pixels and depths it exercises: flat tops and
bottoms, left- and right-pointing triangles, edges off every side of the
viewport, shared edges (the depth test's -1e-4 epsilon, reference
fragthrd.cpp:227), equal-depth overlaps (first one wins), zero-area and
needle triangles, back faces with and without culling, z-reject
(drawvao.cpp:51-56), depth test off, strong perspective, and a seeded random
soup with heavy overlap.  Odd viewport sizes exercise the integer half-size
viewport mapping (rasterizer.cpp:30-31).
"""
from __future__ import annotations

import numpy as np

from puresoft3d_gb300 import scenes as S


def _tri_mesh(clip):
    """clip: (n_tris*3, 4) positions -> a mesh with normal/uv varyings."""
    clip = np.asarray(clip, dtype=np.float32).reshape(-1, 4)
    n = len(clip)
    idx = np.arange(n)
    normal = np.stack([np.sin(idx * 0.7), np.cos(idx * 0.3), np.ones(n) * 0.5, np.zeros(n)], 1).astype(np.float32)
    uv = np.stack([(idx % 7) / 3.0 - 0.5, (idx % 5) / 2.0 - 0.25], 1).astype(np.float32)
    tangent = np.stack([np.ones(n), np.sin(idx * 0.2) * 0.3, np.zeros(n), np.zeros(n)], 1).astype(np.float32)
    binormal = np.stack([np.cos(idx * 0.5) * 0.2, np.ones(n), np.sin(idx * 0.4) * 0.2, np.zeros(n)], 1).astype(np.float32)
    # vertex colour (B, G, R, A floats), partly outside 0..255 so that the clamp works
    colour = np.stack([(idx * 37) % 300 - 20, (idx * 53) % 256, (idx * 71) % 280, (idx * 13) % 256],
                      1).astype(np.float32)
    return {"position": clip, "normal": normal, "uv": uv, "tangent": tangent, "binormal": binormal,
            "colour": colour}


def _alpha_texture(seed):
    """A 16x16 BGRA texture whose alpha runs over 0..255 in a seeded checker,
    so an alpha test discards some fragments and blending weights differ."""
    rng = np.random.default_rng(seed)
    img = S.checker_noise_bgra(16, 4, rng).copy()
    yy, xx = np.mgrid[0:16, 0:16]
    img[..., 3] = (np.array([0, 90, 140, 255], dtype=np.uint8)[(yy // 4 + xx // 4) % 4]
                   + rng.integers(0, 20, size=(16, 16))).clip(0, 255).astype(np.uint8)
    return img


def _bump_texture(seed):
    """A 16x16 BGRA tangent-space bump map: r, g around 128, b near 255."""
    rng = np.random.default_rng(seed)
    img = np.empty((16, 16, 4), dtype=np.uint8)
    img[..., 2] = rng.integers(70, 186, size=(16, 16))   # r -> x
    img[..., 1] = rng.integers(70, 186, size=(16, 16))   # g -> y
    img[..., 0] = rng.integers(200, 256, size=(16, 16))  # b -> z
    img[..., 3] = 255
    return img


def _scene(name, w, h, clip, lit=True, behavior_off=0, texture_seed=7, fp=None, behavior_on=0):
    b = S._Builder()
    rng = np.random.default_rng(texture_seed)
    tex = b.texture(_alpha_texture(texture_seed) if (fp == S.FP_LIT1A or behavior_on & S.ALPHABLEND)
                    else S.checker_noise_bgra(16, 4, rng))
    depth = b.empty_texture(w, h)
    mesh = _tri_mesh(clip)
    if fp == S.FP_DEF03:  # the reference's bump-mapped processors (tex1bump1light1.cpp)
        bump = b.texture(_bump_texture(texture_seed + 1))
        prog = b.programme(S.VP_DEF03, S.IP_DEF03, S.FP_DEF03)
        vao = b.vao(mesh, slots=(0, 1, 2, 3, 4))
    elif fp == S.FP_DEF02:  # the reference's vertex-colour processors (colr1light1.cpp)
        prog = b.programme(S.VP_DEF02, S.IP_DEF02, S.FP_DEF02)
        vao = b.vao(mesh, slots={0: "position", 1: "normal", 2: "colour"})
    elif lit:
        prog = b.programme(S.VP_DEF01, S.IP_DEF01, fp or S.FP_LIT1)
        vao = b.vao(mesh, slots=(0, 3, 4))
    else:
        prog = b.programme(S.VP_SHADOW, S.IP_DEF05, S.FP_DEF05)
        vao = b.vao(mesh, slots=(0,))
    eye = np.eye(4)
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF101010)
    if behavior_off:
        b.f("disable", behavior_off)
    if behavior_on:
        b.f("enable", behavior_on)
    b.f("useProgramme", prog)
    b.f("setUniform", 3, S.col_major(eye))
    b.f("setUniform", 4, S.col_major(eye))
    b.f("setUniform", 5, S.col_major(eye))
    b.f("setUniform", 7, S.vec4(0.3, 0.5, 0.81))
    b.f("setUniform", 8, S.vec4(0, 0, 2, 1))
    b.f("setUniform", 9, np.array([tex], dtype=np.int32))
    if fp == S.FP_DEF03:
        b.f("setUniform", 10, np.array([bump], dtype=np.int32))
    b.f("drawVAO", vao)
    return S.Scene(name, w, h, b.setup, b.frame, {"triangles": len(mesh["position"]) // 3, "depth_texture": depth})


def _cube_faces(size, seed):
    """Six size x size BGRA faces: a per-face base colour, a 4-texel
    checker and seeded noise, alpha varying, so that every face and texel
    is told apart."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:size, 0:size]
    faces = []
    for f in range(6):
        img = np.empty((size, size, 4), dtype=np.uint8)
        base = np.array([40 * f + 20, 255 - 35 * f, (97 * f) % 256], dtype=np.int32)
        chk = ((yy // 4 + xx // 4) % 2) * 50
        for c in range(3):
            img[..., c] = np.clip(base[c] + chk + rng.integers(-12, 13, size=(size, size)), 0, 255)
        img[..., 3] = np.clip(60 + 3 * xx + 2 * yy + 10 * f, 0, 255)
        faces.append(img)
    return faces


def _rot(yaw, pitch, roll=0.0):
    cy, sy, cp, sp, cr, sr = (np.cos(yaw), np.sin(yaw), np.cos(pitch), np.sin(pitch), np.cos(roll), np.sin(roll))
    ry = np.array([[cy, 0, sy, 0], [0, 1, 0, 0], [-sy, 0, cy, 0], [0, 0, 0, 1]])
    rx = np.array([[1, 0, 0, 0], [0, cp, -sp, 0], [0, sp, cp, 0], [0, 0, 0, 1]])
    rz = np.array([[cr, -sr, 0, 0], [sr, cr, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]])
    v = rz @ rx @ ry
    v[:3, 3] = [0.3, -0.2, 1.5]  # a translation, which the skybox's rotation drops
    return v


def _skybox_scene(name, w, h, view, face_size, wrap, soup_seed=None, blend=False):
    """The reference's skybox (skybox.cpp; the demo's Skybox::draw,
    test/testobjs.cpp:162-224): a full-view quad of two triangles in clip
    space, depth test and update off, the cube map at uniform 2 and the view
    at uniform 1; then, optionally, a DEF01 soup over it with depth on."""
    b = S._Builder()
    cube = b.layered_texture(_cube_faces(face_size, 5 + face_size), wrap=wrap)
    depth = b.empty_texture(w, h)
    quad = np.array([[-1, 1, 0, 1], [-1, -1, 0, 1], [1, -1, 0, 1],
                     [1, -1, 0, 1], [1, 1, 0, 1], [-1, 1, 0, 1]], dtype=np.float32)
    sky = b.programme(S.VP_DEF04, S.IP_DEF04, S.FP_DEF04)
    sky_vao = b.vao({"position": quad}, slots=(0,))
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0x80101010)
    if blend:
        b.f("enable", S.ALPHABLEND)
    b.f("useProgramme", sky)
    b.f("setUniform", 1, S.col_major(view))
    b.f("setUniform", 2, np.array([cube], dtype=np.int32))
    b.f("disable", S.UPDATE_DEPTH | S.TEST_DEPTH)
    b.f("drawVAO", sky_vao)
    b.f("enable", S.UPDATE_DEPTH | S.TEST_DEPTH)
    tris = 2
    if soup_seed is not None:
        rng = np.random.default_rng(soup_seed)
        tex = b.texture(S.checker_noise_bgra(16, 4, rng))
        mesh = _tri_mesh(random_soup(150, soup_seed))
        prog = b.programme(S.VP_DEF01, S.IP_DEF01, S.FP_DEF01)
        vao = b.vao(mesh, slots=(0, 3, 4))
        eye = np.eye(4)
        b.f("useProgramme", prog)
        b.f("setUniform", 3, S.col_major(eye))
        b.f("setUniform", 4, S.col_major(eye))
        b.f("setUniform", 5, S.col_major(eye))
        b.f("setUniform", 7, S.vec4(0.3, 0.5, 0.81))
        b.f("setUniform", 8, S.vec4(0, 0, 2, 1))
        b.f("setUniform", 9, np.array([tex], dtype=np.int32))
        b.f("drawVAO", vao)
        tris += len(mesh["position"]) // 3
    return S.Scene(name, w, h, b.setup, b.frame, {"triangles": tris, "depth_texture": depth})


def _post_scene(name, w, h, seed):
    """The post-processing hook (post.cpp:3-19) between passes: a DEF01
    soup, the demo's per-byte add with wrap-around, a second soup over it,
    depth fog, and the add again with the demo's default addend."""
    b = S._Builder()
    rng = np.random.default_rng(seed)
    tex = b.texture(S.checker_noise_bgra(16, 4, rng))
    depth = b.empty_texture(w, h)
    m1, m2 = _tri_mesh(random_soup(150, seed)), _tri_mesh(random_soup(150, seed + 1))
    prog = b.programme(S.VP_DEF01, S.IP_DEF01, S.FP_LIT1)
    v1, v2 = b.vao(m1, slots=(0, 3, 4)), b.vao(m2, slots=(0, 3, 4))
    eye = np.eye(4)
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF101010)
    b.f("useProgramme", prog)
    for slot in (3, 4, 5):
        b.f("setUniform", slot, S.col_major(eye))
    b.f("setUniform", 7, S.vec4(0.3, 0.5, 0.81))
    b.f("setUniform", 8, S.vec4(0, 0, 2, 1))
    b.f("setUniform", 9, np.array([tex], dtype=np.int32))
    b.f("drawVAO", v1)
    b.f("postProcess", S.PP_ADD8, S.add8_params(10, 200, 77, 5))
    b.f("drawVAO", v2)
    b.f("postProcess", S.PP_FOG, S.fog_params(0xFF8040C0, -0.2, 0.9))
    b.f("postProcess", S.PP_ADD8, None)
    return S.Scene(name, w, h, b.setup, b.frame, {"triangles": 300, "depth_texture": depth})


def _setfbo_scene(name, w, h, seed):
    """Render to texture through setFBO (pipeline.cpp:260-275): a soup drawn
    into a 64x48 BGRA8 texture bound as FBO slot 0 (rows bottom-up, its
    seeded contents where nothing is drawn), the demo's add and depth fog
    post-processed on it (postProcess runs on slot 0, post.cpp:14), and a
    blended soup over it; clearColour meanwhile clears the display only
    (pipeline.cpp:340-343).  Then slot 0 back to the display and a second
    soup drawn there sampling the texture.  Colour, depth and the texture
    are compared."""
    b = S._Builder()
    rng = np.random.default_rng(seed)
    src = b.texture(_alpha_texture(seed))
    tw, th = 64, 48
    target = b.texture(S.checker_noise_bgra(64, 8, rng, noise=40)[:th], wrap=True)
    d1, d2 = b.empty_texture(tw, th), b.empty_texture(w, h)
    m1, m2, m3 = (_tri_mesh(random_soup(120, seed + k)) for k in range(3))
    prog = b.programme(S.VP_DEF01, S.IP_DEF01, S.FP_LIT1)
    v1, v2, v3 = (b.vao(m, slots=(0, 3, 4)) for m in (m1, m2, m3))
    eye = np.eye(4)
    b.f("setDepth", d1)
    b.f("clearDepth", 1.0)
    b.f("setFBO", 0, target)
    b.f("clearColour", 0xFF204060)  # the display, not the texture
    b.f("setViewport", tw, th)
    b.f("useProgramme", prog)
    for slot in (3, 4, 5):
        b.f("setUniform", slot, S.col_major(eye))
    b.f("setUniform", 7, S.vec4(0.3, 0.5, 0.81))
    b.f("setUniform", 8, S.vec4(0, 0, 2, 1))
    b.f("setUniform", 9, np.array([src], dtype=np.int32))
    b.f("drawVAO", v1)
    b.f("postProcess", S.PP_ADD8, S.add8_params(30, 5, 200, 9))
    b.f("postProcess", S.PP_FOG, S.fog_params(0xFF40C080, -0.3, 0.8))
    b.f("enable", S.ALPHABLEND)
    b.f("drawVAO", v2)
    b.f("disable", S.ALPHABLEND)
    b.f("setFBO", 0, -1)
    b.f("setDepth", d2)
    b.f("clearDepth", 1.0)
    b.f("setViewport", w, h)
    b.f("setUniform", 9, np.array([target], dtype=np.int32))
    b.f("drawVAO", v3)
    return S.Scene(name, w, h, b.setup, b.frame, {"triangles": 360, "depth_texture": d2, "read_textures": [target]})


def _planet_scene(name, w, h, seed, fp, blend=False):
    """The reference demo's planet processors (test/testproc.cpp) with the
    projective 4-tap Poisson shadow lookup (samplrproj.cpp): a depth-only
    pass renders a seeded soup from a light's view into a 64x64 FP32 shadow
    map, then the soup is drawn with VP_Planet / IP_Planet and FP_Earth (or
    FP_Satellite), its shadow coordinate projected by uniform 16 (the
    light's transform, x and y mapped to [0, 1])."""
    b = S._Builder()
    rng = np.random.default_rng(seed)
    diffuse = b.texture(S.checker_noise_bgra(32, 4, rng), wrap=True)
    bump = b.texture(_bump_texture(seed + 1), wrap=True)
    spec = b.texture(S.checker_noise_bgra(16, 2, rng, noise=60, lo=10, hi=240), wrap=True)
    night = b.texture(S.checker_noise_bgra(16, 8, rng, noise=20, lo=0, hi=90), wrap=True)
    shadow = b.empty_texture(64, 64)
    depth = b.empty_texture(w, h)
    mesh = _tri_mesh(random_soup(260, seed))
    shadow_prog = b.programme(S.VP_SHADOW, S.IP_DEF05, S.FP_DEF05)
    planet = b.programme(S.VP_PLANET, S.IP_PLANET, fp)
    vao = b.vao(mesh, slots=(0, 1, 2, 3, 4))
    c, s_ = np.cos(0.35), np.sin(0.35)
    light = np.array([[0.8 * c, 0.1, 0.5 * s_, 0.05], [0.0, 0.8, 0.1, -0.05], [-0.4 * s_, 0.0, 0.4 * c, 0.0],
                      [0.0, 0.0, 0.0, 1.0]])
    bias = np.array([[0.5, 0, 0, 0.5], [0, 0.5, 0, 0.5], [0, 0, 1, 0], [0, 0, 0, 1]])
    eye = np.eye(4)
    b.f("setViewport", 64, 64)
    b.f("setDepth", shadow)
    b.f("clearDepth", 1.0)
    b.f("useProgramme", shadow_prog)
    b.f("setUniform", 3, S.col_major(light))
    b.f("setUniform", 4, S.col_major(eye))
    b.f("drawVAO", vao)
    b.f("setViewport", w, h)
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF202020)
    if blend:
        b.f("enable", S.ALPHABLEND)
    b.f("useProgramme", planet)
    for slot in (3, 4, 5):
        b.f("setUniform", slot, S.col_major(eye))
    b.f("setUniform", 16, S.col_major(bias @ light))
    b.f("setUniform", 7, S.vec4(0.3, 0.9, 1.6))
    b.f("setUniform", 8, S.vec4(0, 0, 2, 1))
    for slot, tex in ((9, diffuse), (10, bump), (11, spec), (12, night), (15, shadow)):
        b.f("setUniform", slot, np.array([tex], dtype=np.int32))
    b.f("drawVAO", vao)
    return S.Scene(name, w, h, b.setup, b.frame, {"triangles": 520, "depth_texture": depth,
                                                   "shadow_texture": shadow})


def _cloud_scene(name, w, h, seed):
    """The reference demo's cloud processors (test/testproc.cpp): an
    alpha-tested depth-only pass (VP_CloudShadow / FP_CloudShadow: texels
    whose red is below 150 discard) into a 64x64 shadow map, then the
    clouds blended over the frame (VP_Cloud / FP_Cloud: alpha = the texel's
    red, lambert x the projective shadow factor, packed with the SSE
    saturating conversions)."""
    b = S._Builder()
    rng = np.random.default_rng(seed)
    cloud = b.texture(S.checker_noise_bgra(16, 4, rng, noise=90, lo=60, hi=230), wrap=True)
    shadow = b.empty_texture(64, 64)
    depth = b.empty_texture(w, h)
    mesh = _tri_mesh(random_soup(220, seed))
    shadow_prog = b.programme(S.VP_CLOUDSHADOW, S.IP_CLOUDSHADOW, S.FP_CLOUDSHADOW)
    cloud_prog = b.programme(S.VP_CLOUD, S.IP_CLOUD, S.FP_CLOUD)
    vao = b.vao(mesh, slots=(0, 3, 4))
    c, s_ = np.cos(0.5), np.sin(0.5)
    light = np.array([[0.8 * c, 0.1, 0.5 * s_, 0.05], [0.0, 0.8, 0.1, -0.05], [-0.4 * s_, 0.0, 0.4 * c, 0.0],
                      [0.0, 0.0, 0.0, 1.0]])
    bias = np.array([[0.5, 0, 0, 0.5], [0, 0.5, 0, 0.5], [0, 0, 1, 0], [0, 0, 0, 1]])
    eye = np.eye(4)
    b.f("setViewport", 64, 64)
    b.f("setDepth", shadow)
    b.f("clearDepth", 1.0)
    b.f("useProgramme", shadow_prog)
    b.f("setUniform", 3, S.col_major(light))
    b.f("setUniform", 4, S.col_major(eye))
    b.f("setUniform", 9, np.array([cloud], dtype=np.int32))
    b.f("drawVAO", vao)
    b.f("setViewport", w, h)
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF402010)
    b.f("enable", S.ALPHABLEND)
    b.f("useProgramme", cloud_prog)
    for slot in (3, 4, 5):
        b.f("setUniform", slot, S.col_major(eye))
    b.f("setUniform", 16, S.col_major(bias @ light))
    b.f("setUniform", 7, S.vec4(0.3, 0.9, 1.6))
    b.f("setUniform", 8, S.vec4(0, 0, 2, 1))
    b.f("setUniform", 15, np.array([shadow], dtype=np.int32))
    b.f("drawVAO", vao)
    b.f("disable", S.ALPHABLEND)
    return S.Scene(name, w, h, b.setup, b.frame, {"triangles": 440, "depth_texture": depth,
                                                   "shadow_texture": shadow})


def _viewer_scene(name, w, h, seed):
    """The scene viewer demo's processors (test2/testproc.cpp, uniform slots
    test2/testproc.h:4-30): a depth-only pass (VP_Shadow: positions x0.9,
    IP_Null, FP_Null) into a 64x64 shadow map, then an unlit single-colour
    draw, a lit single-colour draw and a textured draw under a spotlight
    whose 25-degree cone covers part of the frame (cos^150 fall-off outside
    it), each with the 4-tap projective shadow lookup."""
    b = S._Builder()
    rng = np.random.default_rng(seed)
    tex = b.texture(S.checker_noise_bgra(32, 8, rng, noise=24, lo=50, hi=210), wrap=True)
    shadow = b.empty_texture(64, 64)
    depth = b.empty_texture(w, h)
    vaos = [b.vao(_tri_mesh(random_soup(n, seed + k)), slots=(0, 3, 4)) for k, n in enumerate((60, 140, 140))]
    shadow_prog = b.programme(S.VP_SHADOW2, S.IP_NULL, S.FP_NULL)
    progs = [b.programme(S.VP_POSITIONONLY, S.IP_NULL, S.FP_SINGLECOLOURNL),
             b.programme(S.VP_SINGLECOLOUR, S.IP_SINGLECOLOUR, S.FP_SINGLECOLOUR),
             b.programme(S.VP_DIFFUSEONLY, S.IP_DIFFUSEONLY, S.FP_DIFFUSEONLY)]
    c, s_ = np.cos(0.4), np.sin(0.4)
    light = np.array([[0.85 * c, 0.0, 0.45 * s_, 0.02], [0.05, 0.85, 0.0, -0.03], [-0.4 * s_, 0.0, 0.4 * c, 0.0],
                      [0.0, 0.0, 0.0, 1.0]])
    bias = np.array([[0.5, 0, 0, 0.5], [0, 0.5, 0, 0.5], [0, 0, 1, 0], [0, 0, 0, 1]])
    eye = np.eye(4)
    lpos = np.array([0.4, 0.3, 2.2])
    ldir = lpos - np.array([0.1, 0.0, 0.0])
    ldir /= np.linalg.norm(ldir)
    b.f("setViewport", 64, 64)
    b.f("setDepth", shadow)
    b.f("clearDepth", 1.0)
    b.f("useProgramme", shadow_prog)
    b.f("setUniform", 5, S.col_major(light))
    for v in vaos:
        b.f("drawVAO", v)
    b.f("setViewport", w, h)
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF203040)
    for slot in (0, 1, 5):
        b.f("setUniform", slot, S.col_major(eye))
    b.f("setUniform", 6, S.col_major(bias @ light))
    b.f("setUniform", 20, S.vec4(*lpos))
    b.f("setUniform", 21, S.vec4(*ldir))
    b.f("setUniform", 22, S.vec4(0, 0, 2))
    b.f("setUniform", 23, np.array([shadow], dtype=np.int32))
    b.f("setUniform", 30, S.vec4(0.25, 0.2, 0.15, 0.0))
    b.f("setUniform", 31, S.vec4(0.8, 0.55, 0.3, 1.0))
    b.f("setUniform", 32, S.vec4(0.9, 0.9, 1.0, 1.0))
    b.f("setUniform", 33, np.array([20.0], dtype=np.float32))
    b.f("setUniform", 40, np.array([tex], dtype=np.int32))
    for prog, v in zip(progs, vaos):
        b.f("useProgramme", prog)
        b.f("drawVAO", v)
    return S.Scene(name, w, h, b.setup, b.frame, {"triangles": 340, "depth_texture": depth,
                                                   "shadow_texture": shadow})


def _v(x, y, z=0.0, w=1.0):
    return [x * w, y * w, z * w, w]


def basic_cases(w=64, h=48):
    """Hand-placed triangles (counter-clockwise = front)."""
    T = []
    T += [_v(-0.9, 0.5, 0.1), _v(-0.5, 0.5, 0.1), _v(-0.7, 0.9, 0.1)]      # flat bottom
    T += [_v(-0.3, 0.9, 0.2), _v(-0.5, 0.5, 0.2), _v(-0.1, 0.9, 0.2)]      # flat top
    T += [_v(0.1, 0.3, 0.3), _v(0.5, 0.5, 0.3), _v(0.2, 0.9, 0.3)]         # right-pointing
    T += [_v(0.9, 0.3, 0.3), _v(0.8, 0.9, 0.3), _v(0.6, 0.6, 0.3)]         # left-pointing
    T += [_v(-1.4, -0.2, 0.0), _v(-0.8, -0.1, 0.0), _v(-1.1, 0.25, 0.0)]    # off the left edge
    T += [_v(0.8, -0.2, 0.0), _v(1.5, -0.1, 0.0), _v(1.1, 0.25, 0.0)]      # off the right edge
    T += [_v(-0.2, 0.85, 0.0), _v(0.2, 0.85, 0.0), _v(0.0, 1.4, 0.0)]      # off the top
    T += [_v(-0.2, -1.5, 0.0), _v(0.2, -0.85, 0.0), _v(-0.3, -0.8, 0.0)]   # off the bottom
    T += [_v(-0.6, -0.6, 0.5), _v(-0.2, -0.6, 0.5), _v(-0.2, -0.2, 0.5)]   # quad, shared diagonal
    T += [_v(-0.6, -0.6, 0.5), _v(-0.2, -0.2, 0.5), _v(-0.6, -0.2, 0.5)]
    T += [_v(0.0, -0.6, 0.4), _v(0.4, -0.6, 0.4), _v(0.2, -0.2, 0.4)]      # equal-depth overlap pair
    T += [_v(0.05, -0.55, 0.4), _v(0.45, -0.55, 0.4), _v(0.25, -0.15, 0.4)]
    T += [_v(0.5, -0.6, 0.40005), _v(0.9, -0.6, 0.40005), _v(0.7, -0.2, 0.40005)]  # within epsilon
    T += [_v(0.5, -0.6, 0.3999), _v(0.9, -0.6, 0.3999), _v(0.7, -0.2, 0.3999)]     # beyond epsilon
    T += [_v(0.1, 0.1, 0.0), _v(0.1, 0.1, 0.0), _v(0.3, 0.2, 0.0)]         # zero area (repeated vertex)
    T += [_v(-0.5, 0.0, 0.0), _v(0.0, 0.0, 0.0), _v(0.5, 0.0, 0.0)]        # collinear, horizontal
    T += [_v(-0.95, -0.95, 0.0), _v(0.95, -0.9, 0.0), _v(-0.95, -0.93, 0.0)]  # needle, tiny dy
    T += [_v(0.6, 0.0, 0.2), _v(0.62, 0.0, 0.2), _v(0.61, 0.8, 0.2)]       # thin vertical sliver
    T += [_v(-0.1, -0.1, 0.2), _v(-0.3, 0.1, 0.2), _v(0.1, 0.1, 0.2)]      # back face (clockwise)
    T += [_v(-0.9, -0.9, 1.2), _v(-0.7, -0.9, 0.0), _v(-0.8, -0.7, 0.0)]   # z-reject: z > 1
    T += [_v(0.3, -0.95, -1.3), _v(0.5, -0.95, 0.0), _v(0.4, -0.7, 0.0)]   # z-reject: z < -1
    T += [_v(-0.3, -0.3, -0.2, 0.5), _v(0.3, -0.3, 0.6, 3.0), _v(0.0, 0.3, 0.2, 1.2)]  # perspective
    pix = [[(2 * px / w - 1), (2 * py / h - 1)] for px, py in ((10, 5), (20, 5), (15, 15))]
    T += [_v(pix[0][0], pix[0][1], -0.5), _v(pix[1][0], pix[1][1], -0.5), _v(pix[2][0], pix[2][1], -0.5)]
    return np.array(T, dtype=np.float32)


def random_soup(n, seed, persp=True):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        c = rng.uniform(-1.1, 1.1, size=2)
        z = rng.uniform(-0.95, 0.95)
        size = rng.uniform(0.02, 0.7)
        for _v_ in range(3):
            w = rng.uniform(0.6, 2.5) if persp else 1.0
            p = c + rng.normal(size=2) * size
            zz = np.clip(z + rng.normal() * 0.05, -0.99, 0.99)
            out.append([p[0] * w, p[1] * w, zz * w, w])
    return np.array(out, dtype=np.float32)


def kat_scenes():
    """(name, scene) pairs used for the golden fixtures and the GPU parity tests."""
    out = []
    base = basic_cases()
    out.append(("kat_basic_lit_64x48", _scene("kat_basic_lit", 64, 48, base)))
    out.append(("kat_basic_depth_64x48", _scene("kat_basic_depth", 64, 48, base, lit=False)))
    out.append(("kat_basic_nocull_61x37", _scene("kat_basic_nocull", 61, 37, base, behavior_off=S.FACE_CULLING)))
    out.append(("kat_basic_notest_64x48", _scene("kat_basic_notest", 64, 48, base, behavior_off=S.TEST_DEPTH)))
    out.append(("kat_soup_lit_96x64", _scene("kat_soup_lit", 96, 64, random_soup(300, 11))))
    out.append(("kat_soup_depth_97x63", _scene("kat_soup_depth", 97, 63, random_soup(400, 12), lit=False)))
    out.append(("kat_soup_ortho_nocull_80x80",
                _scene("kat_soup_ortho", 80, 80, random_soup(300, 13, persp=False), behavior_off=S.FACE_CULLING)))
    # blending (fbo.cpp:208-229) and discard (fragthrd.cpp:233-237): every
    # passing fragment is shaded, in order
    out.append(("kat_blend_lit_96x64", _scene("kat_blend_lit", 96, 64, random_soup(300, 14),
                                              behavior_on=S.ALPHABLEND)))
    out.append(("kat_alphatest_96x64", _scene("kat_alphatest", 96, 64, random_soup(300, 15), fp=S.FP_LIT1A)))
    out.append(("kat_alphatest_blend_nocull_88x72",
                _scene("kat_alphatest_blend", 88, 72, random_soup(300, 16), fp=S.FP_LIT1A,
                       behavior_on=S.ALPHABLEND, behavior_off=S.FACE_CULLING)))
    out.append(("kat_blend_notest_64x48", _scene("kat_blend_notest", 64, 48, random_soup(120, 17),
                                                 behavior_on=S.ALPHABLEND, behavior_off=S.TEST_DEPTH)))
    # the reference's own textured processors (x86 rcpps / rsqrtss inside: the
    # oracle's IEEE restatement matches their depth exactly, colour closely)
    out.append(("kat_def01_soup_96x64", _scene("kat_def01_soup", 96, 64, random_soup(300, 18), fp=S.FP_DEF01)))
    out.append(("kat_def03_soup_96x64", _scene("kat_def03_soup", 96, 64, random_soup(300, 19), fp=S.FP_DEF03)))
    out.append(("kat_def02_soup_96x64", _scene("kat_def02_soup", 96, 64, random_soup(300, 20), fp=S.FP_DEF02)))
    # the skybox's cube-map sampler (samplrcube.cpp): views that put the
    # major axis on each face, face edges and the Y faces' sign rule on Z
    out.append(("kat_def04_sky_soup_96x64", _skybox_scene("kat_def04_sky_soup", 96, 64, _rot(0.7, 0.4), 24, False,
                                                         soup_seed=21)))
    out.append(("kat_def04_sky_up_wrap_80x80", _skybox_scene("kat_def04_sky_up_wrap", 80, 80, _rot(2.1, -1.2, 0.3),
                                                            17, True)))
    out.append(("kat_def04_sky_down_blend_72x56", _skybox_scene("kat_def04_sky_down_blend", 72, 56,
                                                               _rot(-2.6, 1.05, -0.5), 32, False, blend=True)))
    # the post-processing hook between passes
    out.append(("kat_post_add_fog_96x64", _post_scene("kat_post_add_fog", 96, 64, 22)))
    # render to texture through setFBO, then sampling it
    out.append(("kat_setfbo_rtt_96x64", _setfbo_scene("kat_setfbo_rtt", 96, 64, 28)))
    # the reference demo's planet processors with the projective shadow lookup
    out.append(("kat_def0_planet_earth_96x64", _planet_scene("kat_planet_earth", 96, 64, 23, S.FP_EARTH)))
    out.append(("kat_def0_planet_satellite_80x60", _planet_scene("kat_planet_satellite", 80, 60, 24, S.FP_SATELLITE)))
    out.append(("kat_def0_planet_cloud_88x64", _cloud_scene("kat_cloud", 88, 64, 25)))
    out.append(("kat_def0_viewer_spot_96x72", _viewer_scene("kat_viewer_spot", 96, 72, 26)))
    out.append(("kat_def0_viewer_spot_80x64", _viewer_scene("kat_viewer_spot_b", 80, 64, 27)))
    return out
