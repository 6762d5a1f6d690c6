"""Seeded synthetic scenes for the benchmark configurations.

A scene is a recorded sequence of pipeline calls, split into a ``setup`` list
(textures, processors, programmes, vertex arrays: the resident resources) and a
``frame`` list (clears, uniforms, state, draws).  ``replay_setup`` and
``replay_frame`` issue those calls, by the reference's method names
(PuresoftPipeline, src/puresoft3d/pipeline.h:26-69), on any object that has
them: the GPU pipeline (``puresoft3d_gb300.pipeline.PuresoftPipeline``) or a CPU
checker.  All inputs are generated here once, in numpy, so every
implementation receives byte-identical vertex, texture and uniform data.

Conventions (shared by every config):
  * vertices are non-indexed triangle lists; VBO slots follow the reference's
    demos (src/test/scenobj.cpp:135-157): 0 position vec4 (w=1), 1 tangent vec4
    (w = handedness), 3 normal vec4 (w=0), 4 uv vec2;
  * front faces are counter-clockwise on screen (the reference culls a face
    whose projected (v1-v0) x (v2-v1) has negative z, vertthrd.cpp:56-65);
  * matrices are column-major float32 (mcemaths, matrix.cpp:515-557); uniform
    slots 3 = PV, 4 = M, 5 = Mrot, 6 = light PV, 7 = direction to the light,
    8 = camera position, 9 = albedo texture (or chain {first, levels}),
    10 = normal-map chain, 11 = shadow map, 12 = {lodScale, shadowBias, 0, 0};
  * textures are BGRA8 rows stored bottom-up (tex.cpp:17); a mip chain is a
    run of consecutive textures, level k of size max(1, S >> k), built by a
    2x2 box filter with round-half-up integer averaging;
  * the colour target is BGRA8 and the depth target an FP32 texture the scene
    creates and binds with setDepth, so every implementation reads the same
    buffer layout back.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Any, Dict, List, Tuple

import numpy as np

# processor ids (include/ps3d.h)
VP_DEF01, IP_DEF01, FP_DEF01 = 0x0101, 0x0102, 0x0103
VP_DEF02, IP_DEF02, FP_DEF02 = 0x0201, 0x0202, 0x0203
VP_DEF03, IP_DEF03, FP_DEF03 = 0x0301, 0x0302, 0x0303
VP_DEF04, IP_DEF04, FP_DEF04 = 0x0401, 0x0402, 0x0403
VP_DEF05, IP_DEF05, FP_DEF05 = 0x0501, 0x0502, 0x0503
VP_SHADOW = 0x0601
# the reference demo's planet set (src/test/testproc.cpp)
VP_PLANET, IP_PLANET, FP_EARTH, FP_SATELLITE = 0x0701, 0x0702, 0x0703, 0x0713
VP_CLOUD, IP_CLOUD, FP_CLOUD = 0x0801, 0x0802, 0x0803
VP_CLOUDSHADOW, IP_CLOUDSHADOW, FP_CLOUDSHADOW = 0x0901, 0x0902, 0x0903
# the scene viewer demo's sets (test2/testproc.h)
VP_POSITIONONLY, IP_NULL, FP_SINGLECOLOURNL = 0x0A01, 0x0A02, 0x0A03
VP_SINGLECOLOUR, IP_SINGLECOLOUR, FP_SINGLECOLOUR = 0x0B01, 0x0B02, 0x0B03
VP_DIFFUSEONLY, IP_DIFFUSEONLY, FP_DIFFUSEONLY = 0x0C01, 0x0C02, 0x0C03
VP_SHADOW2, FP_NULL = 0x0D01, 0x0D03
FP_LIT1, FP_LIT1A, FP_LIT3 = 0x1103, 0x1403, 0x1303
VP_LIT2, IP_LIT2, FP_LIT2 = 0x1201, 0x1202, 0x1203

UPDATE_DEPTH, TEST_DEPTH, FACE_CULLING, ALPHABLEND = 1, 2, 4, 8
PP_ADD8, PP_FOG = 0x7001, 0x7002  # built-in post-processors


def add8_params(b: int, g: int, r: int, a: int) -> bytes:
    """PP_ADD8's parameter: the per-byte addends of a BGRA pixel."""
    return bytes([b & 255, g & 255, r & 255, a & 255])


def fog_params(bgra: int, near: float, far: float) -> bytes:
    """PP_FOG's parameter: fog colour (BGRA word) and the depth range."""
    import struct
    return struct.pack("<Iff", bgra & 0xFFFFFFFF, near, far)


@dataclasses.dataclass
class Scene:
    name: str
    width: int
    height: int
    setup: List[Tuple[Any, ...]]
    frame: List[Tuple[Any, ...]]
    info: Dict[str, Any]

    def triangles(self) -> int:
        return int(self.info.get("triangles", 0))


# --------------------------------------------------------------------------
# matrices (column-major, float32 results; built in float64)


def _f32(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, dtype=np.float64).astype(np.float32))


def col_major(m4: np.ndarray) -> np.ndarray:
    """4x4 row-major math matrix -> 16 float32 in column-major storage."""
    return _f32(np.asarray(m4).T.reshape(16))


def perspective(znear, zfar, aspect, fov_rad) -> np.ndarray:
    """mcemaths_make_proj_perspective (matrxgl.cpp:9-22), as a math matrix."""
    h = 1.0 / math.tan(fov_rad / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = h / aspect
    m[1, 1] = h
    m[2, 2] = (zfar + znear) / (znear - zfar)
    m[3, 2] = -1.0
    m[2, 3] = 2.0 * (znear * zfar) / (znear - zfar)
    return m


def orthographic(znear, zfar, left, right, bottom, top) -> np.ndarray:
    """mcemaths_make_proj_orthographic (matrxgl.cpp:24-34)."""
    m = np.eye(4)
    m[0, 0] = 2.0 / (right - left)
    m[1, 1] = 2.0 / (top - bottom)
    m[2, 2] = -2.0 / (zfar - znear)
    m[0, 3] = -(right + left) / (right - left)
    m[1, 3] = -(top + bottom) / (top - bottom)
    m[2, 3] = -(zfar + znear) / (zfar - znear)
    return m


def look_at(eye, target, up) -> np.ndarray:
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def translation(x, y, z) -> np.ndarray:
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def rotation_axis(axis, angle) -> np.ndarray:
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    x, y, z = a
    c, s, ic = math.cos(angle), math.sin(angle), 1 - math.cos(angle)
    m = np.eye(4)
    m[:3, :3] = [[c + x * x * ic, x * y * ic - z * s, x * z * ic + y * s],
                 [y * x * ic + z * s, c + y * y * ic, y * z * ic - x * s],
                 [z * x * ic - y * s, z * y * ic + x * s, c + z * z * ic]]
    return m


def quaternion_rotation(q) -> np.ndarray:
    w, x, y, z = np.asarray(q, dtype=np.float64) / np.linalg.norm(q)
    m = np.eye(4)
    m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return m


def scaling(s) -> np.ndarray:
    m = np.eye(4)
    m[0, 0] = m[1, 1] = m[2, 2] = s
    return m


def vec4(x, y, z, w=0.0) -> np.ndarray:
    return np.array([x, y, z, w], dtype=np.float32)


# --------------------------------------------------------------------------
# meshes: dict of float32 arrays, one row per vertex of a triangle list


def _expand(pos, nrm, tan, uv, tris) -> Dict[str, np.ndarray]:
    t = np.asarray(tris, dtype=np.int64).reshape(-1)
    n = len(t)
    out = {
        "position": np.concatenate([pos[t], np.ones((n, 1))], 1),
        "normal": np.concatenate([nrm[t], np.zeros((n, 1))], 1),
        "tangent": np.concatenate([tan[t], np.ones((n, 1))], 1),
        "uv": uv[t],
    }
    return {k: _f32(v) for k, v in out.items()}


def uv_sphere(segments: int, stacks: int, radius: float = 1.0, poles: str = "fan") -> Dict[str, np.ndarray]:
    """UV sphere.  poles="fan": proper pole fans, segments*(2*stacks-2)
    triangles.  poles="grid": a full quad grid (2*segments*stacks triangles)
    with the south-pole row of zero-area triangles dropped, so the north pole
    keeps ``segments`` zero-area triangles (config 1's 992 = 32*31 rule)."""
    i = np.arange(stacks + 1)[:, None]
    j = np.arange(segments + 1)[None, :]
    theta = np.pi * i / stacks            # 0 at the south pole
    phi = 2 * np.pi * j / segments
    x = -np.sin(theta) * np.sin(phi)
    y = -np.cos(theta) * np.ones_like(phi)
    z = -np.sin(theta) * np.cos(phi)
    nrm = np.stack([x, y, z], -1).reshape(-1, 3)
    pos = nrm * radius
    tan = np.stack([-np.cos(phi) * np.ones_like(theta), np.zeros_like(theta * phi),
                    np.sin(phi) * np.ones_like(theta)], -1).reshape(-1, 3)
    uv = np.stack([(j / segments) * np.ones_like(theta), (i / stacks) * np.ones_like(phi)], -1).reshape(-1, 2)
    idx = lambda a, b: a * (segments + 1) + b  # noqa: E731
    tris = []
    for a in range(stacks):
        for b in range(segments):
            v00, v01, v10, v11 = idx(a, b), idx(a, b + 1), idx(a + 1, b), idx(a + 1, b + 1)
            t1, t2 = (v00, v01, v11), (v00, v11, v10)
            # on the south row v00 == v01 (t1 has zero area); on the north
            # row v10 == v11 (t2 has zero area)
            if a == 0:
                tris.append(t2)
            elif a == stacks - 1 and poles == "fan":
                tris.append(t1)
            else:
                tris += [t1, t2]
    return _expand(pos, nrm, tan, uv, tris)


def torus(major_seg: int, minor_seg: int, R: float = 1.0, r: float = 0.35) -> Dict[str, np.ndarray]:
    i = np.arange(major_seg + 1)[:, None]
    j = np.arange(minor_seg + 1)[None, :]
    u = 2 * np.pi * i / major_seg
    v = 2 * np.pi * j / minor_seg
    cx, cz = np.cos(u), np.sin(u)
    nx, ny, nz = np.cos(v) * cx, np.sin(v) * np.ones_like(u), np.cos(v) * cz
    pos = np.stack([R * cx + r * nx, r * ny, R * cz + r * nz], -1).reshape(-1, 3)
    nrm = np.stack([nx, ny, nz], -1).reshape(-1, 3)
    tan = np.stack([-np.sin(u) * np.ones_like(v), np.zeros_like(u * v), np.cos(u) * np.ones_like(v)], -1).reshape(-1, 3)
    uv = np.stack([(i / major_seg) * np.ones_like(v) * 4.0, (j / minor_seg) * np.ones_like(u)], -1).reshape(-1, 2)
    idx = lambda a, b: a * (minor_seg + 1) + b  # noqa: E731
    tris = []
    for a in range(major_seg):
        for b in range(minor_seg):
            v00, v01, v10, v11 = idx(a, b), idx(a, b + 1), idx(a + 1, b), idx(a + 1, b + 1)
            tris += [(v00, v01, v11), (v00, v11, v10)]
    return _expand(pos, nrm, tan, uv, tris)


def box(div: int, half: float = 1.0) -> Dict[str, np.ndarray]:
    faces = [((1, 0, 0), (0, 0, -1), (0, 1, 0)), ((-1, 0, 0), (0, 0, 1), (0, 1, 0)),
             ((0, 1, 0), (1, 0, 0), (0, 0, -1)), ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
             ((0, 0, 1), (1, 0, 0), (0, 1, 0)), ((0, 0, -1), (-1, 0, 0), (0, 1, 0))]
    P, N, T, U, tris = [], [], [], [], []
    base = 0
    g = np.linspace(-1.0, 1.0, div + 1)
    for n, t, b in faces:
        n, t, b = (np.asarray(v, dtype=np.float64) for v in (n, t, b))
        s_, r_ = np.meshgrid(g, g, indexing="ij")  # s along t, r along b
        p = (n[None, None] + s_[..., None] * t + r_[..., None] * b) * half
        P.append(p.reshape(-1, 3))
        N.append(np.broadcast_to(n, p.shape).reshape(-1, 3))
        T.append(np.broadcast_to(t, p.shape).reshape(-1, 3))
        U.append(np.stack([(s_ + 1) / 2, (r_ + 1) / 2], -1).reshape(-1, 2))
        for a in range(div):
            for c in range(div):
                v00 = base + a * (div + 1) + c
                v10, v01, v11 = v00 + (div + 1), v00 + 1, v00 + (div + 1) + 1
                tris += [(v00, v10, v11), (v00, v11, v01)]
        base += (div + 1) * (div + 1)
    return _expand(np.concatenate(P), np.concatenate(N), np.concatenate(T), np.concatenate(U), tris)


def mesh_triangles(mesh) -> int:
    return len(mesh["position"]) // 3


# --------------------------------------------------------------------------
# textures


def checker_noise_bgra(size: int, squares: int, rng: np.random.Generator, noise: int = 16,
                       lo: int = 64, hi: int = 192) -> np.ndarray:
    """size x size BGRA8: squares x squares checker of lo/hi grey plus uniform
    integer noise in [-noise, noise] per colour channel, clamped; alpha 255."""
    cell = size // squares
    yy, xx = np.mgrid[0:size, 0:size]
    grey = np.where(((yy // cell) + (xx // cell)) % 2 == 0, lo, hi).astype(np.int32)
    img = np.empty((size, size, 4), dtype=np.int32)
    img[..., :3] = grey[..., None] + rng.integers(-noise, noise + 1, size=(size, size, 3))
    img[..., 3] = 255
    return np.clip(img, 0, 255).astype(np.uint8)


def procedural_bgra(size: int, rng: np.random.Generator) -> np.ndarray:
    """A seeded procedural albedo: coloured checker + stripes + noise."""
    cells = int(rng.integers(4, 17))
    base = rng.integers(40, 216, size=(2, 3))
    yy, xx = np.mgrid[0:size, 0:size]
    chk = ((yy * cells // size) + (xx * cells // size)) % 2
    img = np.empty((size, size, 4), dtype=np.int32)
    stripes = ((xx + yy) * 16 // size) % 2 * 24
    img[..., :3] = base[chk] + stripes[..., None] + rng.integers(-12, 13, size=(size, size, 3))
    img[..., 3] = 255
    return np.clip(img, 0, 255).astype(np.uint8)


def mip_chain_u8(level0: np.ndarray) -> List[np.ndarray]:
    """2x2 box filter with (a+b+c+d+2)>>2 per channel; level k is
    max(1, S >> k) on a side."""
    chain = [level0]
    cur = level0.astype(np.int32)
    while cur.shape[0] > 1 or cur.shape[1] > 1:
        h, w = cur.shape[:2]
        if h > 1:
            cur = cur[0::2] + cur[1::2]
        else:
            cur = cur * 2
        if w > 1:
            cur = cur[:, 0::2] + cur[:, 1::2]
        else:
            cur = cur * 2
        cur = (cur + 2) >> 2
        chain.append(cur.astype(np.uint8))
    return chain


def perlin2d(size: int, cells: int, rng: np.random.Generator) -> np.ndarray:
    """Classic gradient noise on a size x size grid with `cells` lattice cells."""
    ang = rng.uniform(0, 2 * np.pi, size=(cells + 1, cells + 1))
    gx, gy = np.cos(ang), np.sin(ang)
    t = (np.arange(size) + 0.5) * cells / size
    i0 = np.floor(t).astype(int)
    f = t - i0
    fade = f * f * f * (f * (f * 6 - 15) + 10)
    X0, Y0 = np.meshgrid(i0, i0, indexing="xy")
    FX, FY = np.meshgrid(f, f, indexing="xy")
    UX, UY = np.meshgrid(fade, fade, indexing="xy")

    def dot(ix, iy, dx, dy):
        return gx[iy, ix] * dx + gy[iy, ix] * dy

    n00 = dot(X0, Y0, FX, FY)
    n10 = dot(X0 + 1, Y0, FX - 1, FY)
    n01 = dot(X0, Y0 + 1, FX, FY - 1)
    n11 = dot(X0 + 1, Y0 + 1, FX - 1, FY - 1)
    nx0 = n00 + (n10 - n00) * UX
    nx1 = n01 + (n11 - n01) * UX
    return nx0 + (nx1 - nx0) * UY


def normal_map_rgba16f(size: int, rng: np.random.Generator, strength: float = 6.0) -> List[np.ndarray]:
    """Tangent-space normal map from seeded Perlin height (two octaves), as an
    RGBA16F mip chain (xyz = normal, w = 1; lower levels box-filtered in
    float32, not renormalised)."""
    h = perlin2d(size, 16, rng) + 0.5 * perlin2d(size, 32, rng)
    dx = (np.roll(h, -1, 1) - np.roll(h, 1, 1)) * 0.5 * strength
    dy = (np.roll(h, -1, 0) - np.roll(h, 1, 0)) * 0.5 * strength
    n = np.stack([-dx, -dy, np.ones_like(h)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    lvl = np.concatenate([n, np.ones_like(h)[..., None]], -1).astype(np.float32)
    chain = [lvl.astype(np.float16)]
    cur = lvl
    while cur.shape[0] > 1:
        cur = (cur[0::2, 0::2] + cur[1::2, 0::2] + cur[0::2, 1::2] + cur[1::2, 1::2]) * np.float32(0.25)
        chain.append(cur.astype(np.float16))
    return chain


# --------------------------------------------------------------------------
# scene builder


class _Builder:
    def __init__(self):
        self.setup: List[Tuple[Any, ...]] = []
        self.frame: List[Tuple[Any, ...]] = []
        self.ntex = 0
        self.nproc = 0
        self.nprog = 0
        self.nvao = 0

    def texture(self, pixels: np.ndarray, elem_len: int = 4, wrap: bool = True) -> int:
        pixels = np.ascontiguousarray(pixels)
        h = pixels.shape[0]
        row_bytes = pixels.nbytes // h
        width = row_bytes // elem_len
        self.setup.append(("createTexture", width, h, row_bytes, elem_len, pixels, int(wrap)))
        self.ntex += 1
        return self.ntex - 1

    def layered_texture(self, layers: List[np.ndarray], wrap: bool = False) -> int:
        """A texture with extra layers (six BGRA faces in +x, -x, +y, -y, +z,
        -z order make a cube map): the first image is the texture itself,
        the others its extra layers."""
        layers = [np.ascontiguousarray(a) for a in layers]
        h = layers[0].shape[0]
        row_bytes = layers[0].nbytes // h
        self.setup.append(("createTextureLayers", row_bytes // 4, h, row_bytes, 4, layers, int(wrap)))
        self.ntex += 1
        return self.ntex - 1

    def empty_texture(self, width: int, height: int, elem_len: int = 4, wrap: bool = False) -> int:
        """A zeroed texture; for depth targets the scanline is rounded up to
        whole 16-byte vectors as the reference's default depth buffer does
        (pipeline.cpp:31) -- its clear16 requires it (fbo.cpp:348-371)."""
        scan = (width * elem_len + 15) // 16 * 16
        self.setup.append(("createTexture", width, height, scan, elem_len, None, int(wrap)))
        self.ntex += 1
        return self.ntex - 1

    def chain_u8(self, level0: np.ndarray) -> Tuple[int, int]:
        chain = mip_chain_u8(level0)
        first = self.ntex
        for lvl in chain:
            self.texture(lvl)
        return first, len(chain)

    def chain_f16(self, chain: List[np.ndarray]) -> Tuple[int, int]:
        first = self.ntex
        for lvl in chain:
            # an RGBA16F level rides in a 4-byte-element texture twice as wide
            self.texture(lvl.view(np.uint8).reshape(lvl.shape[0], -1))
        return first, len(chain)

    def programme(self, vp: int, ip: int, fp: int) -> int:
        self.setup.append(("programme", vp, ip, fp))
        self.nproc += 3
        self.nprog += 1
        return self.nprog - 1

    def vao(self, mesh: Dict[str, np.ndarray], slots=(0, 1, 3, 4)) -> int:
        """VBO slots from mesh arrays: `slots` lists slots of the default
        layout (0 position, 1 tangent, 2 binormal, 3 normal, 4 uv) or maps
        slot -> array name."""
        names = {0: "position", 1: "tangent", 2: "binormal", 3: "normal", 4: "uv"}
        if not isinstance(slots, dict):
            slots = {s: names[s] for s in slots}
        vbos = {s: np.ascontiguousarray(mesh[n]) for s, n in slots.items()}
        self.setup.append(("vao", vbos))
        self.nvao += 1
        return self.nvao - 1

    def f(self, *op):
        self.frame.append(op)


def _u(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v))


def scene_c1(seed: int = 1235, width: int = 640, height: int = 480) -> Scene:
    """Config 1: one 32x16 UV sphere (992 triangles, the full quad grid less
    the south pole's zero-area row) at the origin; 60 deg FOV camera at
    distance 3 (near 0.1, far 100); one 256^2 texture (8x8 checker of 64/192
    grey + uniform noise in [-16, 16]); LIT1 shader (directional Lambert +
    Blinn-Phong s=32, bilinear REPEAT); default behaviour (depth test + write,
    back-face culling)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    tex = b.texture(checker_noise_bgra(256, 8, rng))
    depth = b.empty_texture(width, height)
    prog = b.programme(VP_DEF01, IP_DEF01, FP_LIT1)
    mesh = uv_sphere(32, 16, 1.0, poles="grid")
    assert mesh_triangles(mesh) == 992
    vao = b.vao(mesh, slots=(0, 3, 4))
    P = perspective(0.1, 100.0, width / height, math.radians(60.0))
    V = translation(0, 0, -3.0)
    M = rotation_axis((0.3, 1.0, 0.1), 0.7) @ rotation_axis((1, 0, 0), 0.35)
    light = np.array([0.5, 0.7, 0.5])
    light /= np.linalg.norm(light)
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF202020)
    b.f("useProgramme", prog)
    b.f("setUniform", 3, col_major(P @ V))
    b.f("setUniform", 4, col_major(M))
    b.f("setUniform", 5, col_major(M))
    b.f("setUniform", 7, vec4(*light))
    b.f("setUniform", 8, vec4(0, 0, 3.0, 1.0))
    b.f("setUniform", 9, _u(np.array([tex], dtype=np.int32)))
    b.f("drawVAO", vao)
    return Scene("c1", width, height, b.setup, b.frame,
                 {"triangles": 992, "depth_texture": depth, "draws": 1})


def _random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    return quaternion_rotation(q)


def scene_c2(seed: int = 1236, width: int = 1920, height: int = 1080, shadow_size: int = 2048,
             meshes: int = 64, tex_size: int = 1024, spread: float = 20.0) -> Scene:
    """Config 2: 64 seeded meshes (sphere / torus / box, uniform type, scale
    U[0.2, 2], rotation uniform on SO(3), position U[-20, 20]^3), ~200k
    triangles; four tex_size^2 BGRA8 albedo mip chains and one RGBA16F
    tangent-space normal-map chain (seeded Perlin), trilinear; a
    shadow_size^2 FP32 shadow pass (VP_SHADOW: DEF05 without its x0.9 scale)
    then a width x height LIT2 pass (Blinn-Phong s=32 with 3x3 PCF)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    albedo = [b.chain_u8(procedural_bgra(tex_size, rng)) for _ in range(4)]
    normal = b.chain_f16(normal_map_rgba16f(tex_size, rng))
    shadow = b.empty_texture(shadow_size, shadow_size)
    depth = b.empty_texture(width, height)
    prog_shadow = b.programme(VP_SHADOW, IP_DEF05, FP_DEF05)
    prog_lit = b.programme(VP_LIT2, IP_LIT2, FP_LIT2)
    kinds = rng.integers(0, 3, size=meshes)
    tri_total = 0
    objs = []
    for k in range(meshes):
        kind = int(kinds[k])
        mesh = uv_sphere(40, 40) if kind == 0 else torus(40, 40) if kind == 1 else box(16)
        scale = float(rng.uniform(0.2, 2.0))
        R = _random_rotation(rng)
        pos = rng.uniform(-spread, spread, size=3)
        M = translation(*pos) @ R @ scaling(scale)
        vao = b.vao(mesh)
        tri_total += mesh_triangles(mesh)
        objs.append((vao, M, R, albedo[int(rng.integers(0, 4))], scale, kind))
    eye = np.array([0.0, 10.0, 55.0]) * (spread / 20.0)
    P = perspective(1.0 * spread / 20.0, 200.0 * spread / 20.0, width / height, math.radians(60.0))
    V = look_at(eye, (0, 0, 0), (0, 1, 0))
    light = np.array([0.4, 0.8, 0.45])
    light /= np.linalg.norm(light)
    k = spread / 20.0
    LV = look_at(light * 70.0 * k, (0, 0, 0), (0, 1, 0))
    LP = orthographic(1.0 * k, 140.0 * k, -38.0 * k, 38.0 * k, -38.0 * k, 38.0 * k)
    LPV = col_major(LP @ LV)
    focal = (height / 2) / math.tan(math.radians(30.0))
    # shadow pass
    b.f("setDepth", shadow)
    b.f("clearDepth", 1.0)
    b.f("setViewport", shadow_size, shadow_size)
    b.f("useProgramme", prog_shadow)
    b.f("setUniform", 3, LPV)
    for vao, M, R, alb, scale, kind in objs:
        b.f("setUniform", 4, col_major(M))
        b.f("drawVAO", vao)
    # lit pass
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF303840)
    b.f("setViewport", width, height)
    b.f("useProgramme", prog_lit)
    b.f("setUniform", 3, col_major(P @ V))
    b.f("setUniform", 6, LPV)
    b.f("setUniform", 7, vec4(*light))
    b.f("setUniform", 8, vec4(*eye, 1.0))
    b.f("setUniform", 10, _u(np.array(normal, dtype=np.int32)))
    b.f("setUniform", 11, _u(np.array([shadow], dtype=np.int32)))
    for vao, M, R, alb, scale, kind in objs:
        # texels per world unit along the surface, over the focal length in px
        extent = {0: 2 * math.pi, 1: 2 * math.pi * 1.35 / 4.0, 2: 2.0}[kind] * scale
        lod_scale = tex_size / extent / focal
        b.f("setUniform", 4, col_major(M))
        b.f("setUniform", 5, col_major(R))
        b.f("setUniform", 9, _u(np.array(alb, dtype=np.int32)))
        b.f("setUniform", 12, vec4(lod_scale, 0.004, 0.0, 0.0))
        b.f("drawVAO", vao)
    return Scene("c2", width, height, b.setup, b.frame,
                 {"triangles": tri_total, "depth_texture": depth, "shadow_texture": shadow,
                  "draws": 2 * meshes, "shadow_size": shadow_size})


def scene_c3(seed: int = 1237, width: int = 3840, height: int = 2160, meshes: int = 256,
             tri_target: int = 2_000_000, tex_size: int = 2048, textures: int = 16) -> Scene:
    """Config 3: fill/texture stress.  `meshes` seeded spheres and tori
    totalling ~tri_target triangles, arranged in four overlapping layers along
    the view axis (depth complexity ~4); `textures` tex_size^2 BGRA8 mip
    chains sampled trilinear (LIT3)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    chains = [b.chain_u8(procedural_bgra(tex_size, rng)) for _ in range(textures)]
    depth = b.empty_texture(width, height)
    prog = b.programme(VP_DEF01, IP_DEF01, FP_LIT3)
    per = max(8, tri_target // meshes)
    seg = max(4, int(round(math.sqrt(per / 2))))
    eye = np.array([0.0, 0.0, 30.0])
    fov = math.radians(60.0)
    aspect = width / height
    tri_total = 0
    objs = []
    for k in range(meshes):
        layer = k % 4
        zc = -6.0 * layer
        dist = 30.0 - zc
        half_h = math.tan(fov / 2) * dist
        half_w = half_h * aspect
        x = rng.uniform(-half_w * 0.85, half_w * 0.85)
        y = rng.uniform(-half_h * 0.85, half_h * 0.85)
        scale = float(rng.uniform(0.5, 1.0)) * half_h * 0.32
        mesh = uv_sphere(seg, seg) if k % 2 == 0 else torus(seg, seg)
        R = _random_rotation(rng)
        M = translation(x, y, zc) @ R @ scaling(scale)
        vao = b.vao(mesh, slots=(0, 3, 4))
        tri_total += mesh_triangles(mesh)
        objs.append((vao, M, R, chains[int(rng.integers(0, textures))], scale))
    P = perspective(1.0, 200.0, aspect, fov)
    V = look_at(eye, (0, 0, 0), (0, 1, 0))
    light = np.array([-0.3, 0.6, 0.75])
    light /= np.linalg.norm(light)
    focal = (height / 2) / math.tan(fov / 2)
    b.f("setDepth", depth)
    b.f("clearDepth", 1.0)
    b.f("clearColour", 0xFF101418)
    b.f("useProgramme", prog)
    b.f("setUniform", 3, col_major(P @ V))
    b.f("setUniform", 7, vec4(*light))
    b.f("setUniform", 8, vec4(*eye, 1.0))
    for vao, M, R, chain, scale in objs:
        b.f("setUniform", 4, col_major(M))
        b.f("setUniform", 5, col_major(R))
        b.f("setUniform", 9, _u(np.array(chain, dtype=np.int32)))
        b.f("setUniform", 12, vec4(tex_size / (2 * math.pi * scale) / focal, 0.0, 0.0, 0.0))
        b.f("drawVAO", vao)
    return Scene("c3", width, height, b.setup, b.frame,
                 {"triangles": tri_total, "depth_texture": depth, "draws": meshes})


def mesh_with_triangles(n: int, kind: int) -> Dict[str, np.ndarray]:
    """A sphere / torus / box tessellated to roughly n triangles."""
    if kind == 0:
        s_ = max(3, int(round(math.sqrt(n / 4.0))))
        return uv_sphere(2 * s_, s_)
    if kind == 1:
        b_ = max(3, int(round(math.sqrt(n / 4.0))))
        return torus(2 * b_, b_)
    return box(max(1, int(round(math.sqrt(n / 12.0)))))


def scene_c4(seed: int = 1238, views: int = 4096, size: int = 128, tex_size: int = 256,
             tri_min: int = 100, tri_max: int = 5000):
    """Config 4: `views` independent size x size views, each with its own
    seeded mesh (sphere / torus / box, triangles log-uniform in
    [tri_min, tri_max]), its own orbit camera (azimuth U[0, 2pi), elevation
    U[-60, 60] deg, distance U[2.5, 4]) and its own tex_size^2 texture; LIT1.

    Returns (batched, plain): `batched` renders every view in one pass into
    tiles of a square atlas (ps3d_set_viewport_rect), `plain` is the same
    setup with one frame per view (info["view_frames"]) for a size x size
    pipeline.  View v's tile origin is info["origins"][v]."""
    rng = np.random.default_rng(seed)
    cols = int(math.ceil(math.sqrt(views)))
    rows_ = int(math.ceil(views / cols))
    b = _Builder()
    prog = b.programme(VP_DEF01, IP_DEF01, FP_LIT1)
    light = np.array([0.3, 0.8, 0.5])
    light /= np.linalg.norm(light)
    P = perspective(0.5, 20.0, 1.0, math.radians(50.0))
    yy, xx = np.mgrid[0:tex_size, 0:tex_size]
    per_view = []
    tri_total = 0
    for v in range(views):
        n = int(round(math.exp(rng.uniform(math.log(tri_min), math.log(tri_max)))))
        kind = int(rng.integers(0, 3))
        mesh = mesh_with_triangles(n, kind)
        tri_total += mesh_triangles(mesh)
        cells = int(rng.integers(2, 9))
        base = rng.integers(30, 226, size=(2, 3))
        chk = ((yy * cells // tex_size) + (xx * cells // tex_size)) % 2
        img = np.empty((tex_size, tex_size, 4), dtype=np.uint8)
        img[..., :3] = base[chk]
        img[..., 3] = 255
        tex = b.texture(img)
        vao = b.vao(mesh, slots=(0, 3, 4))
        az = rng.uniform(0, 2 * math.pi)
        el = math.radians(rng.uniform(-60, 60))
        dist = rng.uniform(2.5, 4.0)
        eye = dist * np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
        V = look_at(eye, (0, 0, 0), (0, 1, 0))
        R = _random_rotation(rng)
        per_view.append((vao, tex, col_major(P @ V), col_major(R), eye))
    origins = [((v % cols) * size, (v // cols) * size) for v in range(views)]
    common = [("useProgramme", prog), ("setUniform", 7, vec4(*light))]

    def view_ops(v):
        vao, tex, PV, R, eye = per_view[v]
        return [("setUniform", 3, PV), ("setUniform", 4, R), ("setUniform", 5, R),
                ("setUniform", 8, vec4(*eye, 1.0)), ("setUniform", 9, _u(np.array([tex], dtype=np.int32))),
                ("drawVAO", vao)]

    frame = [("clearDepth", 1.0), ("clearColour", 0xFF000000)] + common
    for v in range(views):
        frame.append(("setViewportRect", origins[v][0], origins[v][1], size, size))
        frame += view_ops(v)
    batched = Scene("c4", cols * size, rows_ * size, b.setup, frame,
                    {"triangles": tri_total, "views": views, "view_size": size, "origins": origins,
                     "depth_texture": None})
    view_frames = [[("clearDepth", 1.0), ("clearColour", 0xFF000000)] + common + view_ops(v) for v in range(views)]
    plain = Scene("c4_plain", size, size, b.setup, [], {"triangles": tri_total, "views": views,
                                                        "view_size": size, "view_frames": view_frames})
    return batched, plain


C5_RESOLUTIONS = ((256, 256), (512, 512), (1024, 1024), (1920, 1080))


def scene_c5_pool(seed: int = 1239, meshes: int = 128, tri_min: int = 1000, tri_max: int = 500_000,
                  textures: int = 64, tex_size: int = 512) -> Scene:
    """Config 5's device-resident pool: `meshes` seeded meshes (sphere / torus
    / box, triangles log-uniform in [tri_min, tri_max]) and `textures`
    tex_size^2 procedural mip chains, plus the LIT3 programme (trilinear).
    Setup only; jobs come from `c5_jobs`."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    chains = [b.chain_u8(procedural_bgra(tex_size, rng)) for _ in range(textures)]
    prog = b.programme(VP_DEF01, IP_DEF01, FP_LIT3)
    vaos, tris = [], []
    for _ in range(meshes):
        n = int(round(math.exp(rng.uniform(math.log(tri_min), math.log(tri_max)))))
        mesh = mesh_with_triangles(n, int(rng.integers(0, 3)))
        vaos.append(b.vao(mesh, slots=(0, 3, 4)))
        tris.append(mesh_triangles(mesh))
    light = np.array([0.35, 0.75, 0.55])
    light /= np.linalg.norm(light)
    return Scene("c5_pool", 0, 0, b.setup, [], {
        "programme": prog, "vaos": vaos, "mesh_triangles": tris, "chains": chains, "tex_size": tex_size,
        "common": [("useProgramme", prog), ("setUniform", 7, vec4(*light))]})


@dataclasses.dataclass
class Job:
    """One render request: a mesh of the pool seen by an orbit camera at one
    resolution.  `ops` are the calls that draw it into the current viewport
    (no clears, no viewport)."""
    id: int
    arrival: float          # seconds after the stream starts
    width: int
    height: int
    mesh: int
    triangles: int
    ops: List[Tuple[Any, ...]]


def c5_jobs(pool: Scene, n: int = 2000, rate: float = 1000.0, seed: int = 1240) -> List[Job]:
    """A seeded Poisson stream of n jobs at `rate` jobs/s: resolution uniform
    over C5_RESOLUTIONS, mesh and texture uniform over the pool, camera on a
    random orbit (azimuth U[0, 2pi), elevation U[-60, 60] deg, distance
    U[2.5, 4]), object under a random rotation."""
    rng = np.random.default_rng(seed)
    info = pool.info
    t = 0.0
    jobs = []
    for k in range(n):
        t += float(rng.exponential(1.0 / rate))
        w, h = C5_RESOLUTIONS[int(rng.integers(0, len(C5_RESOLUTIONS)))]
        m = int(rng.integers(0, len(info["vaos"])))
        chain = info["chains"][int(rng.integers(0, len(info["chains"])))]
        az = rng.uniform(0, 2 * math.pi)
        el = math.radians(rng.uniform(-60, 60))
        dist = rng.uniform(2.5, 4.0)
        eye = dist * np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
        P = perspective(0.5, 20.0, w / h, math.radians(50.0))
        V = look_at(eye, (0, 0, 0), (0, 1, 0))
        R = _random_rotation(rng)
        focal = (h / 2) / math.tan(math.radians(25.0))
        lod = info["tex_size"] / (2 * math.pi) / focal * dist
        ops = [("setUniform", 3, col_major(P @ V)), ("setUniform", 4, col_major(R)), ("setUniform", 5, col_major(R)),
               ("setUniform", 8, vec4(*eye, 1.0)), ("setUniform", 9, _u(np.array(chain, dtype=np.int32))),
               ("setUniform", 12, vec4(lod, 0.0, 0.0, 0.0)), ("drawVAO", info["vaos"][m])]
        jobs.append(Job(k, t, w, h, m, info["mesh_triangles"][m], ops))
    return jobs


# --------------------------------------------------------------------------
# replay


def replay_setup(scene: Scene, pipe) -> Dict[str, List[int]]:
    """Create the scene's resources on `pipe`; returns the indices handed
    out, which every implementation assigns in creation order."""
    got: Dict[str, List[int]] = {"texture": [], "programme": [], "vao": []}
    for op in scene.setup:
        kind = op[0]
        if kind == "createTexture":
            _, w, h, scan, elem, pixels, wrap = op
            got["texture"].append(pipe.createTexture(w, h, scan, elem, pixels, wrap))
        elif kind == "createTextureLayers":
            _, w, h, scan, elem, layers, wrap = op
            idx = pipe.createTexture(w, h, scan, elem, layers[0], wrap, extra_layers=len(layers) - 1)
            for k in range(1, len(layers)):
                pipe.writeTextureLayer(idx, k, layers[k])
            got["texture"].append(idx)
        elif kind == "programme":
            _, vp, ip, fp = op
            got["programme"].append(pipe.createProgramme(pipe.addProcessor(vp), pipe.addProcessor(ip),
                                                         pipe.addProcessor(fp)))
        elif kind == "vao":
            vao = pipe.createVAO()
            for slot, arr in op[1].items():
                pipe.attachVBO(vao, slot, arr)
            got["vao"].append(vao)
        else:
            raise ValueError(kind)
    return got


def replay_frame(scene: Scene, pipe) -> None:
    for op in scene.frame:
        getattr(pipe, op[0])(*op[1:])


def replay_ops(ops, pipe) -> None:
    for op in ops:
        getattr(pipe, op[0])(*op[1:])


SCENES = {"c1": scene_c1, "c2": scene_c2, "c3": scene_c3}
