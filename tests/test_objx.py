"""OBJX mesh files (the reference's objcvt/objxio.cpp): the byte layout
against an independent parse, write/read round trips, tangent derivation,
the reference's own sphere.objx where the reference tree is present, and
(on the GPU) the demo's vertex arrays rendered with the bump-mapped
processors against the oracle."""
import os
import struct

import numpy as np
import pytest

from puresoft3d_gb300 import objx
from puresoft3d_gb300 import scenes as S

REF_SPHERE = os.path.join(os.environ.get("PS3D_REFERENCE", "/root/reference"), "src", "test", "sphere.objx")


def parse(path):
    """Independent reader of the packed layout (objxio.cpp:9-45)."""
    d = open(path, "rb").read()
    version, nmesh, mhs, _ = struct.unpack_from("<4I", d, 0)
    off = 16 + 16 + 16 + 32 * 4
    meshes = []
    for _ in range(nmesh):
        name = d[off:off + 260].split(b"\0")[0].decode()
        nv, ni = struct.unpack_from("<2I", d, off + 260)
        has_tc, has_n, has_t = d[off + 268], d[off + 269], d[off + 270]
        nxt = struct.unpack_from("<I", d, off + 1623)[0]
        p = off + mhs
        start = p
        m = {"name": name, "vertices": np.frombuffer(d, np.float32, 4 * nv, p).reshape(nv, 4)}
        p += 16 * nv
        if has_n:
            m["normals"] = np.frombuffer(d, np.float32, 4 * nv, p).reshape(nv, 4)
            p += 16 * nv
        if has_t:
            m["tangents"] = np.frombuffer(d, np.float32, 4 * nv, p).reshape(nv, 4)
            p += 16 * nv
        if has_tc:
            m["texcoords"] = np.frombuffer(d, np.float32, 2 * nv, p).reshape(nv, 2)
            p += 8 * nv
        if ni:
            m["indices"] = np.frombuffer(d, np.int32, ni, p)
            p += 4 * ni
        assert p - start == nxt
        meshes.append(m)
        off = start + nxt
    return version, mhs, meshes


def uv_sphere(stacks=6, slices=8, radius=1.0):
    """Non-indexed triangles of a UV sphere with normals and uv."""
    pos, nrm, uv = [], [], []
    for i in range(stacks):
        for j in range(slices):
            quad = []
            for di, dj in ((0, 0), (1, 0), (1, 1), (0, 1)):
                th, ph = np.pi * (i + di) / stacks, 2 * np.pi * (j + dj) / slices
                n = [np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph), 0.0]
                quad.append((n, [(j + dj) / slices, (i + di) / stacks]))
            for k in (0, 1, 2, 0, 2, 3):
                n, t = quad[k]
                pos.append([radius * n[0], radius * n[1], radius * n[2], 0.0])
                nrm.append(n)
                uv.append(t)
    return (np.array(pos, np.float32), np.array(nrm, np.float32), np.array(uv, np.float32))


def norm4(v):
    v = v.astype(np.float32)
    s = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + (v[:, 2] * v[:, 2] + v[:, 3] * v[:, 3])
    with np.errstate(all="ignore"):  # degenerate triangles at the poles give inf / nan, as in C
        r = np.float32(1.0) / np.sqrt(s)
        return v * r[:, None]


def tangents_nonindexed(p, t):
    """The documented tangent of each triangle (ps3d_objx_read_mesh), float32."""
    out = np.empty_like(p)
    for i in range(0, len(p), 3):
        a, b, c, ta, tb, tc = p[i], p[i + 1], p[i + 2], t[i], t[i + 1], t[i + 2]
        du1, dv1, du2, dv2 = tc[0] - ta[0], tc[1] - ta[1], tb[0] - ta[0], tb[1] - ta[1]
        v1, v2 = (c - a) * dv2, (b - a) * dv1
        with np.errstate(all="ignore"):
            f = np.float32(1.0) / (du1 * dv2 - dv1 * du2)
            out[i:i + 3] = norm4(((v1 - v2) * f)[None])[0]
    return out


def test_layout_and_round_trip(tmp_path):
    pos, nrm, uv = uv_sphere()
    idx = np.arange(len(pos), dtype=np.int32)[::-1].copy()
    tan = np.tile(np.array([1, 0, 0, 0], np.float32), (len(pos), 1))
    meshes = [{"name": "ball", "vertices": pos, "normals": nrm, "texcoords": uv, "tangents": tan,
               "diffuse": np.array([0.2, 0.4, 0.6, 1.0], np.float32), "diffuse_file": "ball.png", "programme": "p"},
              {"name": "bare", "vertices": pos[:6]},
              {"name": "indexed", "vertices": pos, "normals": nrm, "indices": idx}]
    path = str(tmp_path / "m.objx")
    scene = {"camera_pos": [1, 2, 3, 1], "light_dir": np.array([[0, -1, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0],
                                                                   [0, 0, 0, 0]], np.float32)}
    objx.write_objx(path, scene, meshes)
    version, mhs, parsed = parse(path)
    assert version == 0x010003 and mhs == 1627 and [m["name"] for m in parsed] == ["ball", "bare", "indexed"]
    scn, got = objx.read_objx(path)
    assert list(scn["camera_pos"]) == [1, 2, 3, 1] and scn["light_types"] == [1, 0, 0, 0]
    for m, g, q in zip(meshes, got, parsed):
        for k in ("vertices", "normals", "tangents", "texcoords", "indices"):
            assert (k in m) == (k in g) == (k in q), k
            if k in m:
                assert np.array_equal(m[k], g[k]) and np.array_equal(m[k], q[k]), k
    assert np.allclose(got[0]["diffuse"], [0.2, 0.4, 0.6, 1.0]) and got[0]["diffuse_file"] == "ball.png"


def test_derived_tangents(tmp_path):
    pos, nrm, uv = uv_sphere()
    path = str(tmp_path / "t.objx")
    objx.write_objx(path, {}, [{"name": "s", "vertices": pos, "normals": nrm, "texcoords": uv}])
    _, (m,) = objx.read_objx(path, tangents=True)
    want = tangents_nonindexed(pos, uv)
    ok = np.isfinite(want).all(1)
    assert ok.sum() > len(pos) // 2
    assert np.array_equal(m["tangents"][ok].view(np.uint32), want[ok].view(np.uint32))


def test_truncated_and_foreign_files(tmp_path):
    bad = tmp_path / "bad.objx"
    bad.write_bytes(b"\x00" * 40)
    with pytest.raises(ValueError):
        objx.read_objx(str(bad))
    pos, nrm, uv = uv_sphere()
    path = str(tmp_path / "cut.objx")
    objx.write_objx(path, {}, [{"name": "s", "vertices": pos, "normals": nrm}])
    data = open(path, "rb").read()
    open(path, "wb").write(data[:-100])
    with pytest.raises(ValueError):
        objx.read_objx(path)


@pytest.mark.skipif(not os.path.exists(REF_SPHERE), reason="the reference tree is not on this host")
def test_reference_sphere():
    """The reference's own demo mesh (test/sphere.objx): 528 triangles with
    normals, tangents and texture coordinates."""
    _, _, parsed = parse(REF_SPHERE)
    scn, (m,) = objx.read_objx(REF_SPHERE)
    assert m["name"] == "sphere" and m["num_vertices"] == 1584 and m["num_indices"] == 0
    for k in ("vertices", "normals", "tangents", "texcoords"):
        assert np.array_equal(m[k], parsed[0][k]), k


@pytest.mark.gpu
def test_objx_vao_renders_like_the_oracle(tmp_path, gpu_lib):
    """A mesh written as OBJX, loaded as the reference demo loads it
    (positions w = 1, derived tangents, binormal = normalise(cross(n, t))),
    drawn with the bump-mapped processors: the same image as the oracle's
    from the same arrays."""
    from common import assert_depth_exact, colour_diff
    from cpu_backends import OraclePipeline
    from kat_scenes import _bump_texture
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    pos, nrm, uv = uv_sphere(10, 14, 0.8)
    path = str(tmp_path / "sphere.objx")
    objx.write_objx(path, {}, [{"name": "sphere", "vertices": pos, "normals": nrm, "texcoords": uv}])
    p4 = pos.copy()
    p4[:, 3] = 1.0
    tan = tangents_nonindexed(pos, uv)
    n, t = nrm, tan
    cross = np.stack([n[:, 1] * t[:, 2] - n[:, 2] * t[:, 1], n[:, 2] * t[:, 0] - n[:, 0] * t[:, 2],
                      n[:, 0] * t[:, 1] - n[:, 1] * t[:, 0], n[:, 3] * t[:, 3] - n[:, 3] * t[:, 3]], 1)
    arrays = {0: p4, 1: tan, 2: norm4(cross), 3: nrm, 4: uv}
    rng = np.random.default_rng(3)
    diffuse, bump = S.checker_noise_bgra(32, 4, rng), _bump_texture(4)
    view = np.eye(4, dtype=np.float32)
    view[2, 3] = -2.5
    proj = S.perspective(0.1, 10.0, 96 / 64, np.radians(60.0))

    def frame(pipe, vao):
        tx = pipe.createTexture(32, 32, 128, 4, diffuse, 1)
        bx = pipe.createTexture(16, 16, 64, 4, bump, 1)
        dt = pipe.createTexture(96, 64, 96 * 4, 4, None, 0)
        prog = pipe.createProgramme(pipe.addProcessor(S.VP_DEF03), pipe.addProcessor(S.IP_DEF03),
                                    pipe.addProcessor(S.FP_DEF03))
        pipe.useProgramme(prog)
        pipe.setDepth(dt)
        pipe.clearDepth(1.0)
        pipe.clearColour(0xFF000000)
        pipe.setUniform(3, S.col_major(proj @ view))
        pipe.setUniform(4, S.col_major(np.eye(4)))
        pipe.setUniform(5, S.col_major(np.eye(4)))
        pipe.setUniform(7, S.vec4(2, 3, 4))
        pipe.setUniform(8, S.vec4(0, 0, 2.5))
        pipe.setUniform(9, np.array([tx], np.int32))
        pipe.setUniform(10, np.array([bx], np.int32))
        pipe.drawVAO(vao)
        return pipe.readColour(), pipe.readDepthTexture(dt).copy()

    g = PuresoftPipeline(96, 64)
    gc, gd = frame(g, g.loadObjxVao(path))
    o = OraclePipeline(96, 64)
    vao = o.createVAO()
    for slot, a in arrays.items():
        o.attachVBO(vao, slot, np.ascontiguousarray(a))
    oc, od = frame(o, vao)
    assert (gd < 1.0).sum() > 500
    assert_depth_exact(gd, od, "objx sphere")
    assert colour_diff(gc, oc)[0] <= 1
