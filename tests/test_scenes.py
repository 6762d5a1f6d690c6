"""The seeded scene generators."""
import numpy as np

from puresoft3d_gb300 import scenes as S


def test_c1_sphere_rule():
    m = S.uv_sphere(32, 16, poles="grid")
    assert S.mesh_triangles(m) == 992
    p = m["position"][:, :3].reshape(-1, 3, 3).astype(np.float64)
    area = np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 1]), axis=1)
    assert (area < 1e-9).sum() == 32  # the north pole's zero-area row


def test_meshes_wind_counter_clockwise_outside():
    for m in (S.uv_sphere(12, 8), S.torus(10, 8), S.box(3)):
        p = m["position"][:, :3].reshape(-1, 3, 3).astype(np.float64)
        n = m["normal"][:, :3].reshape(-1, 3, 3).astype(np.float64).mean(1)
        s = (np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 1]) * n).sum(1)
        assert (s > 0).all()


def test_mip_chain_rounding():
    lvl = np.array([[[0, 1, 2, 3], [1, 1, 1, 1]], [[2, 2, 2, 2], [3, 3, 3, 255]]], dtype=np.uint8)
    chain = S.mip_chain_u8(lvl)
    assert len(chain) == 2 and chain[1].shape == (1, 1, 4)
    assert chain[1][0, 0].tolist() == [(0 + 1 + 2 + 3 + 2) >> 2, (1 + 1 + 2 + 3 + 2) >> 2, (2 + 1 + 2 + 3 + 2) >> 2,
                                       (3 + 1 + 2 + 255 + 2) >> 2]


def test_scene_determinism():
    a, b = S.scene_c1(), S.scene_c1()
    for x, y in zip(a.setup, b.setup):
        if x[0] == "vao":
            for k in x[1]:
                assert np.array_equal(x[1][k], y[1][k])


def test_c2_small_counts():
    sc = S.scene_c2(width=160, height=90, shadow_size=128, meshes=6, tex_size=32, spread=5.0)
    draws = [op for op in sc.frame if op[0] == "drawVAO"]
    assert len(draws) == 12 and sc.info["triangles"] > 0
