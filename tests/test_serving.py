"""Serving: the packer, the result arena, the job stream (CPU), and on the
GPU that every served image is the same alone and in the mix."""
import numpy as np
import pytest

from puresoft3d_gb300 import scenes as S
from puresoft3d_gb300.serving import PlainLoop, RenderServer, ResultArena, ShelfPacker, summarize


def test_shelf_packer_no_overlap_in_bounds():
    rng = np.random.default_rng(3)
    pk = ShelfPacker(1000, 800)
    rects = []
    while True:
        w, h = int(rng.integers(20, 300)), int(rng.integers(20, 300))
        xy = pk.place(w, h)
        if xy is None:
            break
        rects.append((xy[0], xy[1], w, h))
    assert len(rects) > 5
    occ = np.zeros((800, 1000), dtype=np.int32)
    for x, y, w, h in rects:
        assert 0 <= x and x + w <= 1000 and 0 <= y and y + h <= 800
        occ[y:y + h, x:x + w] += 1
    assert occ.max() == 1


def test_shelf_packer_refuses_oversized():
    pk = ShelfPacker(512, 512)
    assert pk.place(513, 10) is None and pk.place(10, 513) is None
    assert pk.place(512, 512) == (0, 0)
    assert pk.place(1, 1) is None


def test_result_arena_first_fit_and_coalescing():
    a = ResultArena(4096, pinned=False)
    o1, o2, o3 = a.alloc(1000), a.alloc(1000), a.alloc(1000)
    assert (o1, o2, o3) == (0, 1024, 2048)
    assert a.alloc(2000) is None
    a.release(o2, 1000)
    a.release(o1, 1000)
    assert a.alloc(2000) == 0          # the two freed blocks merged
    a.release(0, 2000)
    a.release(o3, 1000)
    assert a.free == [(0, 4096)]


def test_job_stream_is_seeded_poisson():
    pool = S.scene_c5_pool(meshes=6, tri_min=100, tri_max=2000, textures=3, tex_size=32)
    a = S.c5_jobs(pool, n=400, rate=800.0, seed=9)
    b = S.c5_jobs(pool, n=400, rate=800.0, seed=9)
    assert [(j.arrival, j.width, j.mesh) for j in a] == [(j.arrival, j.width, j.mesh) for j in b]
    gaps = np.diff([0.0] + [j.arrival for j in a])
    assert 0.8 / 800 < gaps.mean() < 1.2 / 800
    assert {(j.width, j.height) for j in a} == set(S.C5_RESOLUTIONS)


def test_summarize():
    class J:
        def __init__(self, t):
            self.arrival = t
    from puresoft3d_gb300.serving import Done
    done = [Done(J(0.0), 0.0, 0.010, None, 0), Done(J(0.005), 0.0, 0.010, None, 0), Done(J(0.02), 0.02, 0.030, None, 1)]
    s = summarize(done)
    assert s["images"] == 3 and s["batches"] == 2
    assert abs(s["makespan_s"] - 0.030) < 1e-12
    assert abs(s["p50_ms"] - 10.0) < 1e-9


RES = ((64, 64), (128, 96), (200, 120))


@pytest.mark.gpu
def test_served_images_equal_alone(gpu_lib, monkeypatch):
    """Jobs of mixed resolutions and meshes, served with continuous batching
    (two slots, a small atlas so that batches are several), each give the
    image the job gives rendered alone in a pipeline of its own size."""
    monkeypatch.setattr(S, "C5_RESOLUTIONS", RES)
    pool = S.scene_c5_pool(meshes=8, tri_min=200, tri_max=20000, textures=4, tex_size=64)
    jobs = S.c5_jobs(pool, n=40, rate=4000.0, seed=21)
    srv = RenderServer(pool, atlas=(400, 256), slots=2)
    done = srv.serve(jobs, keep_images=True)
    assert sorted(d.job.id for d in done) == list(range(len(jobs)))
    assert len({d.batch for d in done}) >= 3
    plain = PlainLoop(pool, resolutions=RES)
    alone = {d.job.id: d.image for d in plain.serve(jobs, keep_images=True, realtime=False)}
    covered = 0
    for d in done:
        assert np.array_equal(d.image, alone[d.job.id]), "job %d differs in the mix" % d.job.id
        covered += int((d.image[..., :3].max(axis=2) > 0).sum())
    assert covered > 5000
    # and each served image is the oracle's render of the job (within 1 LSB)
    from cpu_backends import OraclePipeline
    from puresoft3d_gb300.serving import job_ops
    oracles = {}
    for wh in RES:
        oracles[wh] = OraclePipeline(wh[0], wh[1])
        S.replay_setup(pool, oracles[wh])
    for d in done:
        o = oracles[(d.job.width, d.job.height)]
        S.replay_ops(job_ops(pool, d.job), o)
        diff = np.abs(d.image.astype(np.int32) - o.readColour().astype(np.int32)).max()
        assert diff <= 1, "job %d: served image differs from the oracle by %d LSB" % (d.job.id, diff)
    for o in oracles.values():
        o.close()
    s = summarize(done)
    assert s["p99_ms"] >= s["p50_ms"] > 0
    srv.close()
    plain.close()


@pytest.mark.gpu
def test_job_larger_than_the_atlas_is_refused(gpu_lib, monkeypatch):
    monkeypatch.setattr(S, "C5_RESOLUTIONS", ((200, 120),))
    pool = S.scene_c5_pool(meshes=2, tri_min=200, tri_max=400, textures=1, tex_size=32)
    jobs = S.c5_jobs(pool, n=2, rate=1000.0, seed=3)
    srv = RenderServer(pool, atlas=(128, 128), slots=1)
    with pytest.raises(ValueError, match="never be admitted"):
        srv.serve(jobs)
    srv.close()


@pytest.mark.gpu
def test_jobs_wait_for_memory_and_all_complete(gpu_lib, monkeypatch):
    """A result arena with room for one 200x120 image and a scratch budget of
    a few thousand triangles per batch: jobs wait for memory to free up,
    every job still completes, and each image equals the job alone."""
    monkeypatch.setattr(S, "C5_RESOLUTIONS", RES)
    pool = S.scene_c5_pool(meshes=6, tri_min=200, tri_max=6000, textures=2, tex_size=32)
    jobs = S.c5_jobs(pool, n=24, rate=20000.0, seed=5)
    arena = 200 * 120 * 4 + 256
    budget = 2 * 7000 * 232   # two slots' share of scratch for ~7000 triangles each
    srv = RenderServer(pool, atlas=(400, 256), slots=2, hbm_budget=budget, arena_bytes=arena)
    done = srv.serve(jobs, keep_images=True)
    assert sorted(d.job.id for d in done) == list(range(len(jobs)))
    assert len({d.batch for d in done}) >= 6   # memory, not the atlas, bounds the batches
    plain = PlainLoop(pool, resolutions=RES)
    alone = {d.job.id: d.image for d in plain.serve(jobs, keep_images=True, realtime=False)}
    for d in done:
        assert np.array_equal(d.image, alone[d.job.id]), d.job.id
    srv.close()
    plain.close()
