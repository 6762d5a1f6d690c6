"""Generates the golden fixtures in this directory by rendering each case on
the reference's own pipeline core (oracle/_ref/libps3dref.so: the reference
sources compiled unmodified on Linux, see oracle/Makefile).

Each fixture records
  * ``digest``     -- sha256 of the scene's inputs (every call and array);
  * ``colour_sha`` / ``depth_sha`` (/ ``shadow_sha``) -- sha256 of the
    read-back buffers;
  * for the small known-answer scenes, the buffers themselves;
  * ``covered``    -- pixels whose depth is below the clear value.

The full-size cases (``full_cases``: configs 2 and 3 exactly as the benchmark
renders them) keep hashes only.

Run from the repository root on an x86-64 host with the reference tree:
    python tests/golden/make_golden.py [case name ...]
(no names: every case, the full-size ones included).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from puresoft3d_gb300 import scenes as S  # noqa: E402
import kat_scenes  # noqa: E402


def scene_digest(scene) -> str:
    h = hashlib.sha256()
    for op in list(scene.setup) + ["|"] + list(scene.frame):
        for item in (op if isinstance(op, tuple) else (op,)):
            if isinstance(item, np.ndarray):
                h.update(str(item.dtype).encode() + str(item.shape).encode())
                h.update(np.ascontiguousarray(item).tobytes())
            elif isinstance(item, dict):
                for k in sorted(item):
                    h.update(str(k).encode())
                    h.update(np.ascontiguousarray(item[k]).tobytes())
            elif isinstance(item, list):  # the layers of a layered texture
                for a in item:
                    h.update(str(a.dtype).encode() + str(a.shape).encode())
                    h.update(np.ascontiguousarray(a).tobytes())
            else:
                h.update(repr(item).encode())
    return h.hexdigest()


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden_cases():
    cases = list(kat_scenes.kat_scenes())
    cases.append(("c1_640x480", S.scene_c1()))
    cases.append(("c2_small_320x180", S.scene_c2(width=320, height=180, shadow_size=256, meshes=12, tex_size=64, spread=5.0)))
    cases.append(("c3_small_384x216", S.scene_c3(width=384, height=216, meshes=16, tri_target=20000, tex_size=64,
                                                 textures=2)))
    return cases


def full_cases():
    """Configs 2 and 3 at the size the benchmark renders them (the same
    generator calls as bench.py's workloads): hash-only fixtures."""
    return [("c2_1920x1080", S.scene_c2()), ("c3_3840x2160", S.scene_c3())]


def render(pipe_cls, scene):
    p = pipe_cls(scene.width, scene.height)
    S.replay_setup(scene, p)
    S.replay_frame(scene, p)
    out = {"colour": p.readColour(), "depth": p.readDepthTexture(scene.info["depth_texture"])}
    if "shadow_texture" in scene.info:
        out["shadow"] = p.readDepthTexture(scene.info["shadow_texture"])
    for t in scene.info.get("read_textures", []):
        out["tex%d" % t] = p.readTexture(t)
    p.close()
    return out


def main():
    from cpu_backends import RefPipeline, ref_available
    if not ref_available():
        raise SystemExit("the reference sources are needed to make golden fixtures")
    only = set(sys.argv[1:])
    for name, make in [(n, (lambda s=s: s)) for n, s in golden_cases()] + [
            ("c2_1920x1080", S.scene_c2), ("c3_3840x2160", S.scene_c3)]:
        if only and name not in only:
            continue
        scene = make()
        out = render(RefPipeline, scene)
        rec = {"digest": scene_digest(scene), "colour_sha": sha(out["colour"]), "depth_sha": sha(out["depth"]),
               "covered": int((out["depth"] < 1.0).sum())}
        if "shadow" in out:
            rec["shadow_sha"] = sha(out["shadow"])
        for k in out:
            if k.startswith("tex"):
                rec[k + "_sha"] = sha(out[k])
                rec[k] = out[k]
        if name.startswith("kat_"):
            rec["colour"] = out["colour"]
            rec["depth"] = out["depth"]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
        print(name, rec["covered"], rec["colour_sha"][:12], rec["depth_sha"][:12])


if __name__ == "__main__":
    main()
