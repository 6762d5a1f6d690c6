"""Shared helpers for the parity tests (test infrastructure)."""
from __future__ import annotations

import hashlib
import os

import numpy as np

from puresoft3d_gb300 import scenes as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def render(pipe, scene):
    S.replay_setup(scene, pipe)
    S.replay_frame(scene, pipe)
    out = {"colour": pipe.readColour(), "depth": pipe.readDepthTexture(scene.info["depth_texture"])}
    if "shadow_texture" in scene.info:
        out["shadow"] = pipe.readDepthTexture(scene.info["shadow_texture"])
    for t in scene.info.get("read_textures", []):  # textures a scene renders into (setFBO)
        out["tex%d" % t] = pipe.readTexture(t)
    return out


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def assert_depth_exact(a, b, what=""):
    a32, b32 = np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32)
    bad = np.argwhere(a32 != b32)
    assert bad.size == 0, "%s: %d depth values differ, first at (row, col) %s: %r vs %r" % (
        what, len(bad), tuple(bad[0]), a[tuple(bad[0])], b[tuple(bad[0])])


def colour_diff(a, b):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    return int(d.max()), float(d.mean())
