"""The C++ adapter (include/ps3d.hpp: the reference's class and method names
over the C ABI) renders known-answer scenes as the oracle does, and the
in-place VBO update (getVBO(vao, idx)->updateContent, as the reference's
demo loads its meshes, test/scenobj.cpp:135-157) takes effect for the draws
after it only.

The scene's calls are recorded in Python (CallRecorder has the pipeline's
method names, so scenes.replay_* drive it like a pipeline) and played by a
small C++ program built against the library (tests/adapter_player.cpp)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from common import assert_depth_exact, colour_diff, render
from cpu_backends import OraclePipeline

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PLAYER_SRC = os.path.join(ROOT, "tests", "adapter_player.cpp")

(END, CREATE_TEXTURE, WRITE_LAYER, ADD_PROCESSOR, CREATE_PROGRAMME, USE_PROGRAMME, CREATE_VAO, ATTACH_VBO,
 SET_UNIFORM, SET_DEPTH, SET_VIEWPORT, ENABLE, DISABLE, CLEAR_DEPTH, CLEAR_COLOUR, DRAW_VAO, UPDATE_VBO,
 READ_TEXTURE, POST_PROCESS) = range(19)


class CallRecorder:
    """Records PuresoftPipeline calls in adapter_player's stream format; the
    create calls return the indices every implementation hands out (creation
    order)."""

    def __init__(self, width, height):
        self.width, self.height = width, height
        self.buf = bytearray(struct.pack("<ii", width, height))
        self.ntex = self.nproc = self.nprog = self.nvao = 0
        self.tex = {}
        self.reads = []

    def _op(self, op, *ints):
        self.buf += struct.pack("<i", op) + b"".join(struct.pack("<i", int(v)) for v in ints)

    def _bytes(self, data):
        b = b"" if data is None else np.ascontiguousarray(data).tobytes()
        self.buf += struct.pack("<q", len(b)) + b

    def createTexture(self, width, height, scanline, elem_len, pixels, wrap, extra_layers=0):
        self._op(CREATE_TEXTURE, width, height, scanline, elem_len, int(wrap), extra_layers)
        self._bytes(pixels)
        self.tex[self.ntex] = (width, height, scanline, elem_len)
        self.ntex += 1
        return self.ntex - 1

    def writeTextureLayer(self, idx, layer, pixels):
        self._op(WRITE_LAYER, idx, layer)
        self._bytes(pixels)

    def addProcessor(self, pid):
        self._op(ADD_PROCESSOR, pid)
        self.nproc += 1
        return self.nproc - 1

    def createProgramme(self, v, i, f):
        self._op(CREATE_PROGRAMME, v, i, f)
        self.nprog += 1
        return self.nprog - 1

    def useProgramme(self, idx):
        self._op(USE_PROGRAMME, idx)

    def createVAO(self):
        self._op(CREATE_VAO)
        self.nvao += 1
        return self.nvao - 1

    def attachVBO(self, vao, slot, arr):
        arr = np.ascontiguousarray(arr)
        self._op(ATTACH_VBO, vao, slot, arr.nbytes // max(len(arr), 1), len(arr))
        self._bytes(arr)

    def updateVBO(self, vao, slot, arr):
        self._op(UPDATE_VBO, vao, slot)
        self._bytes(arr)

    def setUniform(self, idx, data):
        self._op(SET_UNIFORM, idx)
        self._bytes(data)

    def setDepth(self, idx=-1):
        self._op(SET_DEPTH, idx)

    def setViewport(self, w, h):
        self._op(SET_VIEWPORT, w, h)

    def enable(self, bits):
        self._op(ENABLE, bits)

    def disable(self, bits):
        self._op(DISABLE, bits)

    def clearDepth(self, v=1.0):
        self.buf += struct.pack("<if", CLEAR_DEPTH, v)

    def clearColour(self, bgra=0):
        self.buf += struct.pack("<iI", CLEAR_COLOUR, bgra & 0xFFFFFFFF)

    def drawVAO(self, vao):
        self._op(DRAW_VAO, vao)

    def postProcess(self, pp_id, params=None):
        self._op(POST_PROCESS, pp_id)
        self._bytes(None if params is None else np.frombuffer(bytes(params), dtype=np.uint8))

    def readTexture(self, idx):
        w, h, scan, elem = self.tex[idx]
        self._op(READ_TEXTURE, idx, scan, h)
        self.reads.append((idx, scan, h))

    def play(self, exe, tmp_path):
        """Runs the recorded calls through the adapter; returns the colour
        buffer and the textures read, in order."""
        calls, out = tmp_path / "calls.bin", tmp_path / "out.bin"
        calls.write_bytes(bytes(self.buf) + struct.pack("<i", END))
        r = subprocess.run([str(exe), str(calls), str(out)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        raw = out.read_bytes()
        n = self.width * self.height * 4
        colour = np.frombuffer(raw[:n], dtype=np.uint8).reshape(self.height, self.width, 4)
        reads, off = [], n
        for idx, scan, h in self.reads:
            reads.append(np.frombuffer(raw[off:off + scan * h], dtype=np.uint8).reshape(h, scan))
            off += scan * h
        return colour, reads


@pytest.fixture(scope="module")
def player(tmp_path_factory, gpu_lib):
    from puresoft3d_gb300 import build
    lib = build.build()
    exe = tmp_path_factory.mktemp("adapter") / "adapter_player"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), PLAYER_SRC, lib,
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], check=True)
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["kat_soup_lit", "kat_def03_soup", "kat_def04_sky_soup", "c2_small",
                                  "kat_post_add_fog"])
def test_adapter_renders_like_the_oracle(player, tmp_path, case):
    from golden.make_golden import golden_cases
    from puresoft3d_gb300 import scenes as S
    name, scene = [c for c in golden_cases() if c[0].startswith(case)][0]
    rec = CallRecorder(scene.width, scene.height)
    S.replay_setup(scene, rec)
    S.replay_frame(scene, rec)
    targets = [scene.info["depth_texture"]] + ([scene.info["shadow_texture"]] if "shadow_texture" in scene.info
                                               else [])
    for t in targets:
        rec.readTexture(t)
    colour, reads = rec.play(player, tmp_path)
    ora = render(OraclePipeline(scene.width, scene.height), scene)
    w = scene.width
    assert_depth_exact(reads[0].view(np.float32)[:, :w], ora["depth"], name + " through the adapter")
    if len(reads) > 1:
        ss = ora["shadow"].shape[1]
        assert_depth_exact(reads[1].view(np.float32)[:, :ss], ora["shadow"], name + " shadow map")
    mx, mean = colour_diff(colour, ora["colour"])
    assert mx <= 1, "%s: colour differs by up to %d LSB (mean %.4f)" % (name, mx, mean)


def _moved(scene, dx):
    """The scene's first VAO's positions shifted by dx in x (model space)."""
    vao_op = [op for op in scene.setup if op[0] == "vao"][0]
    pos = np.array(vao_op[1][0], dtype=np.float32, copy=True)
    pos[:, 0] += dx
    return pos


@pytest.mark.gpu
def test_vbo_update_in_place(player, tmp_path):
    """Frame, then updateContent of the positions, then the frame again:
    through the adapter and through the C ABI from Python, each frame equals
    the oracle's render with the VBO attached with those contents; a draw
    recorded before the update still reads the old contents."""
    from golden.make_golden import golden_cases
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    name, scene = [c for c in golden_cases() if c[0].startswith("kat_soup_lit")][0]
    moved = _moved(scene, 0.15)

    def oracle(pos):
        o = OraclePipeline(scene.width, scene.height)
        S.replay_setup(scene, o)
        if pos is not None:
            o.attachVBO(0, 0, pos)  # replaces the first VAO's positions
        S.replay_frame(scene, o)
        return o.readColour(), o.readDepthTexture(scene.info["depth_texture"]).copy()

    before, after = oracle(None), oracle(moved)
    assert colour_diff(before[0], after[0])[0] > 0, "the move must change the frame"

    # through the adapter: frame (read), update, frame (read)
    rec = CallRecorder(scene.width, scene.height)
    S.replay_setup(scene, rec)
    S.replay_frame(scene, rec)
    rec.readTexture(scene.info["depth_texture"])
    rec.updateVBO(0, 0, moved)
    S.replay_frame(scene, rec)
    rec.readTexture(scene.info["depth_texture"])
    colour, reads = rec.play(player, tmp_path)
    w = scene.width
    assert_depth_exact(reads[0].view(np.float32)[:, :w], before[1], "before the update")
    assert_depth_exact(reads[1].view(np.float32)[:, :w], after[1], "after the update")
    assert colour_diff(colour, after[0])[0] <= 1

    # through the C ABI: a frame recorded before the update (not yet
    # finished) still renders the old contents
    g = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, g)
    S.replay_frame(scene, g)
    g.updateVBO(0, 0, moved)
    assert_depth_exact(g.readDepthTexture(scene.info["depth_texture"]), before[1], "recorded before the update")
    S.replay_frame(scene, g)
    assert_depth_exact(g.readDepthTexture(scene.info["depth_texture"]), after[1], "recorded after the update")
    assert colour_diff(g.readColour(), after[0])[0] <= 1
    with pytest.raises(IndexError):
        g.updateVBO(0, 7, moved)  # an empty slot
    g.close()
