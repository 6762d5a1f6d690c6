"""The two CPU checkers, behind the reference's PuresoftPipeline method names so
that puresoft3d_gb300.scenes.replay_* can drive them like the GPU pipeline.

* ``OraclePipeline`` -- the C restatement (oracle/ps3d_oracle.c), built by
  ``make -C oracle port``; runs on any host.
* ``RefPipeline`` -- the reference's own pipeline core compiled from its
  sources (oracle/_ref/libps3dref.so, ``make -C oracle ref``); exists only
  where the reference sources are (x86-64), and is used to make and check the
  golden fixtures.

Test infrastructure only.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libps3d_oracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libps3dref.so")
# the reference tree (read-only): PS3D_REFERENCE, else its checkout in the build container
REF_ROOT = os.environ.get("PS3D_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src", "puresoft3d")

_API = [
    ("texture_create", [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    ("texture_read", [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    ("texture_create_layers", [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                               ctypes.c_int]),
    ("texture_write_layer", [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    ("texture_read_layer", [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    ("processor_add", [ctypes.c_int]),
    ("programme_create", [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("programme_use", [ctypes.c_int]),
    ("vao_create", []),
    ("vbo_attach", [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    ("set_uniform", [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    ("set_depth", [ctypes.c_int]),
    ("set_fbo", [ctypes.c_int, ctypes.c_int]),
    ("set_viewport", [ctypes.c_int, ctypes.c_int]),
    ("enable", [ctypes.c_int]),
    ("disable", [ctypes.c_int]),
    ("clear_depth", [ctypes.c_float]),
    ("clear_colour", [ctypes.c_uint32]),
    ("draw", [ctypes.c_int]),
    ("read_colour", [ctypes.c_void_p]),
    ("post_process", [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
]


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return ORACLE_SO


def ref_available() -> bool:
    return os.path.isdir(REF_SRC) and os.uname().machine in ("x86_64", "AMD64")


def build_ref() -> str:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    return REF_SO


def _bind(lib, prefix):
    for name, args in _API:
        f = getattr(lib, prefix + name)
        f.argtypes = [ctypes.c_void_p] + args
        f.restype = ctypes.c_int


class _CPipeline:
    prefix = ""

    def __init__(self, lib, handle, width, height):
        self.lib, self.h, self.width, self.height = lib, ctypes.c_void_p(handle), width, height
        self._tex = {}

    def _call(self, name, *args):
        rc = getattr(self.lib, self.prefix + name)(self.h, *args)
        if rc < 0:
            raise {-1: IndexError, -2: ValueError, -3: MemoryError}.get(rc, RuntimeError)(f"{name}: {rc}")
        return rc

    def createTexture(self, width, height, scanline, elem_len, pixels, wrap, extra_layers=0):
        if pixels is not None:
            pixels = np.ascontiguousarray(pixels)
            assert pixels.nbytes == scanline * height
        idx = self._call("texture_create_layers", width, height, scanline, elem_len,
                         None if pixels is None else pixels.ctypes.data, int(wrap), int(extra_layers))
        self._tex[idx] = (width, height, scanline, elem_len)
        return idx

    def writeTextureLayer(self, idx, layer, pixels):
        pixels = np.ascontiguousarray(pixels)
        self._call("texture_write_layer", idx, layer, pixels.ctypes.data, pixels.nbytes)

    def readTexture(self, idx, layer=0) -> np.ndarray:
        w, h, scan, elem = self._tex[idx]
        out = np.empty((h, scan), dtype=np.uint8)
        self._call("texture_read_layer", idx, layer, out.ctypes.data, out.nbytes)
        return out

    def addProcessor(self, pid):
        return self._call("processor_add", pid)

    def createProgramme(self, v, i, f):
        return self._call("programme_create", v, i, f)

    def useProgramme(self, idx):
        self._call("programme_use", idx)

    def createVAO(self):
        return self._call("vao_create")

    def attachVBO(self, vao, slot, arr):
        arr = np.ascontiguousarray(arr)
        self._call("vbo_attach", vao, slot, arr.nbytes // len(arr), len(arr), arr.ctypes.data)

    def setUniform(self, idx, data):
        data = np.ascontiguousarray(data)
        self._call("set_uniform", idx, data.ctypes.data, data.nbytes)

    def setDepth(self, idx=-1):
        self._call("set_depth", idx)

    def setFBO(self, idx, tex=-1):
        self._call("set_fbo", idx, tex)

    def setViewport(self, w, h):
        self._call("set_viewport", w, h)

    def enable(self, bits):
        self._call("enable", bits)

    def disable(self, bits):
        self._call("disable", bits)

    def clearDepth(self, v=1.0):
        self._call("clear_depth", v)

    def clearColour(self, bgra=0):
        self._call("clear_colour", bgra)

    def drawVAO(self, vao):
        self._call("draw", vao)

    def postProcess(self, pp_id, params=None):
        buf = None if params is None else ctypes.create_string_buffer(bytes(params), len(params))
        self._call("post_process", pp_id, buf, 0 if params is None else len(params))

    def readColour(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), dtype=np.uint8)
        self._call("read_colour", out.ctypes.data)
        return out

    def readDepthTexture(self, idx) -> np.ndarray:
        w, h, scan, elem = self._tex[idx]
        return self.readTexture(idx).view(np.float32)[:, :w]


class OraclePipeline(_CPipeline):
    prefix = "ps3do_"
    _lib = None

    def __init__(self, width, height, threads=1):
        if OraclePipeline._lib is None:
            lib = ctypes.CDLL(build_oracle())
            lib.ps3do_create.restype = ctypes.c_void_p
            lib.ps3do_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
            lib.ps3do_destroy.argtypes = [ctypes.c_void_p]
            lib.ps3do_fragments_tested.restype = ctypes.c_longlong
            lib.ps3do_fragments_tested.argtypes = [ctypes.c_void_p]
            lib.ps3do_fragments_passed.restype = ctypes.c_longlong
            lib.ps3do_fragments_passed.argtypes = [ctypes.c_void_p]
            lib.ps3do_set_colour_error.argtypes = [ctypes.c_void_p, ctypes.c_int]
            lib.ps3do_colour_error.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_double)] * 2 + [
                ctypes.POINTER(ctypes.c_longlong)] * 2
            _bind(lib, "ps3do_")
            OraclePipeline._lib = lib
        lib = OraclePipeline._lib
        super().__init__(lib, lib.ps3do_create(width, height, threads), width, height)

    def fragments(self):
        return self.lib.ps3do_fragments_tested(self.h), self.lib.ps3do_fragments_passed(self.h)

    def readDepth(self) -> np.ndarray:
        """The default depth buffer, (height, scanline floats): the
        reference's scanline of round(width / 4) * 4 floats (pipeline.cpp:31)."""
        scan = int(self.width / 4.0 + 0.5) * 4
        out = np.empty((self.height, scan), dtype=np.float32)
        self.lib.ps3do_read_depth.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        self.lib.ps3do_read_depth(self.h, out.ctypes.data)
        return out

    def measureColourError(self, on=True):
        """Compare every shaded fragment's FP32 colour with an FP64 re-shade."""
        self.lib.ps3do_set_colour_error(self.h, int(on))

    def colourError(self):
        """{max, mean} |FP32 - FP64| per colour channel (8-bit units), the
        channels compared and how many differed by 1 or more."""
        mx, mean = ctypes.c_double(), ctypes.c_double()
        n, over = ctypes.c_longlong(), ctypes.c_longlong()
        self.lib.ps3do_colour_error(self.h, ctypes.byref(mx), ctypes.byref(mean), ctypes.byref(n), ctypes.byref(over))
        return {"max": mx.value, "mean": mean.value, "channels": n.value, "over_1": over.value}

    def close(self):
        if self.h:
            self.lib.ps3do_destroy(self.h)
            self.h = None

    __del__ = close


class RefPipeline(_CPipeline):
    prefix = "ps3dr_"
    _lib = None

    def __init__(self, width, height, threads=4):
        if RefPipeline._lib is None:
            os.environ.setdefault("PS3D_REF_THREADS", str(threads))
            lib = ctypes.CDLL(build_ref())
            lib.ps3dr_create.restype = ctypes.c_void_p
            lib.ps3dr_create.argtypes = [ctypes.c_int, ctypes.c_int]
            lib.ps3dr_destroy.argtypes = [ctypes.c_void_p]
            _bind(lib, "ps3dr_")
            RefPipeline._lib = lib
        lib = RefPipeline._lib
        super().__init__(lib, lib.ps3dr_create(width, height), width, height)

    def close(self):
        if self.h:
            self.lib.ps3dr_destroy(self.h)
            self.h = None

    __del__ = close
