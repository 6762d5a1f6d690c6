"""Python binding of the C ABI (include/ps3d.h) with the reference's method
names (PuresoftPipeline, src/puresoft3d/pipeline.h:26-69), so scenes and tests
drive the GPU pipeline exactly as the reference's demos drive theirs.

The library is the in-tree CUDA build (puresoft3d_gb300/_lib/libps3d.so).
There is no CPU fallback: if the library or a GPU is missing, construction
raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

PS3D_OK = 0
ERRORS = {-1: IndexError, -2: ValueError, -3: MemoryError, -4: RuntimeError, -5: TimeoutError}


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("draws", "batches", "kernel_launches", "triangles", "fragments",
                                                "fragments_passed", "replays", "bin_pairs", "shaded", "upload_bytes")]


_lib = None
_c_int, _c_void_p, _c_size_t = ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t
_SIGS = {
    "ps3d_pipeline_create": [_c_int, _c_int, _c_void_p, ctypes.POINTER(_c_void_p)],
    "ps3d_pipeline_destroy": [_c_void_p],
    "ps3d_texture_create": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_int],
    "ps3d_texture_create_device": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_int],
    "ps3d_texture_destroy": [_c_void_p, _c_int],
    "ps3d_texture_read": [_c_void_p, _c_int, _c_void_p, _c_size_t],
    "ps3d_selftest_occlusion": [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
    "ps3d_set_span_culling": [_c_void_p, _c_int],
    "ps3d_set_row_split": [_c_void_p, _c_int],
    "ps3d_post_process": [_c_void_p, _c_int, _c_void_p, _c_size_t],
    "ps3d_texture_create_layers": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_int, _c_int],
    "ps3d_texture_write_layer": [_c_void_p, _c_int, _c_int, _c_void_p, _c_size_t],
    "ps3d_texture_read_layer": [_c_void_p, _c_int, _c_int, _c_void_p, _c_size_t],
    "ps3d_texture_device_ptr": [_c_void_p, _c_int, ctypes.POINTER(_c_void_p)],
    "ps3d_processor_add": [_c_void_p, _c_int],
    "ps3d_processor_destroy": [_c_void_p, _c_int],
    "ps3d_programme_create": [_c_void_p, _c_int, _c_int, _c_int],
    "ps3d_programme_destroy": [_c_void_p, _c_int],
    "ps3d_programme_use": [_c_void_p, _c_int],
    "ps3d_vao_create": [_c_void_p],
    "ps3d_vao_destroy": [_c_void_p, _c_int],
    "ps3d_vbo_attach": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "ps3d_vbo_attach_device": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "ps3d_vbo_detach": [_c_void_p, _c_int, _c_int],
    "ps3d_set_uniform": [_c_void_p, _c_int, _c_void_p, _c_size_t],
    "ps3d_set_depth": [_c_void_p, _c_int],
    "ps3d_set_fbo": [_c_void_p, _c_int, _c_int],
    "ps3d_set_viewport": [_c_void_p, _c_int, _c_int],
    "ps3d_set_viewport_rect": [_c_void_p, _c_int, _c_int, _c_int, _c_int],
    "ps3d_enable": [_c_void_p, _c_int],
    "ps3d_disable": [_c_void_p, _c_int],
    "ps3d_clear_depth": [_c_void_p, ctypes.c_float],
    "ps3d_clear_colour": [_c_void_p, ctypes.c_uint32],
    "ps3d_draw": [_c_void_p, _c_int],
    "ps3d_flush": [_c_void_p],
    "ps3d_finish": [_c_void_p],
    "ps3d_finish_noalloc": [_c_void_p],
    "ps3d_vbo_update": [_c_void_p, _c_int, _c_int, _c_void_p],
    "ps3d_allocation_count": [],
    "ps3d_set_bin_width": [_c_void_p, _c_int],
    "ps3d_get_bin_width": [_c_void_p, ctypes.POINTER(_c_int)],
    "ps3d_set_raster_occupancy": [_c_void_p, _c_int],
    "ps3d_set_raster_warp_bins": [_c_void_p, _c_int],
    "ps3d_set_span_items": [_c_void_p, _c_int],
    "ps3d_set_lazy_varyings": [_c_void_p, _c_int],
    "ps3d_selftest_wait": [_c_void_p, _c_int, ctypes.POINTER(ctypes.c_float)],
    "ps3d_read_colour": [_c_void_p, _c_void_p],
    "ps3d_read_depth": [_c_void_p, _c_void_p],
    "ps3d_colour_device_ptr": [_c_void_p, ctypes.POINTER(_c_void_p)],
    "ps3d_read_colour_device": [_c_void_p, _c_void_p],
    "ps3d_copy_colour_rect": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_size_t],
    "ps3d_query": [_c_void_p],
    "ps3d_get_stream": [_c_void_p, ctypes.POINTER(_c_void_p)],
    "ps3d_set_fragment_counting": [_c_void_p, _c_int],
    "ps3d_stats": [_c_void_p, ctypes.POINTER(Stats)],
    "ps3d_cmdbuf_begin": [_c_void_p],
    "ps3d_cmdbuf_end": [_c_void_p, ctypes.POINTER(_c_void_p)],
    "ps3d_cmdbuf_submit": [_c_void_p, _c_void_p, _c_int],
    "ps3d_cmdbuf_destroy": [_c_void_p, _c_void_p],
    "ps3d_cmdbuf_input_bytes": [_c_void_p, _c_void_p, ctypes.POINTER(_c_size_t)],
    "ps3d_timer_begin": [_c_void_p],
    "ps3d_timer_end": [_c_void_p, ctypes.POINTER(ctypes.c_float)],
    "ps3d_profile_enable": [_c_void_p, _c_int],
    "ps3d_l2_scrub": [_c_void_p, _c_size_t],
    "ps3d_selftest_division": [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
    "ps3d_profile_read": [_c_void_p, ctypes.POINTER(_c_int), ctypes.POINTER(ctypes.c_double)],
}

KERNELS = ["setup", "scan", "emit", "bounds", "sort", "raster", "shade", "fill", "post"]


def library(path: str | None = None) -> ctypes.CDLL:
    """Loads (building first if stale) the in-tree CUDA library."""
    global _lib
    if _lib is None:
        path = path or _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        lib = ctypes.CDLL(path)
        for name, args in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        lib.ps3d_last_error.restype = ctypes.c_char_p
        lib.ps3d_last_error.argtypes = []
        lib.ps3d_allocation_count.restype = ctypes.c_ulonglong
        _lib = lib
    return _lib


def selftest_division(pairs: int = 1 << 28):
    """(reciprocal mismatches, quotient mismatches) of the kernels' fast exact
    division against CUDA's IEEE results."""
    lib = library()
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    rc = lib.ps3d_selftest_division(pairs, ctypes.byref(a), ctypes.byref(b))
    if rc < 0:
        raise RuntimeError(lib.ps3d_last_error().decode())
    return int(a.value), int(b.value)


def selftest_occlusion(cases: int = 1 << 22):
    """(spans wrongly declared occluded, spans declared occluded) of the
    raster's span occlusion test against the per-pixel loop."""
    lib = library()
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    rc = lib.ps3d_selftest_occlusion(cases, ctypes.byref(a), ctypes.byref(b))
    if rc < 0:
        raise RuntimeError(lib.ps3d_last_error().decode())
    return int(a.value), int(b.value)


def allocation_count() -> int:
    """Device and pinned-host allocations the library's pipelines have made
    so far (ps3d_allocation_count)."""
    return int(library().ps3d_allocation_count())


def exported_symbols() -> list:
    from . import objx
    return sorted(list(_SIGS) + list(objx._SIGS) + ["ps3d_last_error"])


class PuresoftPipeline:
    """GPU pipeline with the reference's API.  Indices returned by the create
    calls follow the reference's vacant-slot policy."""

    def __init__(self, width: int, height: int, stream: int | None = None):
        self.lib = library()
        h = ctypes.c_void_p()
        self._check(self.lib.ps3d_pipeline_create(width, height, stream, ctypes.byref(h)))
        self.h = h
        self.width, self.height = width, height
        self._tex = {}

    def _check(self, rc: int) -> int:
        if rc < 0:
            msg = self.lib.ps3d_last_error().decode(errors="replace")
            raise ERRORS.get(rc, RuntimeError)(msg)
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.ps3d_pipeline_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- textures
    def createTexture(self, width, height, scanline, elem_len, pixels=None, wrap=0, extra_layers=0) -> int:
        """createTexture(image, extraLayers, mode); `pixels` fills layer 0
        (five extra layers make a cube map, faces +x, -x, +y, -y, +z, -z)."""
        ptr = None
        if pixels is not None:
            pixels = np.ascontiguousarray(pixels)
            if pixels.nbytes != scanline * height:
                raise ValueError("pixel buffer is %d bytes, expected %d" % (pixels.nbytes, scanline * height))
            ptr = pixels.ctypes.data
        idx = self._check(self.lib.ps3d_texture_create_layers(self.h, width, height, scanline, elem_len, ptr,
                                                              int(wrap), int(extra_layers)))
        self._tex[idx] = (width, height, scanline, elem_len)
        return idx

    def writeTextureLayer(self, idx, layer, pixels):
        """Fills one layer (getTexture(idx, image, layer), then writing
        image.pixels, in the reference)."""
        pixels = np.ascontiguousarray(pixels)
        self._check(self.lib.ps3d_texture_write_layer(self.h, idx, layer, pixels.ctypes.data, pixels.nbytes))

    def destroyTexture(self, idx):
        self._check(self.lib.ps3d_texture_destroy(self.h, idx))
        self._tex.pop(idx, None)

    def readTexture(self, idx, layer=0) -> np.ndarray:
        w, h, scan, elem = self._tex[idx]
        out = np.empty((h, scan), dtype=np.uint8)
        self._check(self.lib.ps3d_texture_read_layer(self.h, idx, layer, out.ctypes.data, out.nbytes))
        return out

    def readDepthTexture(self, idx) -> np.ndarray:
        w, h, scan, elem = self._tex[idx]
        return self.readTexture(idx).view(np.float32)[:, :w]

    # -- processors and programmes
    def addProcessor(self, pid) -> int:
        return self._check(self.lib.ps3d_processor_add(self.h, pid))

    def destroyProcessor(self, idx):
        self._check(self.lib.ps3d_processor_destroy(self.h, idx))

    def createProgramme(self, v, i, f) -> int:
        return self._check(self.lib.ps3d_programme_create(self.h, v, i, f))

    def destroyProgramme(self, idx):
        self._check(self.lib.ps3d_programme_destroy(self.h, idx))

    def useProgramme(self, idx):
        self._check(self.lib.ps3d_programme_use(self.h, idx))

    # -- vertex arrays
    def createVAO(self) -> int:
        return self._check(self.lib.ps3d_vao_create(self.h))

    def destroyVAO(self, vao):
        self._check(self.lib.ps3d_vao_destroy(self.h, vao))

    def attachVBO(self, vao, slot, arr):
        arr = np.ascontiguousarray(arr)
        self._check(self.lib.ps3d_vbo_attach(self.h, vao, slot, arr.nbytes // max(len(arr), 1), len(arr),
                                             arr.ctypes.data))

    def updateVBO(self, vao, slot, arr):
        """getVBO(vao, slot)->updateContent(arr): the VBO's contents replaced in
        place (arr must hold exactly its unitBytes * count bytes)."""
        arr = np.ascontiguousarray(arr)
        self._check(self.lib.ps3d_vbo_update(self.h, vao, slot, arr.ctypes.data))

    def detachVBO(self, vao, slot):
        self._check(self.lib.ps3d_vbo_detach(self.h, vao, slot))

    # -- state
    def setUniform(self, idx, data):
        if data is None:
            self._check(self.lib.ps3d_set_uniform(self.h, idx, None, 0))
            return
        data = np.ascontiguousarray(data)
        self._check(self.lib.ps3d_set_uniform(self.h, idx, data.ctypes.data, data.nbytes))

    def setDepth(self, idx=-1):
        self._check(self.lib.ps3d_set_depth(self.h, idx))

    def setFBO(self, idx, texture=-1):
        """setFBO(idx, fbo): a texture as FBO slot idx (-1: none; slot 0 then
        the display).  Draws colour slot 0; clearColour clears the display."""
        self._check(self.lib.ps3d_set_fbo(self.h, idx, texture))

    def setViewport(self, w, h):
        self._check(self.lib.ps3d_set_viewport(self.h, w, h))

    def setViewportRect(self, x, y, w, h):
        self._check(self.lib.ps3d_set_viewport_rect(self.h, x, y, w, h))

    def enable(self, bits):
        self._check(self.lib.ps3d_enable(self.h, bits))

    def disable(self, bits):
        self._check(self.lib.ps3d_disable(self.h, bits))

    def clearDepth(self, v=1.0):
        self._check(self.lib.ps3d_clear_depth(self.h, v))

    def clearColour(self, bgra=0):
        self._check(self.lib.ps3d_clear_colour(self.h, bgra))

    def drawVAO(self, vao):
        self._check(self.lib.ps3d_draw(self.h, vao))

    def flush(self):
        self._check(self.lib.ps3d_flush(self.h))

    def finish(self):
        self._check(self.lib.ps3d_finish(self.h))

    def setBinWidth(self, columns: int):
        """Bin width (8, 16 or 32 columns) of the passes launched from now on."""
        self._check(self.lib.ps3d_set_bin_width(self.h, columns))

    def setRasterOccupancy(self, blocks_per_sm: int):
        """Raster kernel variant: 0 (registers as needed) or 8 blocks per SM."""
        self._check(self.lib.ps3d_set_raster_occupancy(self.h, blocks_per_sm))

    def setRowSplit(self, blocks_per_bin: int):
        """Raster blocks per bin (1, 2, 4 or 8): crowded bins shared out by rows."""
        self._check(self.lib.ps3d_set_row_split(self.h, blocks_per_bin))

    def setWarpBins(self, on: bool):
        """Raster shape: one warp per bin of 8 or 16 columns (on) or four
        warps sharing each bin (off, the default)."""
        self._check(self.lib.ps3d_set_raster_warp_bins(self.h, int(bool(on))))

    def setSpanItems(self, on: bool):
        """Bin short triangles' row spans as set-up items (on) or whole
        triangles whose spans the raster sets up (off, the default)."""
        self._check(self.lib.ps3d_set_span_items(self.h, int(bool(on))))

    def setLazyVaryings(self, on: bool):
        """The shade computes its winners' vertex varyings (on) or the set-up
        stores every binned triangle's (off, the default)."""
        self._check(self.lib.ps3d_set_lazy_varyings(self.h, int(bool(on))))

    def setSpanCulling(self, on: bool):
        """Raster kernel variant: drop occluded spans before their depths are
        computed (on, the default) or not."""
        self._check(self.lib.ps3d_set_span_culling(self.h, int(bool(on))))

    def selftestWait(self, spins: int) -> float:
        """Runs a bounded wait that must run out; raises TimeoutError (with
        the kernel's milliseconds in the message) as the library reports an
        expired device wait.  Returns only if the wait did not run out."""
        ms = ctypes.c_float()
        rc = self.lib.ps3d_selftest_wait(self.h, spins, ctypes.byref(ms))
        if rc == -5:
            raise TimeoutError("%.3f ms: %s" % (ms.value, self.lib.ps3d_last_error().decode(errors="replace")))
        self._check(rc)
        return ms.value

    def binWidth(self) -> int:
        v = _c_int()
        self._check(self.lib.ps3d_get_bin_width(self.h, ctypes.byref(v)))
        return v.value

    def finishNoAlloc(self):
        """ps3d_finish_noalloc: finish() with every pass's scratch taken from
        a fixed 16 MiB device array; allocates no device memory.  Raises
        IndexError (nothing ran) when a pass is too large for the array, and
        MemoryError when a pass's bin lists overflowed it (finish() then
        completes the frame)."""
        self._check(self.lib.ps3d_finish_noalloc(self.h))

    # -- read-back
    def readColour(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 4), dtype=np.uint8)
        self._check(self.lib.ps3d_read_colour(self.h, out.ctypes.data))
        return out

    def readColourDevice(self, dev_ptr: int):
        self._check(self.lib.ps3d_read_colour_device(self.h, dev_ptr))

    def copyColourRect(self, x, y, w, h, dst_ptr: int, pitch: int):
        """Records a read-out of the colour rectangle (x, y, w, h) to dst_ptr
        (device or pinned host memory), rows top-down, `pitch` bytes apart."""
        self._check(self.lib.ps3d_copy_colour_rect(self.h, x, y, w, h, dst_ptr, pitch))

    def loadObjxVao(self, path: str, mesh: int = 0) -> int:
        """A VAO from an OBJX mesh, laid out as the reference demo does
        (positions, tangents, binormals, normals, texture coordinates)."""
        from .objx import load_vao
        return load_vao(self, path, mesh)

    def postProcess(self, pp_id: int, params: bytes = None):
        """postProcess(processor): records a built-in post-processor
        (PS3D_PP_*) over the colour buffer, in order with the draws; `params`
        are its parameter bytes (see scenes.fog_params)."""
        buf = None if params is None else ctypes.create_string_buffer(bytes(params), len(params))
        self._check(self.lib.ps3d_post_process(self.h, pp_id, buf, 0 if params is None else len(params)))

    def query(self) -> bool:
        """True when all launched work has completed (no wait)."""
        return self._check(self.lib.ps3d_query(self.h)) == 1

    def textureDevicePtr(self, idx) -> int:
        v = ctypes.c_void_p()
        self._check(self.lib.ps3d_texture_device_ptr(self.h, idx, ctypes.byref(v)))
        return v.value

    def readDepth(self) -> np.ndarray:
        """The default depth buffer, (height, scanline floats)."""
        scan = int(self.width / 4.0 + 0.5) * 4
        scan = max(scan, (self.width + 3) // 4 * 4)
        out = np.empty((self.height, scan), dtype=np.float32)
        self._check(self.lib.ps3d_read_depth(self.h, out.ctypes.data))
        return out

    def colourDevicePtr(self) -> int:
        v = ctypes.c_void_p()
        self._check(self.lib.ps3d_colour_device_ptr(self.h, ctypes.byref(v)))
        return v.value

    def stream(self) -> int:
        v = ctypes.c_void_p()
        self._check(self.lib.ps3d_get_stream(self.h, ctypes.byref(v)))
        return v.value

    def setFragmentCounting(self, on: bool):
        self._check(self.lib.ps3d_set_fragment_counting(self.h, int(on)))

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.ps3d_stats(self.h, ctypes.byref(s)))
        return {n: int(getattr(s, n)) for n, _ in Stats._fields_}

    # -- command buffers (recorded once, replayed as CUDA graphs)
    def beginCommands(self):
        self._check(self.lib.ps3d_cmdbuf_begin(self.h))

    def endCommands(self) -> "CommandBuffer":
        cb = ctypes.c_void_p()
        self._check(self.lib.ps3d_cmdbuf_end(self.h, ctypes.byref(cb)))
        return CommandBuffer(self, cb)

    # -- timing
    def timerBegin(self):
        self._check(self.lib.ps3d_timer_begin(self.h))

    def timerEnd(self) -> float:
        ms = ctypes.c_float()
        self._check(self.lib.ps3d_timer_end(self.h, ctypes.byref(ms)))
        return float(ms.value)

    def scrubL2(self, nbytes: int = 256 << 20):
        self._check(self.lib.ps3d_l2_scrub(self.h, nbytes))

    def profile(self, on: bool):
        self._check(self.lib.ps3d_profile_enable(self.h, int(on)))

    def profileRead(self) -> dict:
        n = (ctypes.c_int * len(KERNELS))()
        ms = (ctypes.c_double * len(KERNELS))()
        self._check(self.lib.ps3d_profile_read(self.h, n, ms))
        return {k: (int(n[i]), float(ms[i])) for i, k in enumerate(KERNELS)}


class CommandBuffer:
    """A recorded frame; submit() replays it (as a CUDA graph after the first
    submission)."""

    def __init__(self, pipe: PuresoftPipeline, handle):
        self.pipe, self.h = pipe, handle

    def submit(self, upload_inputs: bool = False):
        self.pipe._check(self.pipe.lib.ps3d_cmdbuf_submit(self.pipe.h, self.h, int(upload_inputs)))

    def input_bytes(self) -> int:
        n = ctypes.c_size_t()
        self.pipe._check(self.pipe.lib.ps3d_cmdbuf_input_bytes(self.pipe.h, self.h, ctypes.byref(n)))
        return int(n.value)

    def destroy(self):
        if self.h and self.pipe.h:
            self.pipe._check(self.pipe.lib.ps3d_cmdbuf_destroy(self.pipe.h, self.h))
        self.h = None
