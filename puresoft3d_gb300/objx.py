"""OBJX mesh files (the reference's objcvt/objxio.h:42-52) through the C ABI
(include/ps3d.h ps3d_objx_*): ``read_objx`` returns the scene description and
every mesh with its arrays, ``write_objx`` writes them, and
``PuresoftPipeline.loadObjxVao`` builds the reference demo's vertex arrays
from a mesh.  Reading and writing need no GPU."""
from __future__ import annotations

import ctypes
from typing import Dict, List, Optional, Tuple

import numpy as np

from .pipeline import ERRORS, library

_NAME = 260


class ObjxScene(ctypes.Structure):
    _fields_ = [("camera_pos", ctypes.c_float * 4), ("camera_ypr", ctypes.c_float * 4),
                ("light_pos", (ctypes.c_float * 4) * 4), ("light_dir", (ctypes.c_float * 4) * 4),
                ("light_types", ctypes.c_int * 4)]


class ObjxMeshInfo(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * _NAME), ("num_vertices", ctypes.c_uint), ("num_indices", ctypes.c_uint),
                ("has_texcoords", ctypes.c_int), ("has_normals", ctypes.c_int), ("has_tangents", ctypes.c_int),
                ("ambient", ctypes.c_float * 4), ("diffuse", ctypes.c_float * 4), ("specular", ctypes.c_float * 4),
                ("specular_exponent", ctypes.c_float),
                ("diffuse_file", ctypes.c_char * _NAME), ("bump_file", ctypes.c_char * _NAME),
                ("spc_file", ctypes.c_char * _NAME), ("spe_file", ctypes.c_char * _NAME),
                ("programme", ctypes.c_char * _NAME)]


_P = ctypes.c_void_p
_SIGS = {
    "ps3d_objx_create": [ctypes.c_char_p, ctypes.POINTER(ObjxScene), ctypes.POINTER(_P)],
    "ps3d_objx_write_mesh": [_P, ctypes.POINTER(ObjxMeshInfo), _P, _P, _P, _P, _P],
    "ps3d_objx_open": [ctypes.c_char_p, ctypes.POINTER(ObjxScene), ctypes.POINTER(_P)],
    "ps3d_objx_mesh_count": [_P],
    "ps3d_objx_read_mesh_header": [_P, ctypes.POINTER(ObjxMeshInfo)],
    "ps3d_objx_read_mesh": [_P, _P, _P, _P, _P, _P],
    "ps3d_objx_close": [_P],
    "ps3d_objx_load_vao": [_P, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
}


def _lib():
    lib = library()
    for name, args in _SIGS.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    return lib


def _check(lib, rc):
    if rc < 0:
        raise ERRORS.get(rc, RuntimeError)(lib.ps3d_last_error().decode(errors="replace"))
    return rc


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def read_objx(path: str, tangents: bool = False) -> Tuple[Dict, List[Dict]]:
    """(scene, meshes): each mesh a dict of its header fields and arrays
    ("vertices" (n, 4), "normals" (n, 4), "tangents" (n, 4), "texcoords"
    (n, 2), "indices" (m,)), present as the file has them; with `tangents`,
    tangents missing from the file are derived from the texture
    coordinates."""
    lib = _lib()
    scn, h = ObjxScene(), _P()
    _check(lib, lib.ps3d_objx_open(path.encode(), ctypes.byref(scn), ctypes.byref(h)))
    try:
        meshes = []
        for _ in range(_check(lib, lib.ps3d_objx_mesh_count(h))):
            info = ObjxMeshInfo()
            _check(lib, lib.ps3d_objx_read_mesh_header(h, ctypes.byref(info)))
            nv, ni = info.num_vertices, info.num_indices
            m = {"name": info.name.decode(errors="replace"), "num_vertices": nv, "num_indices": ni,
                 "ambient": np.array(info.ambient[:], np.float32), "diffuse": np.array(info.diffuse[:], np.float32),
                 "specular": np.array(info.specular[:], np.float32), "specular_exponent": info.specular_exponent,
                 "diffuse_file": info.diffuse_file.decode(errors="replace"),
                 "bump_file": info.bump_file.decode(errors="replace"),
                 "spc_file": info.spc_file.decode(errors="replace"), "spe_file": info.spe_file.decode(errors="replace"),
                 "programme": info.programme.decode(errors="replace")}
            m["vertices"] = np.empty((nv, 4), np.float32)
            if info.has_normals:
                m["normals"] = np.empty((nv, 4), np.float32)
            if info.has_tangents or (tangents and info.has_texcoords):
                m["tangents"] = np.empty((nv, 4), np.float32)
            if info.has_texcoords:
                m["texcoords"] = np.empty((nv, 2), np.float32)
            if ni:
                m["indices"] = np.empty(ni, np.int32)
            _check(lib, lib.ps3d_objx_read_mesh(h, _ptr(m["vertices"]), _ptr(m.get("normals")),
                                                _ptr(m.get("tangents")), _ptr(m.get("texcoords")),
                                                _ptr(m.get("indices"))))
            meshes.append(m)
    finally:
        lib.ps3d_objx_close(h)
    s = {"camera_pos": np.array(scn.camera_pos[:], np.float32), "camera_ypr": np.array(scn.camera_ypr[:], np.float32),
         "light_pos": np.array([r[:] for r in scn.light_pos], np.float32),
         "light_dir": np.array([r[:] for r in scn.light_dir], np.float32), "light_types": list(scn.light_types)}
    return s, meshes


def write_objx(path: str, scene: Dict, meshes: List[Dict]) -> None:
    lib = _lib()
    scn = ObjxScene()
    for key in ("camera_pos", "camera_ypr"):
        getattr(scn, key)[:] = [float(v) for v in scene.get(key, np.zeros(4))]
    for l in range(4):
        scn.light_pos[l][:] = [float(v) for v in np.asarray(scene.get("light_pos", np.zeros((4, 4))))[l]]
        scn.light_dir[l][:] = [float(v) for v in np.asarray(scene.get("light_dir", np.zeros((4, 4))))[l]]
    h = _P()
    _check(lib, lib.ps3d_objx_create(path.encode(), ctypes.byref(scn), ctypes.byref(h)))
    try:
        for m in meshes:
            info = ObjxMeshInfo()
            arrs = {k: (np.ascontiguousarray(m[k], np.int32 if k == "indices" else np.float32) if k in m else None)
                    for k in ("vertices", "normals", "tangents", "texcoords", "indices")}
            info.name = m.get("name", "").encode()[:_NAME - 1]
            info.num_vertices = len(arrs["vertices"])
            info.num_indices = 0 if arrs["indices"] is None else len(arrs["indices"])
            for key in ("ambient", "diffuse", "specular"):
                getattr(info, key)[:] = [float(v) for v in m.get(key, np.zeros(4))]
            info.specular_exponent = float(m.get("specular_exponent", 0.0))
            for key in ("diffuse_file", "bump_file", "spc_file", "spe_file", "programme"):
                setattr(info, key, m.get(key, "").encode()[:_NAME - 1])
            _check(lib, lib.ps3d_objx_write_mesh(h, ctypes.byref(info), *[_ptr(arrs[k]) for k in
                                                                           ("vertices", "normals", "tangents",
                                                                            "texcoords", "indices")]))
    finally:
        lib.ps3d_objx_close(h)


def load_vao(pipe, path: str, mesh: int = 0) -> int:
    """SceneObject::findOrCreateVao (test/scenobj.cpp:88-162) on a GPU
    pipeline: returns the new VAO."""
    lib = _lib()
    vao = ctypes.c_int()
    _check(lib, lib.ps3d_objx_load_vao(pipe.h, path.encode(), mesh, ctypes.byref(vao)))
    return vao.value
