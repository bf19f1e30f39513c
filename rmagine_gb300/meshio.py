"""Mesh and map files (rmg_mesh_read / rmg_mesh_write_ply / rmg_map_save / rmg_map_load).

    import_map(path)   -- rmagine's import_embree_map / import_optix_map (EmbreeMap.hpp:94-117):
                          a single-mesh file gives a Map; an OBJ with several objects / groups
                          gives a Scene with one identity instance per group (geom_id =
                          object_id = group index), what EmbreeScene::freeze leaves of a file
                          whose meshes are not instanced.
    read_mesh(path)    -- vertices [N,3] float32, faces [M,3] uint32, face groups [M] uint32.
    write_ply(path, vertices, faces)
    save_map(map, path) / load_map(path) -- the built tree without a rebuild.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L
from .simulation import Instance, Map, Scene, _stream_ptr


def _path(p) -> bytes:
    return os.fsencode(os.fspath(p))


def read_mesh(path):
    m = L.MeshC()
    L.call("rmg_mesh_read", _path(path), C.byref(m))
    try:
        v = np.ctypeslib.as_array(C.cast(m.vertices, C.POINTER(C.c_float)), (m.n_vertices * 3,)).reshape(-1, 3).copy() \
            if m.n_vertices else np.zeros((0, 3), np.float32)
        f = np.ctypeslib.as_array(C.cast(m.faces, C.POINTER(C.c_uint32)), (m.n_faces * 3,)).reshape(-1, 3).copy() \
            if m.n_faces else np.zeros((0, 3), np.uint32)
        g = np.ctypeslib.as_array(C.cast(m.face_group, C.POINTER(C.c_uint32)), (m.n_faces,)).copy() \
            if m.n_faces else np.zeros(0, np.uint32)
    finally:
        L.load().rmg_mesh_free(C.byref(m))
    return v, f, g


def write_ply(path, vertices, faces) -> None:
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
    L.call("rmg_mesh_write_ply", _path(path), v.ctypes.data_as(C.c_void_p), v.shape[0],
           f.ctypes.data_as(C.c_void_p), f.shape[0])


def split_groups(vertices, faces, groups):
    """One (vertices, faces) mesh per group, each with only the vertices it uses."""
    out = []
    for gi in np.unique(groups):
        fg = faces[groups == gi]
        used, inv = np.unique(fg.reshape(-1), return_inverse=True)
        out.append((vertices[used].astype(np.float32), inv.reshape(-1, 3).astype(np.uint32)))
    return out


def import_map(path):
    v, f, g = read_mesh(path)
    if f.shape[0] == 0 or np.all(g == g[0]):
        return Map(v, f)
    meshes = split_groups(v, f, g)
    return Scene([Map(mv, mf) for mv, mf in meshes],
                 [Instance(i, geom_id=i, object_id=i) for i in range(len(meshes))])


def save_map(m: Map, path) -> None:
    L.call("rmg_map_save", m.handle, _path(path))


def load_map(path) -> Map:
    import torch

    h = C.c_void_p()
    L.call("rmg_map_load", _path(path), _stream_ptr() if torch.cuda.is_available() else None, C.byref(h))
    m = Map.__new__(Map)
    m._h = h
    inf = m.info()
    m.n_vertices, m.n_faces = inf["n_vertices"], inf["n_faces"]
    return m
