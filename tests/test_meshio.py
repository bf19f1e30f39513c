"""Mesh files (PLY / OBJ / STL readers, PLY writer) and map files (save / load of the built tree).

The readers stand in for Assimp in rmagine's import_embree_map (EmbreeMap.hpp:94-117).  Files
are written here by independent numpy writers; the reader must return exactly the arrays that
were written (polygons as triangle fans).  Map files are checked to round-trip bit for bit and
to reject damaged or crafted content before anything reaches the device."""
import ctypes as C
import struct

import numpy as np
import pytest

from rmagine_gb300 import scenes

F32 = np.float32


def fan(polys):
    out = []
    for p in polys:
        for k in range(1, len(p) - 1):
            out.append((p[0], p[k], p[k + 1]))
    return np.array(out, np.uint32)


def mesh_with_quads():
    rng = np.random.default_rng(0)
    v = rng.uniform(-5, 5, (9, 3)).astype(F32)
    polys = [(0, 1, 2), (2, 3, 4, 5), (5, 6, 7, 8, 0), (1, 3, 6)]
    return v, polys


def ply_binary(path, v, polys, big=False, double=False, extra=True):
    e = ">" if big else "<"
    hdr = ["ply", f"format binary_{'big' if big else 'little'}_endian 1.0", "comment written by the test",
           f"element vertex {len(v)}"]
    t = "double" if double else "float"
    hdr += [f"property {t} x", f"property {t} y", f"property {t} z"]
    if extra:
        hdr += ["property float nx", "property uchar red"]
    hdr += [f"element face {len(polys)}", "property list uchar int vertex_indices"]
    if extra:
        hdr += ["property int flags", "element edge 1", "property list ushort int edge_vertices"]
    hdr += ["end_header"]
    body = bytearray()
    for p in v:
        body += struct.pack(e + ("ddd" if double else "fff"), *[float(x) for x in p])
        if extra:
            body += struct.pack(e + "fB", 0.5, 7)
    for poly in polys:
        body += struct.pack(e + "B" + "i" * len(poly), len(poly), *poly)
        if extra:
            body += struct.pack(e + "i", 3)
    if extra:
        body += struct.pack(e + "Hii", 2, 0, 1)
    path.write_bytes(("\n".join(hdr) + "\n").encode() + bytes(body))


def ply_ascii(path, v, polys):
    lines = ["ply", "format ascii 1.0", f"element vertex {len(v)}", "property float x", "property float y",
             "property float z", "property uchar green", f"element face {len(polys)}",
             "property list uchar uint vertex_index", "end_header"]
    lines += [f"{repr(float(p[0]))} {repr(float(p[1]))} {repr(float(p[2]))} 12" for p in v]
    lines += [f"{len(q)} " + " ".join(str(i) for i in q) for q in polys]
    path.write_text("\n".join(lines) + "\n")


# ---- CPU: mesh readers -------------------------------------------------------------------
@pytest.mark.parametrize("big,double", [(False, False), (True, False), (False, True), (True, True)])
def test_binary_ply(built, tmp_path, big, double):
    from rmagine_gb300 import meshio

    v, polys = mesh_with_quads()
    p = tmp_path / "m.ply"
    ply_binary(p, v, polys, big=big, double=double)
    rv, rf, rg = meshio.read_mesh(p)
    assert np.array_equal(rv, v) and np.array_equal(rf, fan(polys)) and np.all(rg == 0)


def test_ascii_ply_and_writer_round_trip(built, tmp_path):
    from rmagine_gb300 import meshio

    v, polys = mesh_with_quads()
    p = tmp_path / "a.PLY"
    ply_ascii(p, v, polys)
    rv, rf, _ = meshio.read_mesh(p)
    assert np.array_equal(rv, v) and np.array_equal(rf, fan(polys))
    sc = scenes.box_room(seed=1, n_boxes=20)
    q = tmp_path / "w.ply"
    meshio.write_ply(q, sc.vertices, sc.faces)
    wv, wf, _ = meshio.read_mesh(q)
    assert np.array_equal(wv, sc.vertices) and np.array_equal(wf, sc.faces)


def test_obj_groups_negative_indices_and_slashes(built, tmp_path):
    from rmagine_gb300 import meshio

    v, polys = mesh_with_quads()
    lines = ["# comment", "mtllib none.mtl", "o first"]
    lines += [f"v {float(p[0])!r} {float(p[1])!r} {float(p[2])!r}" for p in v[:6]]
    lines += ["vt 0 0", "vn 0 0 1", "f 1/1/1 2/1/1 3/1/1", "f 3//1 4//1 5//1 6//1", "g second", "s off"]
    lines += [f"v {float(p[0])!r} {float(p[1])!r} {float(p[2])!r}" for p in v[6:]]
    lines += ["f -4 -3 -2 -1 1", "usemtl x", "f 2/1 4/1 7/1"]
    p = tmp_path / "m.obj"
    p.write_text("\n".join(lines) + "\n")
    rv, rf, rg = meshio.read_mesh(p)
    assert np.array_equal(rv, v)
    assert np.array_equal(rf, fan(polys))
    assert list(rg) == [0, 0, 0, 1, 1, 1, 1]


def test_stl_binary_and_ascii(built, tmp_path):
    from rmagine_gb300 import meshio

    v, f = scenes.gen_cube()
    tri = v[f]
    b = bytearray(b"\0" * 80) + struct.pack("<I", len(f))
    for t in tri:
        b += struct.pack("<3f", 0, 0, 0) + struct.pack("<9f", *t.reshape(-1)) + b"\0\0"
    (tmp_path / "b.stl").write_bytes(bytes(b))
    rv, rf, _ = meshio.read_mesh(tmp_path / "b.stl")
    assert np.array_equal(rv, tri.reshape(-1, 3)) and np.array_equal(rf, np.arange(36, dtype=np.uint32).reshape(-1, 3))
    lines = ["solid cube"]
    for t in tri:
        lines += ["facet normal 0 0 0", "outer loop"] + [f"vertex {float(x)!r} {float(y)!r} {float(z)!r}" for x, y, z in t] + \
                 ["endloop", "endfacet"]
    lines += ["endsolid cube"]
    (tmp_path / "a.stl").write_text("\n".join(lines) + "\n")
    av, af, _ = meshio.read_mesh(tmp_path / "a.stl")
    assert np.array_equal(av, rv) and np.array_equal(af, rf)


def test_malformed_files_are_rejected(built, tmp_path):
    from rmagine_gb300 import _lib, meshio

    v, polys = mesh_with_quads()
    p = tmp_path / "t.ply"
    ply_binary(p, v, polys, extra=False)
    data = p.read_bytes()
    (tmp_path / "trunc.ply").write_bytes(data[:-7])
    bad_idx = [(0, 1, 99)]
    ply_binary(tmp_path / "idx.ply", v, bad_idx, extra=False)
    (tmp_path / "f.obj").write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    (tmp_path / "x.off").write_text("OFF\n")
    for name, code in (("trunc.ply", _lib.RMG_ERR_INVALID_ARG), ("idx.ply", _lib.RMG_ERR_INVALID_ARG),
                       ("f.obj", _lib.RMG_ERR_INVALID_ARG), ("x.off", _lib.RMG_ERR_UNSUPPORTED),
                       ("missing.ply", _lib.RMG_ERR_INVALID_ARG)):
        with pytest.raises(_lib.RmgError) as e:
            meshio.read_mesh(tmp_path / name)
        assert e.value.status == code, name


# ---- CPU: map-file validation (no device work happens before the checks) ----------------
def map_file(nodes, tris, faces, verts, order, parents, depth=1, corrupt_sum=False):
    payload = verts.astype(F32).tobytes() + faces.astype(np.uint32).tobytes() + nodes.tobytes() + \
        tris.tobytes() + order.astype(np.uint32).tobytes() + parents.astype(np.int32).tobytes()
    h = 1469598103934665603
    for byte in payload:
        h = ((h ^ byte) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    if corrupt_sum:
        h ^= 1
    hdr = b"RMGLBVH1" + struct.pack("<IIIIIIQQ", 1, len(verts), len(faces), len(nodes), depth, 0, len(payload), h)
    return hdr + payload


def two_triangle_tree(child=(-1, -2)):
    verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], F32)
    faces = np.array([[0, 1, 2], [1, 3, 2]], np.uint32)
    node = np.zeros(16, np.float32)
    node[:12] = [0, 1, 0, 1, 0, 1, 0, 1, 0, 0, 0, 0]  # both children: x, y in [0, 1], z = 0
    links = np.array([child[0], child[1], -1, 0], np.int32)
    node[12:] = links.view(np.float32)
    tris = np.zeros((2, 12), np.float32)
    tris[0, :3], tris[0, 4:7], tris[0, 8:11] = verts[0], verts[1], verts[2]
    tris[1, :3], tris[1, 4:7], tris[1, 8:11] = verts[1], verts[3], verts[2]
    tris[:, 3] = np.array([0, 1], np.uint32).view(np.float32)
    return node[None], tris, faces, verts, np.array([0, 1]), np.array([0, 0])


@pytest.mark.parametrize("damage", ["checksum", "child", "truncated", "magic", "face"])
def test_damaged_map_files_are_rejected_on_the_host(built, tmp_path, damage):
    from rmagine_gb300 import _lib, meshio

    nodes, tris, faces, verts, order, parents = two_triangle_tree()
    if damage == "child":
        nodes, tris, faces, verts, order, parents = two_triangle_tree(child=(-1, -7))  # leaf 6 of 2
    if damage == "face":
        faces = faces.copy()
        faces[1, 2] = 9
    data = map_file(nodes, tris, faces, verts, order, parents, corrupt_sum=damage == "checksum")
    if damage == "truncated":
        data = data[:-3]
    if damage == "magic":
        data = b"RMGLBVH9" + data[8:]
    p = tmp_path / "m.rmgmap"
    p.write_bytes(data)
    with pytest.raises(_lib.RmgError) as e:
        meshio.load_map(p)
    assert e.value.status == _lib.RMG_ERR_INVALID_ARG


# ---- GPU ---------------------------------------------------------------------------------
@pytest.mark.gpu
def test_map_save_load_round_trip(built, tmp_path):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    sc = scenes.terrain(grid=128, n_boxes=100, seed=2, size=80.0)
    m = rm.Map(sc.vertices, sc.faces)
    p = tmp_path / "t.rmgmap"
    m.save(p)
    m2 = rm.Map.load(p)
    assert m2.info() == m.info()
    a, b = m.export(), m2.export()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    model = rm.vlp16_900()
    poses = torch.from_numpy(scenes.terrain_poses(sc, 4, seed=3, size=80.0)).cuda()
    r1 = rm.make_simulator(model, m).simulate(poses)
    r2 = rm.make_simulator(model, m2).simulate(poses)
    for k, t in r1.tensors().items():
        assert torch.equal(torch.nan_to_num(t.float(), 7.0), torch.nan_to_num(getattr(r2, k).float(), 7.0)), k
    # the saved map is a valid tree for the loader's checks, and a refit works on it
    m2.refit(sc.vertices)
    assert m2.status() == 0


@pytest.mark.gpu
def test_import_map_of_a_grouped_obj_is_a_scene(built, tmp_path):
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import meshio

    torch.cuda.set_device(0)
    room = scenes.box_room(seed=3, n_boxes=5, half=4.0)
    bv, bf = scenes.box_mesh([1, 1, 0], [2, 2, 1])
    lines = ["o room"] + [f"v {float(x)!r} {float(y)!r} {float(z)!r}" for x, y, z in room.vertices]
    lines += [f"f {a + 1} {b + 1} {c + 1}" for a, b, c in room.faces]
    off = len(room.vertices)
    lines += ["o box"] + [f"v {float(x)!r} {float(y)!r} {float(z)!r}" for x, y, z in bv]
    lines += [f"f {a + 1 + off} {b + 1 + off} {c + 1 + off}" for a, b, c in bf]
    p = tmp_path / "two.obj"
    p.write_text("\n".join(lines) + "\n")
    imp = meshio.import_map(p)
    assert isinstance(imp, rm.Scene) and len(imp.geometries) == 2
    ref = rm.Scene.from_meshes([(room.vertices, room.faces), (bv, bf)])
    model = rm.vlp16_900()
    poses = torch.from_numpy(scenes.room_poses(3, seed=2, half=4.0)).cuda()
    a = rm.make_simulator(model, imp).simulate(poses)
    b = rm.make_simulator(model, ref).simulate(poses)
    for k, t in a.tensors().items():
        assert torch.equal(torch.nan_to_num(t.float(), 7.0), torch.nan_to_num(getattr(b, k).float(), 7.0)), k
    single = tmp_path / "room.ply"
    meshio.write_ply(single, room.vertices, room.faces)
    assert isinstance(meshio.import_map(single), rm.Map)


@pytest.mark.gpu
def test_hand_written_map_file_loads_and_traces(built, tmp_path):
    """The file format written independently (two triangles under one node) loads and gives the
    known answer of a downward ray."""
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import meshio

    torch.cuda.set_device(0)
    p = tmp_path / "two.rmgmap"
    p.write_bytes(map_file(*two_triangle_tree()))
    m = meshio.load_map(p)
    assert m.info()["n_faces"] == 2 and m.info()["depth"] == 1
    model = rm.OnDnModel(width=2, height=1, range=rm.Interval(0.0, 10.0),
                         origs=np.array([[0.25, 0.25, 1.0], [0.75, 0.75, 1.0]], F32),
                         dirs=np.array([[0, 0, -1], [0, 0, -1]], F32))
    r = rm.make_simulator(model, m).simulate(torch.from_numpy(np.array([[0, 0, 0, 1, 0, 0, 0, 0]], F32)).cuda())
    assert r.ranges.cpu().tolist() == [1.0, 1.0]
    assert r.face_ids.cpu().tolist() == [0, 1]
