"""rmg_lbvh_build_noalloc: the LBVH build for callers that cannot allocate device memory.

Such callers (real-time loops that forbid allocator calls once they run,
hosts that hand the library one fixed device arena and own the rest) pass the
mesh and the output buffers in device memory; the build's temporary data lives
in a fixed array inside the library.  Its trees must equal, bit for bit, the trees
of the allocating rmg_map_build -- on consecutive calls, since the calls
share (and do not reset) that array.

Named test_zz_* so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import rmagine_gb300 as rm
from rmagine_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    torch.cuda.set_device(0)


def build_noalloc(v: np.ndarray, f: np.ndarray, stream=None):
    """Calls the C entry point with torch-owned device buffers (the test plays the caller), on
    `stream` (a torch.cuda.Stream) or torch's current stream."""
    n = f.shape[0]
    nn = max(n - 1, 1)
    vd = torch.from_numpy(np.ascontiguousarray(v, np.float32)).cuda()
    fd = torch.from_numpy(np.ascontiguousarray(f, np.uint32).view(np.int32)).cuda()
    nodes = torch.full((nn, 16), -7.0, dtype=torch.float32, device="cuda")
    tris = torch.full((n, 12), -7.0, dtype=torch.float32, device="cuda")
    order = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    parent = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    flags = torch.full((nn,), 7, dtype=torch.int32, device="cuda")  # the call must clear these
    bufs = _lib.LbvhBuffersC(nodes.data_ptr(), tris.data_ptr(), order.data_ptr(), parent.data_ptr(),
                             flags.data_ptr())
    s_ = stream or torch.cuda.current_stream()
    s_.wait_stream(torch.cuda.current_stream())  # the buffers' fills come first
    st = _lib.load().rmg_lbvh_build_noalloc(C.c_void_p(vd.data_ptr()), v.shape[0], C.c_void_p(fd.data_ptr()), n,
                                            C.byref(bufs), C.c_void_p(s_.cuda_stream))
    torch.cuda.synchronize()
    nodes_h = nodes.cpu().numpy()
    return st, {"boxes": nodes_h[:, :12], "links": nodes_h.view(np.int32)[:, 12:], "tris": tris.cpu().numpy(),
                "leaf_order": order.cpu().numpy().view(np.uint32)}


def same(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


def meshes():
    room = scenes.box_room(seed=0, n_boxes=200)
    ter = scenes.terrain(grid=96, n_boxes=100, seed=3)
    tri = (np.array([[2, -1, -1], [2, 1, -1], [2, 0, 1]], np.float32), np.array([[0, 1, 2]], np.uint32))
    return [("room", room.vertices, room.faces), ("terrain", ter.vertices, ter.faces), ("one", *tri),
            ("room again", room.vertices, room.faces)]


def test_noalloc_build_equals_map_build_on_consecutive_calls():
    for name, v, f in meshes():
        st, got = build_noalloc(v, f)
        assert st == _lib.RMG_OK, (name, _lib.load().rmg_last_error())
        want = rm.Map(v, f, builder="lbvh").export()
        assert same(got["leaf_order"], want["leaf_order"]), name
        assert same(got["links"], want["links"]), name
        assert same(got["boxes"], want["boxes"]), name
        assert same(got["tris"], want["tris"]), name


def test_noalloc_rejects_meshes_beyond_the_limit():
    n = _lib.RMG_NOALLOC_MAX_FACES + 1
    v = np.zeros((3, 3), np.float32)
    f = np.zeros((n, 3), np.uint32)
    st, _ = build_noalloc(v, f)
    assert st == _lib.RMG_ERR_INVALID_ARG
    assert b"RMG_NOALLOC_MAX_FACES" in _lib.load().rmg_last_error()


def test_noalloc_rejects_out_of_range_face_indices():
    v, f = scenes.gen_cube()
    f = f.copy()
    f[5, 1] = 8  # one past the last vertex
    st, _ = build_noalloc(v, f)
    assert st == _lib.RMG_ERR_INVALID_ARG
    # and the next valid call is unaffected
    v, f = scenes.gen_cube()
    st, got = build_noalloc(v, f)
    assert st == _lib.RMG_OK
    assert same(got["links"], rm.Map(v, f, builder="lbvh").export()["links"])


def heightfield(nx: int, ny: int, seed: int = 0):
    """A (nx-1) x (ny-1) grid of quads, two triangles each, with random heights."""
    rng = np.random.default_rng(seed)
    xs, ys = np.meshgrid(np.arange(nx, dtype=np.float32), np.arange(ny, dtype=np.float32), indexing="xy")
    v = np.stack([xs.ravel() * 0.5, ys.ravel() * 0.5, rng.uniform(0, 2, nx * ny).astype(np.float32)], 1)
    i = np.arange(ny - 1)[:, None] * nx + np.arange(nx - 1)[None, :]
    i = i.ravel().astype(np.uint32)
    f = np.concatenate([np.stack([i, i + 1, i + nx], 1), np.stack([i + 1, i + nx + 1, i + nx], 1)])
    return v.astype(np.float32), f.astype(np.uint32)


def test_noalloc_at_the_face_limit_and_on_a_side_stream():
    # 128 x 256 quads = exactly RMG_NOALLOC_MAX_FACES triangles: keys, values, bounds and the sort's
    # temporary storage must all fit the fixed array
    v, f = heightfield(129, 257)
    assert f.shape[0] == _lib.RMG_NOALLOC_MAX_FACES
    want = rm.Map(v, f, builder="lbvh").export()
    side = torch.cuda.Stream()
    for stream in (None, side, side):
        st, got = build_noalloc(v, f, stream)
        assert st == _lib.RMG_OK, _lib.load().rmg_last_error()
        for k in ("leaf_order", "links", "boxes", "tris"):
            assert same(got[k], want[k]), k
