"""The C ABI: the library loads without a GPU and exports every symbol include/*.h declares."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(rmg_\w+)\s*\(", text, flags=re.M):
            if not m.group(0).lstrip().startswith("typedef"):
                names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("rmg_map_build", "rmg_sensor_create", "rmg_simulate", "rmg_status_string"):
        assert n in names
    assert all(n.startswith("rmg_") for n in names)


def test_library_exports_every_declared_symbol(built):
    from rmagine_gb300 import _lib

    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header(built):
    from rmagine_gb300 import _lib

    assert declared_functions() == set(_lib.SIGNATURES), (
        declared_functions() ^ set(_lib.SIGNATURES))


def test_status_strings_and_version(built):
    from rmagine_gb300 import _lib

    lib = _lib.load()
    assert lib.rmg_abi_version() == 1
    for code in range(0, 8):
        s = lib.rmg_status_string(code).decode()
        assert s and s != "unknown status"
    assert lib.rmg_status_string(99).decode() == "unknown status"


def test_invalid_arguments_fail_without_touching_the_gpu(built):
    """Argument checks run before any CUDA call, so they work on a machine without a GPU."""
    from rmagine_gb300 import _lib

    lib = _lib.load()
    out = ctypes.c_void_p()
    assert lib.rmg_map_build(None, 0, None, 0, None, None) == _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_sensor_create(None, None, ctypes.byref(out)) == _lib.RMG_ERR_INVALID_ARG
    m = _lib.ModelC()
    m.kind = 9
    assert lib.rmg_sensor_create(ctypes.byref(m), None, ctypes.byref(out)) == _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_simulate(None, None, None, None, 1, None, None) == _lib.RMG_ERR_INVALID_ARG
    assert b"NULL" in lib.rmg_last_error()
    # a face index outside the vertex array is rejected on the host
    import numpy as np

    v = np.zeros((3, 3), np.float32)
    f = np.array([[0, 1, 5]], np.uint32)
    st = lib.rmg_map_build(v.ctypes.data_as(ctypes.c_void_p), 3, f.ctypes.data_as(ctypes.c_void_p), 1, None,
                           ctypes.byref(out))
    assert st == _lib.RMG_ERR_INVALID_ARG
    # an unknown tree builder is rejected before any device work
    st = lib.rmg_map_build_ex(v.ctypes.data_as(ctypes.c_void_p), 3, f.ctypes.data_as(ctypes.c_void_p), 1, 7, None,
                              ctypes.byref(out))
    assert st == _lib.RMG_ERR_UNSUPPORTED
    assert lib.rmg_host_set_pipeline(0, 9) == _lib.RMG_ERR_UNSUPPORTED
    assert lib.rmg_host_set_pipeline(0, 0) == _lib.RMG_OK
    # the sensor queries reject a NULL sensor or output
    flag = ctypes.c_int(7)
    assert lib.rmg_sensor_visit_order(None, None, ctypes.byref(flag)) == _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_sensor_visit_order(None, None, None) == _lib.RMG_ERR_INVALID_ARG
    w, h = ctypes.c_uint32(), ctypes.c_uint32()
    assert lib.rmg_sensor_size(None, ctypes.byref(w), ctypes.byref(h)) == _lib.RMG_ERR_INVALID_ARG
