"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every entry point include/ddgi.h declares; host-side argument validation
runs without touching the device."""
import ctypes as C
import os
import re

import pytest

from vulkanexp_gb300 import abi, build, ddgi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(ddgi_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return C.CDLL(path)


def test_header_declares_core_entry_points():
    names = declared_functions("ddgi.h")
    for n in ("ddgi_create", "ddgi_destroy", "ddgi_scene_build", "ddgi_update", "ddgi_get_atlas", "ddgi_set_light"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions("ddgi.h"):
        assert hasattr(lib, name), "missing export %s" % name


def test_python_binding_covers_header():
    bound = set(ddgi.exported_symbols())
    for name in declared_functions("ddgi.h"):
        assert name in bound, "binding lacks %s" % name


def test_status_strings(lib):
    lib.ddgi_status_string.restype = C.c_char_p
    assert lib.ddgi_status_string(0) == b"DDGI_OK"
    assert lib.ddgi_status_string(5) == b"DDGI_ERR_TIMEOUT"


@pytest.mark.parametrize("field,value", [
    ("resolution", (1, 4, 4)),
    ("rays_per_probe", 0),
    ("rays_per_probe", 4096),
    ("color_res", 2),
    ("precision", 9),
])
def test_create_rejects_bad_grid_without_gpu(lib, field, value):
    g = abi.make_grid((0, 0, 0), (1, 1, 1), (4, 4, 4), 64)
    if isinstance(value, tuple):
        getattr(g, field)[:] = value
    else:
        setattr(g, field, value)
    h = C.c_void_p()
    lib.ddgi_create.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(C.c_void_p)]
    assert lib.ddgi_create(C.byref(g), C.byref(h)) == 1
    assert not h.value


def test_create_rejects_more_rays_than_32_bit_indices(lib):
    # 2^24 probes (the probe limit) x 1024 rays: 2^34 rays in one update,
    # beyond DDGI_MAX_RAYS_PER_UPDATE; 2^24 x 64 rays is accepted by the check
    g = abi.make_grid((0, 0, 0), (1, 1, 1), (256, 256, 256), 1024)
    h = C.c_void_p()
    lib.ddgi_create.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(C.c_void_p)]
    assert lib.ddgi_create(C.byref(g), C.byref(h)) == 1
    assert not h.value
    assert 256 ** 3 * 1024 > 0xFFF00000 >= 256 ** 3 * 64


@pytest.mark.parametrize("color_res,depth_res", [(16, 8), (8, 17)])
def test_create_rejects_atlases_beyond_32_bit_texel_indices(lib, color_res, depth_res):
    # 2^24 probes with 16 x 16 colour tiles: 2^32 texels, one more than the
    # lookups' 32-bit texel indices reach (15 x 15 tiles would be accepted)
    g = abi.make_grid((0, 0, 0), (1, 1, 1), (256, 256, 256), 1, color_res=color_res, depth_res=depth_res)
    h = C.c_void_p()
    lib.ddgi_create.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(C.c_void_p)]
    assert lib.ddgi_create(C.byref(g), C.byref(h)) == 1
    assert not h.value


def test_create_rejects_empty_extent(lib):
    g = abi.make_grid((0, 0, 0), (1, 0, 1), (4, 4, 4), 64)
    h = C.c_void_p()
    lib.ddgi_create.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(C.c_void_p)]
    assert lib.ddgi_create(C.byref(g), C.byref(h)) == 1
