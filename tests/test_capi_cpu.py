"""The C-ABI library builds for sm_103a, loads, exports every function that
include/collide_gpu.h declares, and its host-only helpers work without a GPU."""
import ctypes as C
import os
import re

import numpy as np

from inmyroom_vulkan_gb300 import build, capi

HEADER = os.path.join(build.ROOT, "include", "collide_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(cg_\w+)\s*\(", text, re.M)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(capi.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(build.build())
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_struct_sizes():
    assert C.sizeof(capi.cg_obb) == 48
    assert capi.QUERY_DTYPE.itemsize == 72
    assert capi.TRI_PAIR_DTYPE.itemsize == 36
    assert capi.LEAF_PAIR_DTYPE.itemsize == 16


def test_relative_matrix_is_bit_identical_to_reference_convention():
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "boxes.npz"))
    m = g["mats"]
    for i in range(64):
        got = capi.relative_matrix(m[i], m[(i * 7 + 3) % 64])
        assert np.array_equal(got.view(np.uint32), g["relative"][i].view(np.uint32))


def test_default_config_and_status_strings():
    cfg = capi.default_config()
    assert cfg.stack_entries & (cfg.stack_entries - 1) == 0
    lib = capi.load_library()
    lib.cg_status_string.restype = C.c_char_p
    assert lib.cg_status_string(0) == b"ok"
    assert lib.cg_status_string(-6) == b"device wait timed out"
