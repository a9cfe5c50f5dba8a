"""The C ABI: the library loads without a GPU, exports every symbol the
header declares, and rejects bad calls with status codes, not crashes."""

import ctypes
import os
import re

import numpy as np
import pytest

from raymond_gb300 import _native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "raymond.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(raymond_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    # and the ctypes table covers them all
    assert set(names) <= set(_native.SIGNATURES)


def test_null_handles_are_rejected():
    lib = _native.lib()
    assert lib.raymond_render(None, None, 0, 0) == _native.EINVAL
    assert lib.raymond_sync(None) == _native.EINVAL
    assert lib.raymond_resize(None, 4, 4) == _native.EINVAL
    assert lib.raymond_read_pixels(None, None, 0, 0, 1) == _native.EINVAL
    lib.raymond_destroy(None)


def test_bvh_builder_rejects_bad_arguments():
    lib = _native.lib()
    nodes = np.zeros(8, dtype=np.uint32)
    order = np.zeros(1, dtype=np.uint32)
    mins = np.zeros(3)
    assert lib.raymond_bvh_build(_native.ptr(mins), _native.ptr(mins), 1, 0, _native.ptr(nodes), _native.ptr(order), 1) == 0
    assert lib.raymond_bvh_build(None, None, 1, 4, _native.ptr(nodes), _native.ptr(order), 1) == 0
    assert lib.raymond_bvh_build(None, None, 0, 4, _native.ptr(nodes), _native.ptr(order), 1) == 1


def test_create_without_gpu_reports_an_error():
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is present")
    lib = _native.lib()
    h = ctypes.c_void_p()
    cfg = _native.Config(device=0)
    rc = lib.raymond_create(ctypes.byref(h), ctypes.byref(cfg))
    assert rc != _native.OK
    assert lib.raymond_last_error(None)
