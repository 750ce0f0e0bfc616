"""The C-ABI library builds, loads and exports every entry point include/pfcuda.h declares."""
import ctypes as C
import os
import re

from conftest import ROOT


def declared_functions():
    with open(os.path.join(ROOT, "include", "pfcuda.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(pf_\w+)\s*\(", text, re.M)))


def test_header_declares_the_abi():
    names = declared_functions()
    assert "pf_ctx_create" in names and "pf_render" in names and "pf_draw" in names
    assert len(names) >= 14


def test_library_exports_every_declared_symbol(pf):
    lib = pf.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) <= set(pf.EXPORTS) | {"pf_last_error"}


def test_abi_version(pf):
    assert pf.load().pf_abi_version() == 5


def test_null_arguments_are_rejected_without_a_device(pf):
    lib = pf.load()
    assert lib.pf_ctx_create(None, None) == 1
    assert lib.pf_scene_upload(None, None) == 1
    assert lib.pf_render(None, None) == 1
    assert lib.pf_ctx_destroy(None) == 0
    assert lib.pf_read_images_async(None, None, 0) == 1
    assert lib.pf_images_wait(None) == 1
    assert isinstance(lib.pf_last_error(None), bytes)
