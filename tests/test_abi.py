"""The C ABI library loads (CPU-only here) and exports every entry point
include/vrg.h declares; host-only entry points behave as documented."""
import ctypes as C
import os
import re

import numpy as np

import vrg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "vrg.h")).read()
    return sorted(set(re.findall(r"VRG_API\s+[\w\s\*]+?\b(vrg_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    assert "vrg_render" in names and "vrg_scene_commit" in names and len(names) >= 30


def test_library_exports_every_declared_symbol(vrglib):
    lib = vrglib.load_library()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_signatures_cover_header(vrglib):
    bound = {n for n, _, _ in vrglib.SIGNATURES}
    extra = {"vrg_build_tl_bvh_noalloc"}  # bound where used
    assert set(_declared()) - bound <= extra


def test_no_device_is_reported(vrglib):
    import torch
    if torch.cuda.is_available():
        return
    h = C.c_void_p()
    lib = vrglib.load_library()
    st = lib.vrg_context_create(None, C.byref(h))
    assert st == vrglib.ERR_NO_DEVICE
    assert lib.vrg_status_string(st) == b"no cuda device"
    assert b"no CUDA device" in lib.vrg_last_error()


def test_null_arguments_rejected(vrglib):
    lib = vrglib.load_library()
    assert lib.vrg_scene_commit(None) == vrglib.ERR_INVALID_ARGUMENT
    assert lib.vrg_render(None, None, None, None, None, None) == vrglib.ERR_INVALID_ARGUMENT
    assert lib.vrg_material_table_set(None, None, 5) == vrglib.ERR_INVALID_ARGUMENT


def test_oracle_library_loads(orc):
    assert orc.lib().orc_mm_combine(0, 0) == 0xe6546b64


def test_struct_layouts(vrglib):
    assert C.sizeof(vrglib.BvhNode) == 40
    assert C.sizeof(vrglib.Material) == 48
    assert C.sizeof(vrglib.Camera) == 56
    assert C.sizeof(vrglib.RenderParams) == 64
