"""The C-ABI library (no GPU needed): it builds for sm_103a, loads, exports
every entry point include/omv.h declares, its struct layouts match the Python
binding, and argument errors come back as status codes."""
import ctypes as C
import os
import re

import numpy as np
from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "omv.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(omv_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_every_declared_symbol(omv):
    omv.build()
    L = omv.lib()
    names = _declared()
    assert "omv_render" in names and "omv_scene_create" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layouts_match_binding(omv):
    capi = omv.capi
    L = omv.lib()
    n = L.omv_struct_sizes(None, 0)
    sizes = (C.c_int64 * n)()
    assert L.omv_struct_sizes(sizes, n) == n
    py = [capi.MeshDesc, capi.InstanceDesc, capi.MaterialDesc, capi.LightDesc, capi.HdriDesc, capi.SceneDesc,
          capi.SceneInfo, capi.Camera, capi.Params, capi.Stats, capi.Hit, capi.Job, capi.TextureDesc,
          capi.TextureRef, capi.AdjointJob]
    assert [C.sizeof(t) for t in py] == list(sizes)
    assert capi.HIT_DTYPE.itemsize == C.sizeof(capi.Hit)


def test_params_default_are_reference_defaults(omv):
    p = omv.capi.Params()
    omv.lib().omv_params_default(C.byref(p))
    q = omv.capi.default_params()
    for f, _ in omv.capi.Params._fields_:
        assert getattr(p, f) == getattr(q, f), f
    r = omv.RendererParameters()
    assert (r.cameraBouncesN, r.lightBouncesN, r.maxPathLength, r.samplesPerPixel) == (10, 10, 8, 20)


def test_argument_errors_are_status_codes(omv):
    L = omv.lib()
    h = C.c_void_p()
    assert L.omv_scene_create(None, 0, C.byref(h)) == 1  # OMV_ERR_INVALID_ARGUMENT
    assert b"NULL" in L.omv_last_error()
    assert L.omv_render(None, None, None, None, None, None, None, None) == 1
    assert L.omv_trace_rays(None, 1, None, None) == 1
    assert L.omv_scene_destroy(None) == 0


def test_no_device_is_reported_not_crashed(omv):
    import torch

    if torch.cuda.is_available():
        return
    out = np.zeros((1, 3), np.float32)
    x = np.zeros((1, 17), np.float32)
    st = omv.lib().omv_brdf_eval_direct(1, omv.capi.fptr(x), omv.capi.fptr(out))
    assert st != 0


def test_log_callback_sees_every_failure(omv):
    seen = []
    omv.set_log_callback(lambda status, msg: seen.append((status, msg)))
    try:
        L = omv.lib()
        assert L.omv_render(None, None, None, None, None, None, None, None) == 1
        assert L.omv_trace_rays(None, 1, None, None) == 1
        assert L.omv_scene_destroy(None) == 0  # success: not reported
    finally:
        omv.set_log_callback(None)
    assert [s for s, _ in seen] == [1, 1]
    assert all(m for _, m in seen)
    L.omv_render(None, None, None, None, None, None, None, None)
    assert len(seen) == 2  # removed
