"""The allocation-free confocal forward, totri_mesh_confocal_forward_noalloc.

It serves callers that cannot allocate device memory (hosts that own all
device memory through a fixed pool, allocation-free latency loops, and
foreign-language hosts that bind only the C ABI); its scratch is a static
24 MiB array inside the library. These tests call it through the C ABI and
compare it with totri_mesh_confocal_forward, which takes a caller workspace,
on two calls in a row (a full-size scene, then a small one, so the second call
starts from the first call's leftovers), and check that an input needing more
scratch than the array holds is refused. This file is collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from totri_gb300 import _lib, scenes
from totri_gb300.totri_cpp import render as R

pytestmark = pytest.mark.gpu

TOL = 1e-6  # shared-memory atomics add in a run-dependent order


def _entry_point(lib):
    fn = lib.totri_mesh_confocal_forward_noalloc
    fn.argtypes = [ctypes.POINTER(_lib.Array)] * 6 + [ctypes.c_float, ctypes.c_float,
                                                      ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_noalloc_matches_workspace_entry_point_twice(cuda_lib):
    fn = _entry_point(cuda_lib)
    for s in (scenes.confocal_differentiable(), scenes.confocal_small(seed=12)):
        bd = s["bin_def"]
        verts, faces = s["verts"].cuda(), s["faces"].cuda()
        colors, sp = s["colors"].cuda(), s["scan_points"].cuda()
        origin = torch.empty_like(sp[:, :0])
        S = sp.shape[1]
        expect = torch.empty((1, bd.num, S), device="cuda")
        R.mesh_confocal_forward(verts, faces, colors, sp, origin, expect, bd.width, bd.offset, 0)
        got = torch.full((1, bd.num, S), float("nan"), device="cuda")
        st = fn(_lib.array(verts), _lib.array(faces), _lib.array(colors), _lib.array(sp),
                _lib.array(origin), _lib.array(got), bd.width, bd.offset, 0,
                _lib.stream_of(got.device))
        assert st == 0, cuda_lib.totri_last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        assert _rel(got, expect) < TOL


def test_noalloc_refuses_inputs_beyond_its_scratch(cuda_lib):
    fn = _entry_point(cuda_lib)
    verts = torch.zeros((1, 64, 3), device="cuda")
    faces = torch.zeros((1, 20480, 3), dtype=torch.int32, device="cuda")
    colors = torch.zeros((1, 64, 0), device="cuda")
    sp = torch.zeros((1, 16384, 3), device="cuda")
    out = torch.zeros((1, 8, 16384), device="cuda")
    # the refusal rests on this input's scratch exceeding the 24 MiB array
    assert cuda_lib.totri_mesh_workspace(1, 64, 20480, 16384) > (24 << 20)
    st = fn(_lib.array(verts), _lib.array(faces), _lib.array(colors), _lib.array(sp),
            _lib.array(sp[:, :0]), _lib.array(out), 0.01, 0.0, 0, _lib.stream_of(out.device))
    assert st == _lib.TOTRI_ERR_WORKSPACE
    assert b"static scratch" in cuda_lib.totri_last_error()
