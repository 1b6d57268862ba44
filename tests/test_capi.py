"""The C ABI on the CPU: the library builds, loads, exports every entry point
declared in include/totri_gb300.h, and rejects malformed arguments before any
device work (no GPU needed: these calls fail validation first)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from totri_gb300 import build, _lib
    build.build()
    return _lib.load()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "totri_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(totri_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_entry_point(lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_workspace_query(lib):
    assert b"sm_103a" in lib.totri_version()
    n = lib.totri_mesh_workspace(1, 10242, 20480, 4096)
    assert 10 << 20 < n < 32 << 20
    assert lib.totri_mesh_workspace(1, 10, 0, 16) == 0


def test_exhaustive_grad_scratch_query(lib):
    """The exhaustive gradient's optional bins-last scratch: all scan points
    when they fit 2 GiB, else whole 256-point tiles of them (or fewer points
    when a tile does not fit), and none when one scan point's lasers x bins
    exceed 2 GiB."""
    assert lib.totri_mesh_exhaustive_grad_scratch(36, 9, 300) == 36 * 9 * 300 * 4 + 64  # aligned
    assert lib.totri_mesh_exhaustive_grad_scratch(1024, 256, 2048) == 1024 * 256 * 2048 * 4
    assert lib.totri_mesh_exhaustive_grad_scratch(4096, 256, 2048) == 1024 * 256 * 2048 * 4
    assert lib.totri_mesh_exhaustive_grad_scratch(4096, 1000, 4096) == 131 * 1000 * 4096 * 4
    assert lib.totri_mesh_exhaustive_grad_scratch(10, 200000, 4096) == 0
    assert lib.totri_mesh_exhaustive_grad_scratch(0, 9, 300) == 0


def _arr(shape, dtype=0, ptr=0x10000):
    from totri_gb300 import _lib
    a = _lib.Array()
    a.data = ptr
    a.dtype = dtype
    a.ndim = len(shape)
    stride = 1
    for i in reversed(range(len(shape))):
        a.shape[i] = shape[i]
        a.strides[i] = stride
        stride *= shape[i]
    return a


def test_mesh_forward_rejects_bad_shapes(lib):
    from totri_gb300 import _lib
    verts = _arr((1, 10, 3))
    faces = _arr((1, 4, 3), dtype=2)
    mat = _arr((1, 10, 0))
    sp = _arr((1, 16, 3))
    so = _arr((1, 0, 3))
    bad_tr = _arr((1, 32, 15))  # last dim must equal the 16 scan points
    st = lib.totri_mesh_confocal_forward(ctypes.byref(verts), ctypes.byref(faces),
                                         ctypes.byref(mat), ctypes.byref(sp), ctypes.byref(so),
                                         ctypes.byref(bad_tr), 0.01, 0.0, 0, None, 0, None)
    assert st == _lib.TOTRI_ERR_INVALID_ARGUMENT
    assert b"transient" in lib.totri_last_error()
    bad_faces = _arr((1, 4, 3), dtype=0)  # float faces
    tr = _arr((1, 32, 16))
    st = lib.totri_mesh_confocal_forward(ctypes.byref(verts), ctypes.byref(bad_faces),
                                         ctypes.byref(mat), ctypes.byref(sp), ctypes.byref(so),
                                         ctypes.byref(tr), 0.01, 0.0, 0, None, 0, None)
    assert st == _lib.TOTRI_ERR_INVALID_ARGUMENT
    too_many = _arr((1, 10, 5))  # at most 4 material channels
    st = lib.totri_mesh_confocal_forward(ctypes.byref(verts), ctypes.byref(faces),
                                         ctypes.byref(too_many), ctypes.byref(sp),
                                         ctypes.byref(so), ctypes.byref(tr), 0.01, 0.0, 0, None,
                                         0, None)
    assert st == _lib.TOTRI_ERR_INVALID_ARGUMENT


def test_mesh_forward_requires_workspace(lib):
    from totri_gb300 import _lib
    verts, faces, mat = _arr((1, 10, 3)), _arr((1, 4, 3), dtype=2), _arr((1, 10, 0))
    sp, so, tr = _arr((1, 16, 3)), _arr((1, 0, 3)), _arr((1, 32, 16))
    st = lib.totri_mesh_confocal_forward(ctypes.byref(verts), ctypes.byref(faces),
                                         ctypes.byref(mat), ctypes.byref(sp), ctypes.byref(so),
                                         ctypes.byref(tr), 0.01, 0.0, 0, None, 0, None)
    assert st == _lib.TOTRI_ERR_WORKSPACE


def test_python_error_mapping(lib):
    from totri_gb300 import _lib
    with pytest.raises(ValueError):
        lib.totri_mesh_visibility  # noqa: B018 (bound)
        _lib.check(_lib.TOTRI_ERR_INVALID_ARGUMENT)
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.TOTRI_ERR_UNSUPPORTED)
    with pytest.raises(RuntimeError):
        _lib.check(_lib.TOTRI_ERR_CUDA)


def test_bounds_checking_build_exports_every_entry_point():
    """TOTRI_BOUNDS_CHECK=1 builds the bounds-checking variant into its own
    directory; it exports the same entry points (built and loaded in a child
    process, since the choice is made when the build module is imported)."""
    import subprocess
    import sys
    code = ("import ctypes, sys; sys.path.insert(0, %r)\n"
            "from totri_gb300 import build\n"
            "assert build.bounds_check() and build.BUILD_DIR.endswith('_build_check')\n"
            "lib = ctypes.CDLL(build.build())\n"
            "missing = [n for n in %r if not hasattr(lib, n)]\n"
            "assert not missing, missing\n" % (ROOT, declared_functions()))
    env = dict(os.environ, TOTRI_BOUNDS_CHECK="1")
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         timeout=900)
    assert res.returncode == 0, res.stderr[-2000:]
