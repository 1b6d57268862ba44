"""Builds the reference's own kernel sources for the CPU (test infrastructure).

The reference's mesh programs (src/render/program/*_optix.cu) and its volume,
backprojection and RBF kernels (src/render/volume_cuda.cu,
src/reconstruct/backprojection_cuda.cu, src/util/rbf2volume_cuda.cu) are
compiled with g++ where they lie in the reference tree, against the stub
headers in oracle/ref_harness/stubs (OptiX, torch accessors, CUDA built-ins).
The launcher functions of the three *_cuda.cu files use the <<<>>> launch
syntax, so only their __global__/__device__ functions are cut out into
oracle/_ref/gen/ at build time and compiled there. Outputs go to oracle/_ref/
only; the shared library runs the reference arithmetic on the CPU to produce
the golden vectors in tests/golden/ (see tests/golden/make_golden.py). This
needs the reference tree, so it runs only where that tree is mounted.
"""
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "ref_harness")
STUBS = os.path.join(HARNESS, "stubs")
OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT, "gen")
# The reference tree: $TOTRI_REFERENCE, else where this container mounts it.
REF_ROOT = os.environ.get("TOTRI_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")
LIB = os.path.join(OUT, "libref_kernels.so")
CUBIN = os.path.join(OUT, "ref_kernels.cubin")

CXX = ["g++", "-std=c++20", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-w",
       "-include", os.path.join(STUBS, "cuda_host_shim.h"), "-I" + STUBS,
       "-I/usr/local/cuda/include"]

PROGRAMS = {
    "mesh_confocal_forward_optix.cu": "mcf",
    "mesh_confocal_grad_verts_optix.cu": "mcg",
    "mesh_exhaustive_forward_optix.cu": "mef",
    "mesh_exhaustive_grad_verts_optix.cu": "meg",
}

KERNEL_FILES = {
    "volume": ("render/volume_cuda.cu", "render"),
    "backprojection": ("reconstruct/backprojection_cuda.cu", "reconstruct"),
    "rbf2volume": ("util/rbf2volume_cuda.cu", "util"),
}


def available():
    return os.path.isdir(REF_SRC)


def _extract_device_code(path):
    """Returns the #defines and the __global__/__device__ function definitions of
    a .cu file (everything except host launchers), in file order."""
    src = open(path).read()
    out = []
    for line in src.splitlines():
        if line.startswith("#define"):
            out.append(line)
    i = 0
    n = len(src)
    while True:
        m = re.search(r"(template\s*<[^>]*>\s*)?__(global|device)__[^;{]*\{", src[i:])
        if not m:
            break
        start = i + m.start()
        j = i + m.end()
        depth = 1
        while depth and j < n:
            if src[j] == "{":
                depth += 1
            elif src[j] == "}":
                depth -= 1
            j += 1
        out.append(src[start:j])
        i = j
    return "\n".join(out)


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("%s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr[-4000:]))


def build(force=False):
    """Compiles the reference kernels for the CPU into oracle/_ref; returns the .so path."""
    if not available():
        raise RuntimeError("reference tree not found at %s" % REF_SRC)
    if os.path.exists(LIB) and not force:
        return LIB
    os.makedirs(GEN, exist_ok=True)
    jobs = []
    for fname, tag in PROGRAMS.items():
        src = os.path.join(REF_SRC, "render", "program", fname)
        obj = os.path.join(OUT, tag + ".o")
        jobs.append(CXX + ["-I" + REF_SRC, "-D__raygen__rg=ref_%s_rg" % tag,
                           "-D__closesthit__ch=ref_%s_ch" % tag, "-D__miss__ms=ref_%s_ms" % tag,
                           "-x", "c++", "-c", src, "-o", obj])
    for name, (rel, ns) in KERNEL_FILES.items():
        inc = os.path.join(GEN, name + "_kernels.inc")
        with open(inc, "w") as f:
            f.write("namespace totri {\nnamespace %s {\n" % ns)
            f.write(_extract_device_code(os.path.join(REF_SRC, rel)))
            f.write("\n}  // namespace %s\n}  // namespace totri\n" % ns)
    for drv in ("mesh_driver.cpp", "kernel_driver.cpp"):
        jobs.append(CXX + ["-I" + REF_SRC, "-I" + GEN, "-c", os.path.join(HARNESS, drv), "-o",
                           os.path.join(OUT, drv + ".o")])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs))
    objs = [os.path.join(OUT, t + ".o") for t in PROGRAMS.values()]
    objs += [os.path.join(OUT, d + ".o") for d in ("mesh_driver.cpp", "kernel_driver.cpp")]
    _run(["g++", "-shared", "-fopenmp", "-o", LIB + ".tmp", *objs])
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_gpu(force=False):
    """Compiles the reference's volume, backprojection and RBF kernels for
    sm_103a (oracle/ref_harness/gpu_kernels.cu around the kernel functions cut
    out by build()) into oracle/_ref/ref_kernels.cubin: a device-only image,
    loaded on a GPU machine through the CUDA driver (oracle/ref_gpu.py)."""
    build(force)
    src = os.path.join(HARNESS, "gpu_kernels.cu")
    if os.path.exists(CUBIN) and not force and os.path.getmtime(CUBIN) >= os.path.getmtime(src):
        return CUBIN
    _run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-cubin",
          "-I" + REF_SRC, "-I" + GEN, src, "-o", CUBIN + ".tmp"])
    os.replace(CUBIN + ".tmp", CUBIN)
    return CUBIN


_lib = None


def load():
    """Builds (if needed) and loads the reference kernels compiled for the CPU."""
    global _lib
    if _lib is None:
        import ctypes
        _lib = ctypes.CDLL(build())
    return _lib


def _p(a):
    import ctypes
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f32(a):
    import numpy as np
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def mesh_confocal_forward(verts, faces, material, scan_points, scan_origin, vis, nbins,
                          bin_width, bin_offset):
    """Reference confocal forward (one item): float32 [T, S]."""
    import ctypes
    import numpy as np
    v, sp = _f32(verts), _f32(scan_points)
    m = _f32(material).reshape(v.shape[0], -1)
    so = _f32(scan_origin if scan_origin is not None else np.zeros((0, 3))).reshape(-1, 3)
    f = np.ascontiguousarray(faces, dtype=np.int32)
    vis = np.ascontiguousarray(vis, dtype=np.uint8)
    out = np.zeros((nbins, sp.shape[0]), np.float32)
    load().ref_mesh_confocal_forward(
        _p(v), v.shape[0], _p(f), f.shape[0], _p(m), m.shape[1], _p(sp), sp.shape[0], _p(so),
        so.shape[0], _p(vis), _p(out), nbins, ctypes.c_float(bin_width),
        ctypes.c_float(bin_offset))
    return out


def mesh_confocal_grad(verts, faces, material, scan_points, scan_origin, vis, nbins, bin_width,
                       bin_offset, transient_grad):
    """Reference confocal gradient (one item): (verts_grad [V,3], material_grad [V,M])."""
    import ctypes
    import numpy as np
    v, sp = _f32(verts), _f32(scan_points)
    m = _f32(material).reshape(v.shape[0], -1)
    so = _f32(scan_origin if scan_origin is not None else np.zeros((0, 3))).reshape(-1, 3)
    f = np.ascontiguousarray(faces, dtype=np.int32)
    vis = np.ascontiguousarray(vis, dtype=np.uint8)
    tg = _f32(transient_grad)
    vg = np.zeros((v.shape[0], 3), np.float32)
    mg = np.zeros((v.shape[0], m.shape[1]), np.float32)
    load().ref_mesh_confocal_grad(
        _p(v), v.shape[0], _p(f), f.shape[0], _p(m), m.shape[1], _p(sp), sp.shape[0], _p(so),
        so.shape[0], _p(vis), _p(tg), nbins, _p(vg), 3, _p(mg), m.shape[1],
        ctypes.c_float(bin_width), ctypes.c_float(bin_offset))
    return vg, mg


def mesh_exhaustive_forward(verts, faces, material, scan_points, laser_points, scan_origin,
                            laser_origin, vis_s, vis_l, nbins, bin_width, bin_offset):
    """Reference exhaustive forward (one item): float32 [T, S, L]."""
    import ctypes
    import numpy as np
    v, sp, lp = _f32(verts), _f32(scan_points), _f32(laser_points)
    m = _f32(material).reshape(v.shape[0], -1)
    so = _f32(scan_origin if scan_origin is not None else np.zeros((0, 3))).reshape(-1, 3)
    lo = _f32(laser_origin if laser_origin is not None else np.zeros((0, 3))).reshape(-1, 3)
    f = np.ascontiguousarray(faces, dtype=np.int32)
    vs = np.ascontiguousarray(vis_s, dtype=np.uint8)
    vl = np.ascontiguousarray(vis_l, dtype=np.uint8)
    out = np.zeros((nbins, sp.shape[0], lp.shape[0]), np.float32)
    load().ref_mesh_exhaustive_forward(
        _p(v), v.shape[0], _p(f), f.shape[0], _p(m), m.shape[1], _p(sp), sp.shape[0], _p(lp),
        lp.shape[0], _p(so), so.shape[0], _p(lo), lo.shape[0], _p(vs), _p(vl), _p(out), nbins,
        ctypes.c_float(bin_width), ctypes.c_float(bin_offset))
    return out


def mesh_exhaustive_grad(verts, faces, material, scan_points, laser_points, scan_origin,
                         laser_origin, vis_s, vis_l, nbins, bin_width, bin_offset,
                         transient_grad):
    import ctypes
    import numpy as np
    v, sp, lp = _f32(verts), _f32(scan_points), _f32(laser_points)
    m = _f32(material).reshape(v.shape[0], -1)
    so = _f32(scan_origin if scan_origin is not None else np.zeros((0, 3))).reshape(-1, 3)
    lo = _f32(laser_origin if laser_origin is not None else np.zeros((0, 3))).reshape(-1, 3)
    f = np.ascontiguousarray(faces, dtype=np.int32)
    vs = np.ascontiguousarray(vis_s, dtype=np.uint8)
    vl = np.ascontiguousarray(vis_l, dtype=np.uint8)
    tg = _f32(transient_grad)
    vg = np.zeros((v.shape[0], 3), np.float32)
    mg = np.zeros((v.shape[0], m.shape[1]), np.float32)
    load().ref_mesh_exhaustive_grad(
        _p(v), v.shape[0], _p(f), f.shape[0], _p(m), m.shape[1], _p(sp), sp.shape[0], _p(lp),
        lp.shape[0], _p(so), so.shape[0], _p(lo), lo.shape[0], _p(vs), _p(vl), _p(tg), nbins,
        _p(vg), 3, _p(mg), m.shape[1], ctypes.c_float(bin_width), ctypes.c_float(bin_offset))
    return vg, mg


def _c(*xs):
    import ctypes
    return [ctypes.c_float(x) if isinstance(x, float) else x for x in xs]


def volume_confocal_forward(volume, mp, nbins, origin, size, bin_width, bin_offset):
    import numpy as np
    v, m = _f32(volume), _f32(mp)
    o, s = _f32(origin), _f32(size)
    out = np.zeros((m.shape[1], nbins), np.float32)
    load().ref_volume_confocal_forward(_p(v), *v.shape, _p(m), m.shape[1], _p(out), nbins, _p(o),
                                       _p(s), *_c(float(bin_width), float(bin_offset)))
    return out


def volume_confocal_grad_volume(transient, shape, mp, origin, size, bin_width, bin_offset):
    import numpy as np
    t, m = _f32(transient), _f32(mp)
    o, s = _f32(origin), _f32(size)
    out = np.zeros(tuple(shape), np.float32)
    load().ref_volume_confocal_grad_volume(_p(out), *shape, _p(m), m.shape[1], _p(t), t.shape[1],
                                           _p(o), _p(s), *_c(float(bin_width), float(bin_offset)))
    return out


def volume_confocal_grad_mp(volume, mp, transient_grad, origin, size, bin_width, bin_offset):
    import numpy as np
    v, m, g = _f32(volume), _f32(mp), _f32(transient_grad)
    o, s = _f32(origin), _f32(size)
    out = np.zeros((3, m.shape[1]), np.float32)
    load().ref_volume_confocal_grad_mp(_p(out), _p(v), *v.shape, _p(m), m.shape[1], _p(g),
                                       g.shape[1], _p(o), _p(s),
                                       *_c(float(bin_width), float(bin_offset)))
    return out


def volume_exhaustive_forward(volume, scan_points, laser_points, nbins, start, end, bin_width,
                              bin_offset):
    """volume [B,D,H,W]; points [B,3,S] / [B,3,L]; returns [B,T,S,L]."""
    import numpy as np
    v, sp, lp = _f32(volume), _f32(scan_points), _f32(laser_points)
    B, D, H, W = v.shape
    so = np.zeros((B, 3, 0), np.float32)
    a, e = _f32(start), _f32(end)
    out = np.zeros((B, nbins, sp.shape[2], lp.shape[2]), np.float32)
    load().ref_volume_exhaustive_forward(_p(v), B, D, H, W, _p(sp), sp.shape[2], _p(lp),
                                         lp.shape[2], _p(so), 0, _p(so), 0, _p(out), nbins, _p(a),
                                         _p(e), *_c(float(bin_width), float(bin_offset)))
    return out


def bp_confocal_velten(transient, scan_points, scan_origin, shape, start, end, bin_width,
                       bin_offset):
    """transient [B,T,S]; scan_points [B,S,3]; scan_origin [B,So,3]; volume [B,D,H,W]."""
    import numpy as np
    t, sp = _f32(transient), _f32(scan_points)
    B = t.shape[0]
    so = _f32(scan_origin) if scan_origin is not None else np.zeros((B, 0, 3), np.float32)
    a, e = _f32(start), _f32(end)
    out = np.zeros((B,) + tuple(shape), np.float32)
    load().ref_backprojection_confocal_velten(_p(t), B, t.shape[1], _p(sp), sp.shape[1], _p(so),
                                              so.shape[1], _p(out), *shape, _p(a), _p(e),
                                              *_c(float(bin_width), float(bin_offset)))
    return out


def bp_exhaustive_velten(transient, scan_points, laser_points, shape, start, end, bin_width,
                         bin_offset):
    """transient [B,T,S,L]; points [B,S,3] / [B,L,3]; volume [B,D,H,W]."""
    import numpy as np
    t, sp, lp = _f32(transient), _f32(scan_points), _f32(laser_points)
    B = t.shape[0]
    so = np.zeros((B, 0, 3), np.float32)
    a, e = _f32(start), _f32(end)
    out = np.zeros((B,) + tuple(shape), np.float32)
    load().ref_backprojection_exhaustive_velten(_p(t), B, t.shape[1], _p(sp), sp.shape[1], _p(lp),
                                                lp.shape[1], _p(so), 0, _p(so), 0, _p(out),
                                                *shape, _p(a), _p(e),
                                                *_c(float(bin_width), float(bin_offset)))
    return out


def bp_exhaustive_arellano(transient, scan_points, laser_points, shape, start, end, bin_width,
                           bin_offset):
    """transient [B,T,S,L]; points [B,3,S] / [B,3,L]; volume [B,D,H,W]."""
    import numpy as np
    t, sp, lp = _f32(transient), _f32(scan_points), _f32(laser_points)
    B = t.shape[0]
    so = np.zeros((B, 3, 0), np.float32)
    a, e = _f32(start), _f32(end)
    out = np.zeros((B,) + tuple(shape), np.float32)
    load().ref_backprojection_exhaustive_arellano(_p(t), B, t.shape[1], _p(sp), sp.shape[2],
                                                  _p(lp), lp.shape[2], _p(so), 0, _p(so), 0,
                                                  _p(out), *shape, _p(a), _p(e),
                                                  *_c(float(bin_width), float(bin_offset)))
    return out


def rbf2volume_forward(rbf, shape, start, end):
    """rbf [B,N,4+A]; volume [B,1+A,D,H,W]."""
    import numpy as np
    r = _f32(rbf)
    B, N, C = r.shape
    a, e = _f32(start), _f32(end)
    out = np.zeros((B, C - 3) + tuple(shape), np.float32)
    load().ref_rbf2volume_forward(_p(r), B, N, C, _p(out), *shape, _p(a), _p(e))
    return out


def rbf2volume_grad(rbf, volume, volume_grad, start, end):
    import numpy as np
    r, v, g = _f32(rbf), _f32(volume), _f32(volume_grad)
    B, N, C = r.shape
    a, e = _f32(start), _f32(end)
    out = np.zeros(r.shape, np.float32)
    load().ref_rbf2volume_grad(_p(r), B, N, C, _p(v), _p(g), *v.shape[2:], _p(out), _p(a), _p(e))
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
