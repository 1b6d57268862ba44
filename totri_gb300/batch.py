"""Batched mesh rendering: many meshes of uneven size in one graph launch.

``BatchedMeshRenderer`` packs a list of meshes into waves that fit an HBM
budget (meshes sorted by face count, each wave padded to its own largest
vertex and face counts; padded faces are -1 rows, which end a face list
exactly as in the reference), keeps every buffer resident, picks tile shapes
with the autotuner per wave, and captures the whole sequence — for every wave
the BVH build, visibility masks, splat, the loss head and the gradient — as
one CUDA graph. A step is then one graph replay for the whole batch instead
of per-mesh launches from Python. New geometry of the same sizes is loaded
with ``load()`` (a device copy into the captured buffers).

Loss heads (``grad``):
  * ``"external"`` — the caller passes d loss / d transient to ``step()``; the
    batch must fit one wave (the gradient of every mesh is held at once);
  * ``"energy"`` — loss = 0.5 * ||transient||^2 per mesh, whose gradient is
    the transient itself (no second transient-sized buffer); any wave count;
  * ``"normal"`` — d loss / d transient of mesh i is a standard normal field
    drawn from seed ``normal_seed + i`` (``totri_fill_normal``: the same values
    for any wave packing), loss = <transient, d loss / d transient>; any wave
    count;
  * a callable ``fn(wave_meshes, transient, transient_grad)`` run inside the
    capture (torch ops on the device), which fills ``transient_grad`` for the
    meshes of the wave (indices into the constructor's list).

Tuned tile values are installed (``totri_tune_set``, a process-wide table)
only while this renderer launches its own kernels and handed back to the
built-in choices afterwards; captured graphs keep the values they were
captured with. Renderers on several threads must not launch concurrently.
"""
import ctypes
import math
import typing

import torch

from . import _lib, autotune
from .totri_cpp._common import mesh_workspace, ws_args
from .types import BinDef


class _Wave:
    def __init__(self, index, members, V, F, dev):
        self.index = index
        self.members = members  # constructor indices of the meshes in this wave
        n = len(members)
        self.verts = torch.zeros((n, V, 3), device=dev)
        self.faces = torch.full((n, F, 3), -1, dtype=torch.int32, device=dev)
        self.colors = torch.ones((n, V, 1), device=dev)
        self.verts_grad = torch.zeros_like(self.verts)
        self.colors_grad = torch.zeros_like(self.colors)
        self.member_ids = torch.tensor(members, dtype=torch.int64, device=dev)


def chunked_dot(a, b, chunk=1 << 30):
    """<a, b> over all elements as a sum of dot products of at most `chunk`
    elements each: cuBLAS takes 32-bit vector lengths, and one mesh's
    exhaustive transient (2,048 bins x 64x64 x 16x16 points) holds 2^31."""
    a, b = a.reshape(-1), b.reshape(-1)
    parts = [torch.dot(a[i:i + chunk], b[i:i + chunk]) for i in range(0, a.numel(), chunk)]
    if not parts:
        return torch.zeros((), dtype=a.dtype, device=a.device)
    return parts[0] if len(parts) == 1 else torch.stack(parts).sum()


class BatchedMeshRenderer:
    """Forward and vertex/albedo gradient of many meshes against one wall setup.

    Args:
        meshes: list of (verts [V_i, 3] float32, faces [F_i, 3] int, colors [V_i, 1] or None)
        scan_points: [S, 3] wall points (detector points for the exhaustive renderer)
        bin_def: BinDef with num set
        laser_points: [L, 3] laser points, or None for the confocal renderer
        grad: loss head, "external", "energy" or a callable (module docstring)
        hbm_budget: bytes for the transient buffers of one wave (default 80 GB)
        graph: capture CUDA graphs (True) or launch eagerly
        tune: run the tile autotuner on each wave's shapes first
    """

    def __init__(self, meshes: typing.Sequence, scan_points: torch.Tensor, bin_def: BinDef,
                 laser_points: typing.Optional[torch.Tensor] = None, device=None,
                 grad="external", hbm_budget: float = 80e9, graph: bool = True,
                 tune: bool = True, normal_seed: int = 0):
        self.device = dev = torch.device(device or "cuda")
        self.lib = _lib.load()
        self.bin_def = bin_def
        self.exhaustive = laser_points is not None
        self.grad = grad
        self.normal_seed = int(normal_seed)
        self.sizes = [(m[0].shape[0], m[1].shape[0]) for m in meshes]
        S = scan_points.shape[0]
        T = bin_def.num
        self.scan_points = scan_points.to(dev, torch.float32).contiguous()
        if self.exhaustive:
            L = laser_points.shape[0]
            self.laser_points = laser_points.to(dev, torch.float32).contiguous()
            item = (T, S, L)
            points = S + L
        else:
            L = 1
            item = (T, S)
            points = S
        item_bytes = 4 * math.prod(item) * (1 if grad == "energy" else 2)
        # the exhaustive gradient's bins-last scratch (at most 2 GiB) comes
        # out of the budget first
        scratch = (int(self.lib.totri_mesh_exhaustive_grad_scratch(S, L, T))
                   if self.exhaustive else 0)
        per_wave = max(1, int((hbm_budget - scratch) // item_bytes))
        if grad == "external" and per_wave < len(meshes):
            raise ValueError("grad='external' needs the whole batch in one wave: %d meshes, "
                             "%d fit the HBM budget" % (len(meshes), per_wave))
        order = sorted(range(len(meshes)), key=lambda i: -self.sizes[i][1])
        self.waves = []
        self.slot = {}  # constructor index -> (wave, position)
        for w0 in range(0, len(order), per_wave):
            members = order[w0:w0 + per_wave]
            V = max(self.sizes[i][0] for i in members)
            F = max(self.sizes[i][1] for i in members)
            wave = _Wave(len(self.waves), members, V, F, dev)
            for pos, i in enumerate(members):
                self.slot[i] = (wave, pos)
            self.waves.append(wave)
        for i, m in enumerate(meshes):
            self.load(i, *m)
        W = max(len(w.members) for w in self.waves)
        self.transient = torch.empty((W,) + item, device=dev)
        self.transient_grad = (self.transient if grad == "energy"
                               else torch.zeros((W,) + item, device=dev))
        self.loss = torch.zeros(len(meshes), device=dev)
        ws = max(int(self.lib.totri_mesh_workspace(len(w.members), w.verts.shape[1],
                                                   w.faces.shape[1], points))
                 for w in self.waves)
        # each wave's gradient finds the scratch past its own mesh layout
        self.workspace = torch.empty(max(ws + scratch, 1), dtype=torch.uint8, device=dev)
        self.stream = torch.cuda.Stream(dev)
        self.tiles = {}
        if tune:
            # Each wave is tuned on a proxy: its median mesh alone (tile choices
            # depend on bins, wall points and face count, not on the batch size).
            splat = "mesh.exhaustive.splat.lt" if self.exhaustive else "mesh.confocal.splat.ts"
            with torch.cuda.stream(self.stream):
                for w in self.waves:
                    pos = len(w.members) // 2
                    cls = autotune.shape_class(F=self.sizes[w.members[pos]][1], S=S, T=T, L=L)
                    self.tiles[w.index] = {
                        key: autotune.tune(key, lambda: self._forward_calls(w, pos), cls,
                                           reps=2)[0]
                        for key in ("mesh.visibility.mode", splat)}
        self.graph_forward = None
        self.graph_step = None
        if graph:
            with torch.cuda.stream(self.stream):
                self._step_calls()  # warm-up: kernel attributes, lazy module loading
            self.stream.synchronize()
            if len(self.waves) == 1:
                self.graph_forward = torch.cuda.CUDAGraph()
                with torch.cuda.graph(self.graph_forward, stream=self.stream):
                    self._forward_calls(self.waves[0])
            self.graph_step = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph_step, stream=self.stream):
                self._step_calls()
        self._restore_tiles()

    # -- device work -------------------------------------------------------

    def _install_tiles(self, w):
        for key, value in self.tiles.get(w.index, {}).items():
            autotune.set_tile(key, value)

    def _restore_tiles(self):
        """Hands the tuned keys back to the built-in choices (other callers of
        the library are not affected by this renderer's tuning)."""
        for key in {k for t in self.tiles.values() for k in t}:
            autotune.set_tile(key, 0)

    def _args(self):
        bd = self.bin_def
        return (float(bd.width), float(bd.offset), 0,
                *ws_args(self.workspace), _lib.stream_of(self.device))

    def _wall(self, w):
        n = len(w.members)
        sp = self.scan_points[None].expand(n, -1, 3)
        empty = self.scan_points[None, :0].expand(n, 0, 3)
        if not self.exhaustive:
            return sp, empty
        lp = self.laser_points[None].expand(n, -1, 3)
        return sp, lp, empty, empty

    def _forward_calls(self, w, only=None):
        """Forward of wave w (of its mesh at position `only` alone, for tuning)."""
        A = _lib.array
        if only is None:
            self._install_tiles(w)
            sl = slice(0, len(w.members))
        else:
            sl = slice(only, only + 1)
        tr = self.transient[:sl.stop - sl.start]
        wall = [A(t[:sl.stop - sl.start]) for t in self._wall(w)]
        mesh = (A(w.verts[sl]), A(w.faces[sl]), A(w.colors[sl]))
        if self.exhaustive:
            st = self.lib.totri_mesh_exhaustive_forward(*mesh, *wall, A(tr), *self._args())
        else:
            st = self.lib.totri_mesh_confocal_forward(*mesh, *wall, A(tr), *self._args())
        _lib.check(st)

    def _backward_calls(self, w):
        A = _lib.array
        n = len(w.members)
        tg = self.transient_grad[:n]
        wall = [A(t) for t in self._wall(w)]
        name = ("totri_mesh_exhaustive_grad_verts_reuse" if self.exhaustive
                else "totri_mesh_confocal_grad_verts_reuse")
        st = getattr(self.lib, name)(A(w.verts), A(w.faces), A(w.colors), *wall, A(tg),
                                     A(w.verts_grad), A(w.colors_grad), *self._args())
        _lib.check(st)

    def _loss_head(self, w):
        n = len(w.members)
        tr = self.transient[:n]
        if self.grad == "energy":
            sq = torch.linalg.vector_norm(tr.reshape(n, -1), dim=1)
            self.loss.index_copy_(0, w.member_ids, 0.5 * sq * sq)
        elif self.grad == "normal":
            tg = self.transient_grad[:n]
            for pos, i in enumerate(w.members):
                _lib.check(self.lib.totri_fill_normal(
                    ctypes.c_void_p(tg[pos].data_ptr()), tg[pos].numel(),
                    self.normal_seed + i, _lib.stream_of(self.device)))
            # one dot product per mesh (no transient-sized temporary)
            dots = torch.stack([chunked_dot(tr[p], tg[p]) for p in range(n)])
            self.loss.index_copy_(0, w.member_ids, dots)
        elif callable(self.grad):
            self.grad(list(w.members), tr, self.transient_grad[:n])

    def _step_calls(self):
        try:
            self._wave_calls()
        finally:
            self._restore_tiles()

    def _wave_calls(self):
        for w in self.waves:
            self._forward_calls(w)
            self._loss_head(w)
            self._backward_calls(w)

    # -- public API --------------------------------------------------------

    def load(self, i, verts, faces=None, colors=None):
        """Copies mesh i (sizes within its wave's capacity) into the batch buffers."""
        w, pos = self.slot[i]
        V = verts.shape[0]
        if V > w.verts.shape[1] or (faces is not None and faces.shape[0] > w.faces.shape[1]):
            raise ValueError("mesh %d does not fit its wave (%d verts, %d faces)"
                             % (i, w.verts.shape[1], w.faces.shape[1]))
        w.verts[pos].zero_()
        w.verts[pos, :V].copy_(verts)
        if faces is not None:
            w.faces[pos].fill_(-1)
            w.faces[pos, :faces.shape[0]].copy_(faces)
        if colors is not None:
            w.colors[pos, :V].copy_(colors.reshape(V, -1)[:, :1])

    def forward(self):
        """Renders every mesh of a one-wave batch; returns the batch transient
        (a resident buffer, rows in wave order: see ``wave_order``)."""
        if len(self.waves) != 1:
            raise ValueError("forward() needs a one-wave batch; use step() with a loss head")
        torch.cuda.current_stream(self.device).synchronize()
        if self.graph_forward is not None:
            self.graph_forward.replay()
        else:
            with torch.cuda.stream(self.stream):
                try:
                    self._forward_calls(self.waves[0])
                finally:
                    self._restore_tiles()
        self.stream.synchronize()
        return self.transient

    def step(self, transient_grad: typing.Optional[torch.Tensor] = None):
        """Forward + loss head + backward for every mesh. With grad='external',
        `transient_grad` (rows in wave order) is copied in first. Returns the
        per-mesh loss (energy and normal heads) or None; gradients via
        ``mesh_grads()``."""
        if transient_grad is not None:
            if self.grad != "external":
                raise ValueError("transient_grad is given only with grad='external'")
            self.transient_grad.copy_(transient_grad)
        torch.cuda.current_stream(self.device).synchronize()
        if self.graph_step is not None:
            self.graph_step.replay()
        else:
            with torch.cuda.stream(self.stream):
                self._step_calls()
        self.stream.synchronize()
        return self.loss if self.grad in ("energy", "normal") else None

    def wave_order(self):
        """Constructor indices of the transient rows of a one-wave batch."""
        return list(self.waves[0].members)

    def mesh_grads(self):
        """Per-mesh (verts_grad [V_i, 3], colors_grad [V_i, 1]) of the last step,
        in constructor order."""
        out = []
        for i, (v, _) in enumerate(self.sizes):
            w, pos = self.slot[i]
            out.append((w.verts_grad[pos, :v], w.colors_grad[pos, :v]))
        return out
