"""Request server: continuous batching of render, gradient and backprojection
requests on one GPU.

Resident state (device memory, kept across requests):
  * meshes — vertices, faces, albedo and the prepared BVH/face records
    (``totri_mesh_prepare``), built once at registration;
  * wall grids — scan points;
  * measurements — transients [T, S] on a registered grid (backprojection
    inputs and gradient targets);
  * visibility masks per (mesh, grid), computed by the first request that
    needs them and kept in an LRU cache (bins do not change visibility).

Requests are admitted first-come-first-served with a bounded look-ahead
whenever a stream slot of their class is free and their device memory
(outputs, scratch, masks still to be computed) fits the HBM budget next to the
resident state; admitted requests run concurrently on separate CUDA streams.
Each request gets a rough GPU-time estimate (``Server.cost_ms``): small
requests run on high-priority streams, large ones (estimated at
``large_ms`` or more: big backprojections, first renders of a large mesh on a
large grid) on normal-priority streams, so the thread blocks of a small
request are dispatched ahead of the blocks a large kernel still has queued
and a small request does not wait for a large one to finish. A request's
result is copied to pinned host memory on its stream and its future resolves
when that copy has completed. Cancelling a future drops a queued request; an
admitted request runs to the end on the GPU, its result is discarded and its
memory returns to the budget when it completes.

Kinds (``Request.kind``):
  * "render"      — confocal mesh transient [T, S] (``mesh``, ``grid``, ``bins``);
  * "grad"        — loss mean((render - target)^2) against measurement
                    ``target`` and its gradients: (loss, verts_grad [V, 3],
                    colors_grad [V, 1]);
  * "backproject" — Velten confocal backprojection of measurement ``target``
                    into ``volume`` (a VolumeDef): volume [D, H, W];
  * "fit_pose"    — ``iterations`` steps of the rigid pose fit of mesh ``mesh``
                    to measurement ``target`` (``fitting.PoseFitting``, no
                    early stop): (translation [3], quaternion [4], losses
                    [iterations]). The pose changes the geometry every step,
                    so each step rebuilds the BVH and masks in its own scratch.
  * "fit_depth_map" — ``iterations`` steps of the depth-map fit
                    (``fitting.DepthMapFitting`` with its default weights and
                    learning-rate schedule) of a height field over ``volume``
                    (resolution (D, H, W): an H x W grid) to measurement
                    ``target``: (depth [H, W], albedo [H, W], losses
                    [iterations]). Enqueued like fit_pose, without host
                    synchronisation.
  * "fit_rbf"     — ``iterations`` driver moves of the Gaussian-blob fit
                    (``fitting.RbfFitting``: add, split, delete, refine) from an
                    empty set of blobs in ``volume`` to measurement ``target``,
                    its random choices drawn from a generator seeded with
                    ``seed``: (blobs [n, 4] as x, y, z, sigma, data loss). The
                    moves accept or reject on the host, so the fit runs on a
                    worker thread with the request's stream current; it always
                    counts as large.
"""
import collections
import concurrent.futures
import dataclasses
import itertools
import threading
import time
import typing

import torch

from . import _lib
from .totri_cpp import reconstruct as K
from .types import BinDef, VolumeDef


@dataclasses.dataclass
class Request:
    kind: str
    grid: str
    mesh: typing.Optional[str] = None
    bins: typing.Optional[BinDef] = None
    target: typing.Optional[str] = None
    volume: typing.Optional[VolumeDef] = None
    iterations: int = 0
    seed: int = 0
    # filled in by the server
    id: int = -1
    arrival: float = 0.0
    admitted: float = 0.0
    done: float = 0.0
    large: bool = False


class Budget:
    """Byte accounting of the HBM budget: resident bytes plus in-flight bytes."""

    def __init__(self, total):
        self.total = int(total)
        self.resident = 0
        self.inflight = 0
        self.peak = 0

    def free(self):
        return self.total - self.resident - self.inflight

    def fits(self, need):
        return need <= self.free()

    def take(self, need):
        self.inflight += need
        self.peak = max(self.peak, self.resident + self.inflight)

    def give(self, need):
        self.inflight -= need


class MaskCache:
    """LRU cache of visibility masks keyed by (mesh, grid). Entries in use by
    in-flight requests are pinned; eviction frees the least recently used
    unpinned entries until the requested bytes fit."""

    Entry = collections.namedtuple("Entry", "buf nbytes ready")

    def __init__(self, budget: Budget):
        self.budget = budget
        self.entries = collections.OrderedDict()
        self.pins = collections.Counter()

    def get(self, key):
        e = self.entries.get(key)
        if e is not None:
            self.entries.move_to_end(key)
        return e

    def put(self, key, entry):
        """Caches a mask whose bytes the admitting request counted in flight;
        the caller moves them from in-flight to resident (Budget.give), so the
        sum, and the peak taken at admission, do not change."""
        self.entries[key] = entry
        self.budget.resident += entry.nbytes

    def pin(self, key):
        self.pins[key] += 1

    def unpin(self, key):
        self.pins[key] -= 1
        if self.pins[key] <= 0:
            del self.pins[key]

    def make_room(self, need):
        """Evicts unpinned entries (LRU first) until `need` bytes fit."""
        for key in list(self.entries):
            if self.budget.fits(need):
                return True
            if self.pins.get(key):
                continue
            e = self.entries.pop(key)
            self.budget.resident -= e.nbytes
        return self.budget.fits(need)


class _Threaded:
    """A request run on a host thread (it needs host decisions between its
    kernels) with its slot's stream current on that thread. ``query()`` is
    True once the thread has returned and the copies it enqueued last have
    completed; ``result`` or ``exc`` then holds the outcome."""

    def __init__(self, fn, stream, device):
        self.result, self.exc, self.event = None, None, None
        self._stream, self._device = stream, device
        self.thread = threading.Thread(target=self._run, args=(fn,), daemon=True)
        self.thread.start()

    def _run(self, fn):
        try:
            torch.cuda.set_device(self._device)
            with torch.cuda.stream(self._stream):
                self.result = fn()
                ev = torch.cuda.Event()
                ev.record(self._stream)
                self.event = ev
        except BaseException as exc:  # reported through the request's future
            self.exc = exc

    def query(self):
        if self.thread.is_alive():
            return False
        return self.event is None or self.event.query()


class _Mesh:
    def __init__(self, verts, faces, colors, ws):
        self.verts, self.faces, self.colors, self.ws = verts, faces, colors, ws
        self.F = faces.shape[1]


class Server:
    """Continuous-batching request server (one GPU): `slots` high-priority CUDA
    streams for small requests and `large_slots` normal-priority streams for
    requests estimated at `large_ms` or more."""

    def __init__(self, device=None, hbm_budget=80e9, slots=4, lookahead=8, large_slots=2,
                 large_ms=5.0):
        device = torch.device(device or "cuda")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        self.lib = _lib.load()
        self.budget = Budget(hbm_budget)
        self.masks = MaskCache(self.budget)
        self.meshes, self.grids, self.measurements = {}, {}, {}
        lo, hi = torch.cuda.Stream.priority_range()
        self.streams = ([torch.cuda.Stream(self.device, priority=hi) for _ in range(slots)] +
                        [torch.cuda.Stream(self.device, priority=lo) for _ in range(large_slots)])
        self.slot_large = [False] * slots + [True] * large_slots
        self.large_ms = large_ms
        self.lookahead = lookahead
        self.queue = collections.deque()
        self.inflight = {}  # slot -> (request, future, event, release, result)
        self.cv = threading.Condition()
        self.ids = itertools.count()
        self.thread = None
        self.running = False
        self.completed = []
        self.cancelled = 0  # requests cancelled while in flight

    # -- resident state -----------------------------------------------------

    def _account(self, *tensors):
        self.budget.resident += sum(t.numel() * t.element_size() for t in tensors)

    def register_mesh(self, name, verts, faces, colors=None):
        """verts [V, 3], faces [F, 3], colors [V, 1]: copied to the device and
        prepared (BVH + face records) once."""
        dev = self.device
        v = verts.to(dev, torch.float32).reshape(1, -1, 3).contiguous()
        f = faces.to(dev, torch.int32).reshape(1, -1, 3).contiguous()
        c = (torch.ones((1, v.shape[1], 1), device=dev) if colors is None
             else colors.to(dev, torch.float32).reshape(1, v.shape[1], -1)[..., :1].contiguous())
        n = int(self.lib.totri_mesh_workspace(1, v.shape[1], f.shape[1], 0))
        ws = torch.empty(max(n, 1), dtype=torch.uint8, device=dev)
        A = _lib.array
        _lib.check(self.lib.totri_mesh_prepare(A(v), A(f), A(c), ctypes_ptr(ws), n,
                                               _lib.stream_of(dev)))
        torch.cuda.current_stream(dev).synchronize()
        self._account(v, f, c, ws)
        self.meshes[name] = _Mesh(v, f, c, ws)

    def register_grid(self, name, scan_points):
        sp = scan_points.to(self.device, torch.float32).reshape(1, -1, 3).contiguous()
        self._account(sp)
        self.grids[name] = sp

    def register_measurement(self, name, transient, grid, bins: BinDef):
        """transient [T, S] on registered grid `grid`, binned by `bins`."""
        tr = transient.to(self.device, torch.float32).reshape(1, *transient.shape[-2:])
        tr = tr.contiguous()
        if tr.shape[2] != self.grids[grid].shape[1]:
            raise ValueError("measurement has %d scan points, grid %s has %d"
                             % (tr.shape[2], grid, self.grids[grid].shape[1]))
        if tr.shape[1] != bins.num:
            raise ValueError("measurement has %d bins, its BinDef %d" % (tr.shape[1], bins.num))
        self._account(tr)
        self.measurements[name] = (tr, grid, bins)

    # -- requests -----------------------------------------------------------

    def submit(self, req: Request) -> concurrent.futures.Future:
        self._validate(req)
        fut = concurrent.futures.Future()
        with self.cv:
            if self.thread is not None and not self.thread.is_alive():
                raise RuntimeError("request server is not running")
            req.id = next(self.ids)
            req.arrival = time.perf_counter()
            self.queue.append((req, fut))
            self.cv.notify()
        return fut

    KINDS = ("render", "grad", "backproject", "fit_pose", "fit_depth_map", "fit_rbf")
    _FITS = ("fit_pose", "fit_depth_map", "fit_rbf")

    def _validate(self, r):
        if r.kind not in self.KINDS:
            raise ValueError("unknown request kind %r" % r.kind)
        if r.grid not in self.grids:
            raise KeyError("unknown grid %r" % r.grid)
        if r.kind in ("render", "grad", "fit_pose"):
            if r.mesh not in self.meshes:
                raise KeyError("unknown mesh %r" % r.mesh)
        if r.kind in ("render", "grad") + self._FITS and r.bins is None:
            raise ValueError("%s requests need bins" % r.kind)
        if r.kind in self._FITS and r.iterations < 1:
            raise ValueError("%s requests need iterations >= 1" % r.kind)
        if r.kind != "render":
            if r.target not in self.measurements:
                raise KeyError("unknown measurement %r" % r.target)
            tr, grid, bins = self.measurements[r.target]
            if grid != r.grid:
                raise ValueError("measurement %r is on grid %r" % (r.target, grid))
            if r.kind != "backproject" and (bins.num, bins.width, bins.offset) != (
                    r.bins.num, r.bins.width, r.bins.offset):
                raise ValueError("measurement %r is binned differently from the request"
                                 % r.target)
        if r.kind in ("backproject", "fit_depth_map", "fit_rbf") and r.volume is None:
            raise ValueError("%s requests need a VolumeDef" % r.kind)
        if r.kind == "fit_depth_map" and min(r.volume.resolution[1:]) < 2:
            raise ValueError("fit_depth_map needs a grid of at least 2 x 2")

    # Rates behind cost_ms, measured on one GB300 (the differentiable
    # 20,480-face workload and the 128^3 Velten backprojection): visibility
    # 9e9 (point, face) pairs/s, splat 1.1e11, gradient 6.5e10, backprojection
    # 9e11 voxel-point pairs/s, device-to-host copies 25 GB/s.
    _RATES = dict(visibility=9e9, splat=1.1e11, grad=6.5e10, backproject=9e11, copy=25e9)

    def cost_ms(self, r):
        """Rough GPU time of request r in ms; it only sorts requests into small
        and large."""
        k = self._RATES
        S = self.grids[r.grid].shape[1]
        if r.kind == "backproject":
            vox = 1
            for n in r.volume.resolution:
                vox *= int(n)
            return 1e3 * (vox * S / k["backproject"] + 4 * vox / k["copy"])
        if r.kind == "fit_depth_map":
            V, F = self._depth_map_size(r)
            return 1e3 * r.iterations * F * S * (1 / k["visibility"] + 1 / k["splat"] +
                                                 1 / k["grad"])
        if r.kind == "fit_rbf":  # each driver move runs hundreds of optimiser steps
            V, F = self._rbf_mesh_bound(r)
            return 1e3 * r.iterations * 300 * F * S * (1 / k["visibility"] + 1 / k["splat"] +
                                                       1 / k["grad"])
        m = self.meshes[r.mesh]
        pairs = m.F * S
        if r.kind == "fit_pose":
            return 1e3 * r.iterations * pairs * (1 / k["visibility"] + 1 / k["splat"] +
                                                 1 / k["grad"])
        sec = pairs / k["splat"]
        if r.kind == "grad":
            sec += pairs / k["grad"] + 4 * 4 * m.verts.shape[1] / k["copy"]
        else:
            sec += 4 * r.bins.num * S / k["copy"]
        if self.masks.get((r.mesh, r.grid)) is None:
            sec += pairs / k["visibility"]
        return 1e3 * sec

    @staticmethod
    def _depth_map_size(r):
        """(vertices, faces) of a depth-map request's H x W grid."""
        H, W = int(r.volume.resolution[1]), int(r.volume.resolution[2])
        return H * W, 2 * (H - 1) * (W - 1)

    @staticmethod
    def _rbf_mesh_bound(r):
        """A planning bound on the (vertices, faces) of the iso-surface of an RBF
        fit's volume (its size is only known as the fit runs): eight faces per
        cell of the three axis-aligned mid-sections."""
        D, H, W = (int(n) for n in r.volume.resolution)
        F = 8 * (D * H + H * W + W * D)
        return 3 * F, F

    def _mask_bytes(self, r):
        S = self.grids[r.grid].shape[1]
        return int(self.lib.totri_mesh_mask_bytes(1, self.meshes[r.mesh].F, S))

    def _need(self, r):
        """Device bytes a request allocates while in flight (outputs, scratch,
        masks it has to compute)."""
        S = self.grids[r.grid].shape[1]
        if r.kind == "backproject":
            return 4 * int(torch.tensor(r.volume.resolution).prod())
        if r.kind in ("fit_depth_map", "fit_rbf"):
            # per step: scratch with masks, transients and their gradients,
            # parameters with gradients and optimiser state (and the RBF volume)
            V, F = (self._depth_map_size(r) if r.kind == "fit_depth_map"
                    else self._rbf_mesh_bound(r))
            ws = int(self.lib.totri_mesh_workspace(1, V, F, S))
            need = ws + 4 * 4 * r.bins.num * S + 32 * 4 * V
            if r.kind == "fit_rbf":
                D, H, W = (int(n) for n in r.volume.resolution)
                need += 64 * D * H * W
            return need
        m = self.meshes[r.mesh]
        if r.kind == "fit_pose":  # per step: scratch with masks, two transients, gradients
            ws = int(self.lib.totri_mesh_workspace(1, m.verts.shape[1], m.F, S))
            return ws + 3 * 4 * r.bins.num * S + 8 * 4 * m.verts.shape[1]
        need = 4 * r.bins.num * S
        if r.kind == "grad":
            need = 2 * need + 4 * 4 * m.verts.shape[1]
        if self.masks.get((r.mesh, r.grid)) is None:
            need += self._mask_bytes(r)
        return need

    # -- execution -----------------------------------------------------------

    def _launch(self, r, stream):
        """Enqueues request r on `stream`; returns (release bytes, host result
        holder, mask key pinned or None)."""
        dev = self.device
        A = _lib.array
        sp = self.grids[r.grid]
        S = sp.shape[1]
        key = None
        if r.kind == "fit_pose":
            return self._fit_pose(r)
        if r.kind == "fit_depth_map":
            return self._fit_depth_map(r)
        if r.kind == "fit_rbf":
            return _Threaded(lambda: self._fit_rbf(r), stream, self.device)
        if r.kind in ("render", "grad"):
            m = self.meshes[r.mesh]
            key = (r.mesh, r.grid)
            e = self.masks.get(key)
            if e is None:
                nbytes = self._mask_bytes(r)
                buf = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
                _lib.check(self.lib.totri_mesh_prepared_visibility(
                    A(m.verts), A(m.faces), A(m.colors), A(sp), ctypes_ptr(m.ws),
                    m.ws.numel(), ctypes_ptr(buf), nbytes, _lib.stream_of(dev)))
                ready = torch.cuda.Event()
                ready.record(stream)
                e = MaskCache.Entry(buf, nbytes, ready)
                self.masks.put(key, e)
            else:
                stream.wait_event(e.ready)
                e.buf.record_stream(stream)
            self.masks.pin(key)
            empty = sp[:, :0]
            bd = r.bins
            tr = torch.empty((1, bd.num, S), device=dev)
            _lib.check(self.lib.totri_mesh_prepared_confocal_forward(
                A(m.verts), A(m.faces), A(m.colors), A(sp), A(empty), A(tr), float(bd.width),
                float(bd.offset), ctypes_ptr(m.ws), m.ws.numel(), ctypes_ptr(e.buf), e.nbytes,
                _lib.stream_of(dev)))
            if r.kind == "render":
                host = torch.empty(tr.shape[1:], dtype=torch.float32, pin_memory=True)
                host.copy_(tr[0], non_blocking=True)
                return host
            target = self.measurements[r.target][0]
            target.record_stream(stream)
            diff = tr - target
            loss = (diff * diff).mean()
            tg = diff.mul_(2.0 / diff.numel())
            vg = torch.empty_like(m.verts)
            cg = torch.empty_like(m.colors)
            _lib.check(self.lib.totri_mesh_prepared_confocal_grad_verts(
                A(m.verts), A(m.faces), A(m.colors), A(sp), A(empty), A(tg), A(vg), A(cg),
                float(bd.width), float(bd.offset), ctypes_ptr(m.ws), m.ws.numel(),
                ctypes_ptr(e.buf), e.nbytes, _lib.stream_of(dev)))
            out = (torch.empty((), dtype=torch.float32, pin_memory=True),
                   torch.empty(vg.shape[1:], dtype=torch.float32, pin_memory=True),
                   torch.empty(cg.shape[1:], dtype=torch.float32, pin_memory=True))
            out[0].copy_(loss, non_blocking=True)
            out[1].copy_(vg[0], non_blocking=True)
            out[2].copy_(cg[0], non_blocking=True)
            return out
        tr, _, bd = self.measurements[r.target]
        tr.record_stream(stream)
        vd = r.volume
        vol = torch.empty((1,) + tuple(vd.resolution), device=dev)
        K.backprojection_confocal_velten_forward(tr, sp, sp[:, :0], vol, vd.start, vd.end,
                                                 bd.width, bd.offset)
        host = torch.empty(vol.shape[1:], dtype=torch.float32, pin_memory=True)
        host.copy_(vol[0], non_blocking=True)
        return host

    def _fit_pose(self, r):
        """Enqueues the pose fit on the current stream; no host synchronisation."""
        from .fitting import PoseFitting
        m = self.meshes[r.mesh]
        target = self.measurements[r.target][0]
        target.record_stream(torch.cuda.current_stream(self.device))
        fitting = PoseFitting(r.bins)
        (t,), (q,) = fitting.fit(target[0], self.grids[r.grid][0], [m.verts[0]],
                                 [m.faces[0]], num_iter=r.iterations, stop_loss=None,
                                 colors_list=[m.colors[0]])
        losses = torch.stack(fitting.losses)
        out = (torch.empty(3, dtype=torch.float32, pin_memory=True),
               torch.empty(4, dtype=torch.float32, pin_memory=True),
               torch.empty(r.iterations, dtype=torch.float32, pin_memory=True))
        out[0].copy_(t.translation.detach()[0], non_blocking=True)
        out[1].copy_(q.quaternion.detach()[0], non_blocking=True)
        out[2].copy_(losses, non_blocking=True)
        return out

    def _fit_depth_map(self, r):
        """Enqueues the depth-map fit on the current stream; no host
        synchronisation."""
        from .fitting import DepthMap, DepthMapFitting
        target = self.measurements[r.target][0]
        target.record_stream(torch.cuda.current_stream(self.device))
        vd = VolumeDef(r.volume.start, r.volume.end, r.volume.resolution)
        dm = DepthMap(vd, device=self.device)
        fitting = DepthMapFitting(r.bins)
        fitting.fit(dm, target[0], self.grids[r.grid][0], num_iter=r.iterations)
        losses = torch.stack(fitting.losses)
        out = (torch.empty(dm.depth.shape, dtype=torch.float32, pin_memory=True),
               torch.empty(dm.color.shape, dtype=torch.float32, pin_memory=True),
               torch.empty(r.iterations, dtype=torch.float32, pin_memory=True))
        out[0].copy_(dm.depth.detach(), non_blocking=True)
        out[1].copy_(dm.color.detach(), non_blocking=True)
        out[2].copy_(losses, non_blocking=True)
        return out

    def _fit_rbf(self, r):
        """The Gaussian-blob fit; runs on a worker thread (see _Threaded)."""
        from .fitting import GaussianRbfBase, RbfFitting, TransientBackgroundEmpty
        target = self.measurements[r.target][0][0]
        target.record_stream(torch.cuda.current_stream(self.device))
        gen = torch.Generator(device=self.device)
        gen.manual_seed(int(r.seed))
        vd = VolumeDef(r.volume.start, r.volume.end, r.volume.resolution)
        fitting = RbfFitting(r.bins, self.grids[r.grid][0], generator=gen)
        base = fitting.fit(GaussianRbfBase(vd, device=self.device), target,
                           num_iter=r.iterations)
        norm = target / target.mean()
        loss = fitting.loss_all(base, TransientBackgroundEmpty(), norm)[0]["data"]
        out = (torch.empty(base.params.shape, dtype=torch.float32, pin_memory=True),
               torch.empty((), dtype=torch.float32, pin_memory=True))
        out[0].copy_(base.params.detach(), non_blocking=True)
        out[1].copy_(loss.detach(), non_blocking=True)
        return out

    def _admit_one(self):
        """Admits the first of the next `lookahead` queued requests that fits
        and has a free stream of its class; drops cancelled ones."""
        free = [i for i in range(len(self.streams)) if i not in self.inflight]
        if not free or not self.queue:
            return False
        cached = sum(e.nbytes for e in self.masks.entries.values())
        ceiling = self.budget.total - (self.budget.resident - cached)
        for qi in range(min(self.lookahead, len(self.queue))):
            r, fut = self.queue[qi]
            if fut.cancelled():
                del self.queue[qi]
                return True
            large = r.kind == "fit_rbf" or self.cost_ms(r) >= self.large_ms
            slots = [i for i in free if self.slot_large[i] == large]
            if not slots:
                continue
            need = self._need(r)
            if need > ceiling:  # could never fit, even on an idle device
                del self.queue[qi]
                fut.set_exception(MemoryError(
                    "request needs %d bytes; the HBM budget leaves %d next to the resident "
                    "state" % (need, ceiling)))
                return True
            if not self.budget.fits(need) and not self.masks.make_room(need):
                continue
            del self.queue[qi]
            slot = slots[0]
            stream = self.streams[slot]
            r.large = large
            key = (r.mesh, r.grid) if r.kind in ("render", "grad") else None
            new_mask = key is not None and key not in self.masks.entries
            self.budget.take(need)
            r.admitted = time.perf_counter()
            try:
                with torch.cuda.stream(stream):
                    result = self._launch(r, stream)
                    if isinstance(result, _Threaded):
                        ev = result  # done when its thread and last copies are
                    else:
                        ev = torch.cuda.Event()
                        ev.record(stream)
            except Exception as exc:  # invalid request data: fail this request only
                if new_mask and key in self.masks.entries:
                    need -= self._mask_bytes(r)  # cached before the failure: now resident
                self.budget.give(need)
                if key is not None and key in self.masks.pins:
                    self.masks.unpin(key)
                fut.set_exception(exc)
                return True
            if new_mask and key in self.masks.entries:
                # the mask computed for this request stays cached: its bytes,
                # counted in `need`, now belong to the resident state
                mb = self._mask_bytes(r)
                self.budget.give(mb)
                need -= mb
            self.inflight[slot] = (r, fut, ev, need, result)
            return True
        return False

    def _reap(self):
        done = False
        for slot in list(self.inflight):
            r, fut, ev, need, result = self.inflight[slot]
            if not ev.query():
                continue
            del self.inflight[slot]
            self.budget.give(need)
            if r.kind in ("render", "grad"):
                self.masks.unpin((r.mesh, r.grid))
            r.done = time.perf_counter()
            if isinstance(result, _Threaded):
                exc, result = result.exc, result.result
                if exc is not None and not fut.cancelled():
                    fut.set_exception(exc)
                    done = True
                    continue
            if fut.cancelled():  # cancelled in flight: the result is dropped
                self.cancelled += 1
            else:
                self.completed.append(r)
                fut.set_result(result)
            done = True
        return done

    def _loop(self):
        try:
            self._serve()
        except BaseException as exc:  # the loop died: fail everything still waiting
            with self.cv:
                pending = [fut for _, fut in self.queue]
                pending += [entry[1] for entry in self.inflight.values()]
                self.queue.clear()
                self.inflight.clear()
                self.running = False
            for fut in pending:
                if not fut.done():
                    fut.set_exception(RuntimeError("request server stopped: %r" % (exc,)))
            raise

    def _serve(self):
        torch.cuda.set_device(self.device)
        while True:
            with self.cv:
                if not self.running and not self.queue and not self.inflight:
                    return
                if not self.queue and not self.inflight:
                    self.cv.wait(timeout=0.05)
                    continue
                progressed = self._reap()
                while self._admit_one():
                    progressed = True
            if not progressed:
                time.sleep(5e-5)

    def start(self):
        if self.thread is None:
            self.running = True
            self.thread = threading.Thread(target=self._loop, daemon=True)
            self.thread.start()
        return self

    def stop(self):
        """Finishes every queued and in-flight request, then stops the loop."""
        with self.cv:
            self.running = False
            self.cv.notify()
        if self.thread is not None:
            self.thread.join()
            self.thread = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    @staticmethod
    def _p50_p99(values):
        lat = sorted(values)
        if not lat:
            return None, None
        pick = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]  # noqa: E731
        return pick(0.5), pick(0.99)

    def latency_ms(self):
        """(p50, p99) of completion - arrival over completed requests, in ms."""
        return self._p50_p99([1e3 * (r.done - r.arrival) for r in self.completed])

    def latency_breakdown(self):
        """p50/p99 (ms) of the queue wait (admission - arrival) and the service
        time (completion - admission), over all completed requests and per
        class (small / large), with the request counts."""
        out = {}
        for name, sel in (("all", lambda r: True), ("small", lambda r: not r.large),
                          ("large", lambda r: r.large)):
            rs = [r for r in self.completed if sel(r)]
            out[name] = {"requests": len(rs),
                         "latency": self._p50_p99([1e3 * (r.done - r.arrival) for r in rs]),
                         "wait": self._p50_p99([1e3 * (r.admitted - r.arrival) for r in rs]),
                         "service": self._p50_p99([1e3 * (r.done - r.admitted) for r in rs])}
        return out


def ctypes_ptr(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr())
