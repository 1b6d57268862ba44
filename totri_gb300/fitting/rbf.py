"""RBF-blob shape fitting: Gaussian blobs -> volume -> marching-cubes mesh ->
transient, fitted to a measurement (reference totri/fitting/rbf.py:19-821).

``GaussianRbfBase`` holds the blobs [N, 4(+1)] (x, y, z, sigma, colour);
its volume is ``Rbf2VolumeGaussian`` with the field zeroed on the border
slices (so every surface closes), its mesh ``MarchingCubesFunction`` at iso
0.5 (rbf.py:88-98). ``RbfFitting.fit`` cycles through five moves
(rbf.py:784-795): add blobs where the backprojected positive residual is
large (after a second-derivative filter), add blobs at mesh vertices with
large loss gradient, split blobs (sigma x 0.75 and a random offset), delete
blobs whose removal costs less than ``delete_Factor``, and refine; each move
is kept only if the loss does not rise. ``optimize`` runs Adam with the loss
normalised to 1, checks every 10 iterations after 20 whether the loss rose
(then restores the last good state and halves the learning rate, at most 8
times) or improved by less than 1% (then stops), rbf.py:418-512. The data
loss is the mean squared error (rbf.py:313-315) after, optionally, scaling
the render by its least-squares factor (``project_transient``,
rbf.py:287-293). TensorBoard and video output are not reproduced; the
background model is any module with the reference's interface
(``TransientBackgroundEmpty`` by default).
"""
import copy
import typing

import torch

from ..reconstruct import (BackprojectionConfocalVelten, BackprojectionExhaustiveVelten,
                           second_derivative_filter)
from ..render import MeshRenderConfocal, MeshRenderExhaustive
from ..types import BinDef, VolumeDef
from ..util import MarchingCubesFunction, Rbf2VolumeGaussian


class TransientBackgroundEmpty(torch.nn.Module):
    """Zero background (reference totri/fitting/background.py:28-46)."""

    def forward(self, scan_points, laser_points=None):
        shape = (scan_points.shape[0], 1, scan_points.shape[1])
        if laser_points is not None:
            shape = shape + (laser_points.shape[1],)
        return torch.zeros(shape, device=scan_points.device, dtype=scan_points.dtype)

    def clone(self):
        return copy.deepcopy(self)

    def param_list(self):
        return list(self.parameters())

    def clamp_parameters(self, foreground, background):
        pass

    def requires_grad(self, flag):
        for p in self.parameters():
            p.requires_grad = flag

    def copy_from(self, other):
        with torch.no_grad():
            for a, b in zip(self.parameters(), other.parameters()):
                a[:] = b[:]


class GaussianRbfBase:
    def __init__(self, volume_def: VolumeDef, has_color: bool = False, sigma_init=0.05,
                 sigma_min=0.00001, sigma_max=0.5, margin=0.1, device="cuda"):
        self.volume_def = volume_def
        self.has_color = has_color
        self.num_channels = 5 if has_color else 4
        self.params = torch.empty((0, self.num_channels), device=device)
        self.sigma_init, self.sigma_min, self.sigma_max = sigma_init, sigma_min, sigma_max
        self.margin = margin
        self.volume_mask_ = None

    def clone(self):
        out = copy.copy(self)
        out.params = self.params.clone()
        return out

    def subdivide(self):
        self.volume_def.resolution = tuple(2 * r for r in self.volume_def.resolution)
        self.volume_mask_ = None

    def difference(self, base):
        ext = self.volume_def.extent()
        d = (self.params - base.params).abs().max(dim=0).values.tolist()
        d[0], d[1], d[2] = d[0] / ext[0], d[1] / ext[1], d[2] / ext[2]
        d[3] = d[3] / (self.sigma_max - self.sigma_min)
        return max(d)

    def requires_grad(self, flag):
        self.params.requires_grad = flag

    def param_list(self):
        return [self.params]

    def num_rbf(self):
        return self.params.shape[0]

    def get_pos(self):
        return self.params[:, :3]

    def get_sigma(self):
        return self.params[:, 3:4]

    def get_color(self):
        return self.params[:, 3:4] if self.has_color else None

    def clamp_params(self):
        if self.num_rbf() == 0:
            return
        with torch.no_grad():
            for a in range(3):
                self.params[:, a] = self.params[:, a].clamp(
                    self.volume_def.start[a] + self.margin, self.volume_def.end[a] - self.margin)
            self.params[:, 3] = self.params[:, 3].clamp(min=self.sigma_min, max=self.sigma_max)
            if self.has_color:
                if self.num_rbf() > 1:
                    scale = 1.0 / (1.e-12 + self.params[:, 4].max())
                    self.params[:, 4] = torch.clamp(self.params[:, 4] * scale, min=1.e-12)
                else:
                    self.params[:, 4] = 1.0

    def volume_mask(self):
        if self.volume_mask_ is None:
            m = torch.ones(self.volume_def.resolution, dtype=torch.float32,
                           device=self.params.device)
            m[[0, -1]] = 0
            m[:, [0, -1]] = 0
            m[:, :, [0, -1]] = 0
            self.volume_mask_ = m
        return self.volume_mask_

    def make_volume(self) -> torch.Tensor:
        vol = Rbf2VolumeGaussian.apply(self.params[None], self.volume_def)[0]
        return torch.cat((vol[:1] * self.volume_mask(), vol[1:]), dim=0)

    def make_verts(self) -> torch.Tensor:
        """Triangle soup [3 T, 3 (+1)] of the blob surface at iso 0.5."""
        return MarchingCubesFunction.apply(self.make_volume()[None], 0.5, self.volume_def.start,
                                           self.volume_def.end)[0]

    def append(self, x, y, z):
        row = [x, y, z, self.sigma_init] + ([1.0] if self.has_color else [])
        new = torch.tensor([row], dtype=torch.float32, device=self.params.device)
        self.params = torch.cat((self.params, new), dim=0)

    def remove(self, idx):
        self.params = torch.cat((self.params[:idx], self.params[idx + 1:]), dim=0)

    def half_distance(self):
        return 1.177 * self.sigma_init


class RbfFitting:
    def __init__(self, bin_def: BinDef, scan_points: torch.Tensor,
                 laser_points: typing.Optional[torch.Tensor] = None,
                 scan_origin: typing.Optional[torch.Tensor] = None,
                 laser_origin: typing.Optional[torch.Tensor] = None,
                 optimize_check_delete: bool = False, delete_Factor: float = 1.001,
                 tensorboard: bool = False, video: bool = False, log_dir: str = None,
                 project_transient: bool = True,
                 generator: typing.Optional[torch.Generator] = None):
        """generator: the random source of the blob moves (volume and surface
        samples, split choices and offsets), on the device of the scan points;
        torch's default generator when None."""
        if tensorboard or video:
            raise NotImplementedError("TensorBoard and video output are not part of totri_gb300")
        self.bin_def_init = bin_def
        self.bin_def = bin_def
        self.scan_points, self.laser_points = scan_points, laser_points
        self.scan_origin, self.laser_origin = scan_origin, laser_origin
        self.optimize_check_delete = optimize_check_delete
        self.delete_Factor = delete_Factor
        self.project_transient = project_transient
        self.log_dir = log_dir
        self.generator = generator

    def reduce_transient(self, transient_input, margin=32):
        """Crops leading and trailing bins without signal (rbf.py:218-243):
        per bin the 0.95-quantile over the wall points, a threshold of a tenth
        of the largest such quantile, the first and last bins at or above it
        widened by `margin`; sets bin_def to the cropped range and returns
        transient_input [T, S(, L)] cut to it."""
        q = torch.quantile(transient_input.flatten(start_dim=1), 0.95, dim=1).cpu()
        threshold = q.max() / 10
        num_bins = q.shape[0]
        start, end = 0, num_bins
        for i in range(num_bins - 1):
            if q[i] < threshold:
                start = i + 1
            else:
                break
        for i in range(num_bins - 1, 0, -1):
            if q[i] < threshold:
                end = i
            else:
                break
        start = max(start - margin, 0)
        end = min(end + margin, num_bins)
        self.bin_def = BinDef(self.bin_def_init.width,
                              self.bin_def_init.offset + self.bin_def_init.width * start,
                              end - start)
        return transient_input[start:end]

    # -- loss ---------------------------------------------------------------

    def render(self, verts, background_model, transient_input):
        """verts [t, 3 (+A)] -> (transient, foreground, background) [T, S(, L)]."""
        color = None
        if verts.shape[1] == 4:
            color = torch.clamp(verts[None, :, 3:4].contiguous(), min=1.e-6)
        v = verts[None, :, :3].contiguous()
        b = lambda t: None if t is None else t[None]  # noqa: E731
        if self.laser_points is None:
            fg = 10 * MeshRenderConfocal.apply(v, None, self.scan_points[None], self.bin_def,
                                               color, b(self.scan_origin))[0]
            bg = background_model(self.scan_points[None])[0]
        else:
            fg = MeshRenderExhaustive.apply(v, None, self.scan_points[None],
                                            self.laser_points[None], self.bin_def, color,
                                            b(self.scan_origin), b(self.laser_origin))[0]
            bg = background_model(self.scan_points[None], self.laser_points[None])[0]
        tr = fg + bg
        if self.project_transient:
            num = (tr * transient_input).sum()
            den = (tr * tr).sum()
            tr = tr * (num / den.clamp(min=1.e-6)).clamp(min=1.e-6)
        return tr, fg, bg

    def base_to_transient(self, base, background_model, transient_input):
        return self.render(base.make_verts(), background_model, transient_input)

    @staticmethod
    def loss_data(transient, transient_input):
        return torch.mean((transient - transient_input) ** 2)

    def loss_all(self, base, background_model, transient_input, return_transients=False,
                 transients=None):
        if transients is None:
            transients = self.base_to_transient(base, background_model, transient_input)
        losses = {"data": self.loss_data(transients[0], transient_input)}
        full = losses["data"]
        if return_transients:
            return losses, full, transients
        return losses, full

    # -- inner optimisation -------------------------------------------------

    def optimize(self, base, background_model, transient_input, num_iter, base_lr=1.e-3):
        loss_eps, lr, lr_multiplier, max_reset = 1.e-2, base_lr, 0.5, 8
        if base.num_rbf() == 0:
            losses, full = self.loss_all(base, background_model, transient_input)
            return losses, full, 0
        base_backup = base.clone()
        bg_backup = background_model.clone()
        base.requires_grad(True)
        background_model.requires_grad(True)
        params = lambda: base.param_list() + background_model.param_list()  # noqa: E731
        optim = torch.optim.Adam(params(), lr=lr)
        losses, full, tr = self.loss_all(base, background_model, transient_input, True)
        scale = 1 / full.detach()
        full = full * scale
        last = full.detach()
        since_reset, resets, iteration = 0, 0, -1
        for iteration in range(num_iter):
            full.backward()
            optim.step()
            base.clamp_params()
            background_model.clamp_parameters(tr[1], tr[2])
            optim.zero_grad()
            since_reset += 1
            losses, full, tr = self.loss_all(base, background_model, transient_input, True)
            full = full * scale
            if since_reset > 20 and since_reset % 10 == 0:
                if full > last:  # the loss rose: back to the last good state, smaller steps
                    if resets == max_reset:
                        break
                    with torch.no_grad():
                        base.params[:] = base_backup.params[:]
                        background_model.copy_from(bg_backup)
                    resets += 1
                    lr *= lr_multiplier
                    optim = torch.optim.Adam(params(), lr=lr)
                    optim.zero_grad()
                    losses, full, tr = self.loss_all(base, background_model, transient_input,
                                                     True)
                    full = full * scale
                    last = full.detach()
                    since_reset = 0
                    continue
                if since_reset >= 20 and (last - full.detach()) / last < loss_eps:
                    break
                with torch.no_grad():
                    base_backup.params[:] = base.params[:]
                    bg_backup.copy_from(background_model)
                    last = full.detach()
        base.requires_grad(False)
        background_model.requires_grad(False)
        full = full.detach() / scale
        losses = {k: (v.detach() if isinstance(v, torch.Tensor) else v) for k, v in losses.items()}
        return losses, full, iteration + 1

    # -- moves ---------------------------------------------------------------

    def _accept(self, base, bg, base_new, bg_new, initial, final):
        return (base_new, bg_new, True) if final <= initial else (base, bg, False)

    def add_blobs_volume(self, base, background_model, transient_input, num_samples=5):
        _, initial, tr = self.loss_all(base, background_model, transient_input, True)
        vd = base.volume_def.clone()
        vd.resolution = tuple(r // 2 for r in vd.resolution)
        err = (transient_input - tr[0]).clamp(min=0)
        b = lambda t: None if t is None else t[None]  # noqa: E731
        if self.laser_points is None:
            ve = BackprojectionConfocalVelten.apply(err[None], self.scan_points[None], vd,
                                                    self.bin_def, b(self.scan_origin))
        else:
            ve = BackprojectionExhaustiveVelten.apply(err[None], self.scan_points[None],
                                                      self.laser_points[None], vd, self.bin_def,
                                                      b(self.scan_origin), b(self.laser_origin))
        ve = second_derivative_filter(ve.clamp(min=0))
        ve = (ve / ve.max()) ** 2
        samples = torch.multinomial(ve.flatten(), num_samples, replacement=False,
                                    generator=self.generator).tolist()
        base_new, bg_new = base.clone(), background_model.clone()
        for smp in samples:
            x, y, z = vd.index_to_coordinates(vd.flat_idx_to_3d_idx(smp))
            base_new.append(x, y, z + 0.5)
        base_new.clamp_params()
        self.optimize(base_new, bg_new, transient_input, num_iter=200)
        _, final = self.loss_all(base_new, bg_new, transient_input)
        return self._accept(base, background_model, base_new, bg_new, initial, final)

    def sample_vertices(self, base, background_model, transient_input, num_samples):
        verts = base.make_verts().detach()
        if verts.shape[0] == 0:
            return []
        verts.requires_grad = True
        trs = self.render(verts, background_model, transient_input)
        loss = self.loss_all(base, background_model, transient_input, transients=trs)[1]
        loss.backward()
        w = (verts.grad ** 2).sum(dim=-1) ** 0.5
        if float(w.sum()) == 0:
            return []
        idx = torch.multinomial(w, min(num_samples, verts.shape[0]), replacement=False,
                                generator=self.generator)
        return verts.detach()[idx].tolist()

    def add_blobs_surface(self, base, background_model, transient_input, num_samples=5):
        _, initial = self.loss_all(base, background_model, transient_input)
        samples = self.sample_vertices(base, background_model, transient_input, num_samples)
        if not samples:
            return base, background_model, False
        base_new, bg_new = base.clone(), background_model.clone()
        for smp in samples:
            base_new.append(*smp[:3])
        base_new.clamp_params()
        self.optimize(base_new, bg_new, transient_input, num_iter=200)
        _, final = self.loss_all(base_new, bg_new, transient_input)
        return self._accept(base, background_model, base_new, bg_new, initial, final)

    def split_blobs(self, base, background_model, transient_input):
        if base.num_rbf() == 0:
            return base, background_model, False
        _, initial = self.loss_all(base, background_model, transient_input)
        n = base.num_rbf()
        new = min(min(32, n), max(0, 500 - n))
        base_new, bg_new = base.clone(), background_model.clone()
        if new > 0:
            picks = torch.multinomial(base.get_sigma()[:, 0], new, replacement=False,
                                      generator=self.generator).tolist()
            for idx in picks:
                base_new.params[idx, 3] = 0.75 * base_new.params[idx, 3]
                base_new.params = torch.cat((base_new.params, base_new.params[None, idx]), 0)
                off = base_new.params[idx, 3] * (2 * torch.rand((2,), device=base.params.device,
                                                                generator=self.generator) - 1)
                base_new.params[idx, :2] += off
                base_new.params[-1, :2] -= off
        _, final, _ = self.optimize(base_new, bg_new, transient_input, num_iter=400)
        return self._accept(base, background_model, base_new, bg_new, initial, final)

    def check_delete(self, base, background_model, transient_input):
        if base.num_rbf() <= 1:
            return base, background_model, 0
        start_opt = (self.delete_Factor - 1) * 3 + 1
        count0 = base.num_rbf()
        loss = self.loss_all(base, background_model, transient_input)[1]
        i = 0
        while i < base.num_rbf():
            bt, bgt = base.clone(), background_model.clone()
            bt.remove(i)
            lt = self.loss_all(bt, bgt, transient_input)[1]
            if self.optimize_check_delete and loss * self.delete_Factor < lt <= loss * start_opt:
                lt = self.optimize(bt, bgt, transient_input, num_iter=50)[1]
            if lt <= loss * self.delete_Factor:
                base, background_model, loss = bt, bgt, lt
            else:
                i += 1
        return base, background_model, count0 - base.num_rbf()

    def refine(self, base, background_model, transient_input):
        base_new, bg_new = base.clone(), background_model.clone()
        _, before = self.loss_all(base, background_model, transient_input)
        _, after, _ = self.optimize(base_new, bg_new, transient_input, num_iter=500)
        return self._accept(base, background_model, base_new, bg_new, before, after)

    # -- driver --------------------------------------------------------------

    def fit(self, base: GaussianRbfBase, transient_input: torch.Tensor,
            background_model=None, num_iter=1000, subdivide_at=(), callback=None,
            **unused) -> GaussianRbfBase:
        """transient_input [T, S] (or [T, S, L]); returns the fitted base."""
        if background_model is None:
            background_model = TransientBackgroundEmpty()
        self.bin_def = self.bin_def_init
        transient_input = transient_input / transient_input.mean()
        self.max_val = transient_input.max()
        for i in range(num_iter):
            step = i % 5
            if step == 0 or base.num_rbf() == 0:
                base, background_model, _ = self.add_blobs_volume(base, background_model,
                                                                  transient_input, 5)
            elif step == 1:
                base, background_model, _ = self.add_blobs_surface(base, background_model,
                                                                   transient_input, 5)
            elif step == 2:
                base, background_model, _ = self.split_blobs(base, background_model,
                                                             transient_input)
            elif step == 3:
                base, background_model, _ = self.check_delete(base, background_model,
                                                              transient_input)
            else:
                base, background_model, _ = self.refine(base, background_model,
                                                        transient_input)
            if i in subdivide_at:
                base.subdivide()
            if callback is not None:
                callback(i, base, background_model)
        return base
