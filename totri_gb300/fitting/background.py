"""Learned transient backgrounds for the fitting loops (reference
totri/fitting/background.py:28-186).

A background is a small MLP over cosine encodings of the wall positions
(cos(k x'), cos(k y') for k = 1..PE, with x', y' the wall coordinates mapped to
[0, pi]) and of time (cos(k t'), k = 1..TE, t' on [0, pi] over T/8 coarse
bins), through Linear -> LeakyReLU -> Linear -> LeakyReLU -> Linear ->
Sigmoid, linearly upsampled to T bins and scaled by a learned intensity that
``clamp_parameters`` keeps at most `clamping_factor` times the foreground's
RMS. The confocal form encodes the scan point; the exhaustive form encodes
the scan and the laser point. These are plain PyTorch modules: nothing here is
on the GPU hot path.
"""
import copy
import math

import torch

from .rbf import TransientBackgroundEmpty

__all__ = ["TransientBackgroundEmpty", "TransientBackgroundConfocal",
           "TransientBackgroundExhaustive"]


class _Background(torch.nn.Module):
    def __init__(self, num_bins, wall_start, wall_end, num_pos_encodings, num_t_encodings,
                 channels, clamping_factor, n_points, device, dtype):
        super().__init__()
        self.num_bins = num_bins
        self.num_bins_sub = max(num_bins // 8, 1)
        self.shift = (-min(wall_start[0], wall_end[0]), -min(wall_start[1], wall_end[1]))
        self.normalization = (math.pi / abs(wall_start[0] - wall_end[0]),
                              math.pi / abs(wall_start[1] - wall_end[1]))
        self.num_pos_encodings, self.num_t_encodings = num_pos_encodings, num_t_encodings
        self.clamping_factor = clamping_factor
        width = 2 * n_points * num_pos_encodings + num_t_encodings
        self.decoder = torch.nn.Sequential(
            torch.nn.Linear(width, channels), torch.nn.LeakyReLU(),
            torch.nn.Linear(channels, channels // 2), torch.nn.LeakyReLU(),
            torch.nn.Linear(channels // 2, 1), torch.nn.Sigmoid())
        self.intensity = torch.nn.Parameter(torch.ones((1,)))
        self.to(device=device, dtype=dtype)

    def _pos(self, pts):
        """[B, n, 2 PE] cosine encodings of wall points [B, n, 3]."""
        x = (pts[..., 0:1] + self.shift[0]) * self.normalization[0]
        y = (pts[..., 1:2] + self.shift[1]) * self.normalization[1]
        k = torch.arange(1, self.num_pos_encodings + 1, device=pts.device, dtype=pts.dtype)
        return torch.cat((torch.cos(k * x), torch.cos(k * y)), dim=-1)

    def _time(self, like):
        t = torch.linspace(0, math.pi, self.num_bins_sub, device=like.device, dtype=like.dtype)
        k = torch.arange(1, self.num_t_encodings + 1, device=like.device, dtype=like.dtype)
        return torch.cos(t[:, None] * k)  # [T0, TE]

    def _upsample(self, coarse):
        """[B, T0, M] -> [B, T, M] (linear, half-pixel centres)."""
        return torch.nn.functional.interpolate(coarse.permute(0, 2, 1), self.num_bins,
                                               mode="linear",
                                               align_corners=False).permute(0, 2, 1)

    def clone(self):
        return copy.deepcopy(self)

    def param_list(self):
        return list(self.parameters())

    def requires_grad(self, flag):
        for p in self.parameters():
            p.requires_grad = flag

    def copy_from(self, other):
        with torch.no_grad():
            for a, b in zip(self.parameters(), other.parameters()):
                a[:] = b[:]

    def clamp_parameters(self, foreground, background):
        with torch.no_grad():
            fg = (foreground ** 2).mean() ** 0.5
            bg = (background ** 2).mean() ** 0.5
            cap = self.clamping_factor * fg
            if bg > cap:
                self.intensity[:] *= cap / bg


class TransientBackgroundConfocal(_Background):
    def __init__(self, num_bins, wall_start=(-1, -1), wall_end=(1, 1), num_pos_encodings=2,
                 num_t_encodings=4, channels=8, clamping_factor=1.0, device="cpu",
                 dtype=torch.float32):
        super().__init__(num_bins, wall_start, wall_end, num_pos_encodings, num_t_encodings,
                         channels, clamping_factor, 1, device, dtype)

    def forward(self, scan_points):
        """scan_points [B, S, 3] -> background [B, T, S]."""
        B, S = scan_points.shape[:2]
        T0 = self.num_bins_sub
        pos = self._pos(scan_points)[:, None].expand(-1, T0, -1, -1)
        tim = self._time(scan_points)[None, :, None].expand(B, -1, S, -1)
        coarse = self.decoder(torch.cat((pos, tim), dim=-1))[..., 0]  # [B, T0, S]
        return self.intensity * self._upsample(coarse)


class TransientBackgroundExhaustive(_Background):
    def __init__(self, num_bins, wall_start=(-1, -1), wall_end=(1, 1), num_pos_encodings=2,
                 num_t_encodings=4, channels=8, device="cpu", dtype=torch.float32):
        super().__init__(num_bins, wall_start, wall_end, num_pos_encodings, num_t_encodings,
                         channels, 1.0, 2, device, dtype)

    def forward(self, scan_points, laser_points):
        """scan [B, S, 3], laser [B, L, 3] -> background [B, T, S, L]."""
        B, S, L = scan_points.shape[0], scan_points.shape[1], laser_points.shape[1]
        T0 = self.num_bins_sub
        ps = self._pos(scan_points)[:, None, :, None].expand(-1, T0, -1, L, -1)
        pl = self._pos(laser_points)[:, None, None].expand(-1, T0, S, -1, -1)
        tim = self._time(scan_points)[None, :, None, None].expand(B, -1, S, L, -1)
        coarse = self.decoder(torch.cat((ps, pl, tim), dim=-1))[..., 0]  # [B, T0, S, L]
        out = self._upsample(coarse.reshape(B, T0, S * L))
        return self.intensity * out.reshape(B, self.num_bins, S, L)
