"""Wall-grid helper of the reference (totri/data/util.py:6-35).

The scan-grid ordering (x fastest) defines how a flat [S] scan axis maps to
a 2-D wall image, so it is kept exactly.
"""
import torch


def make_wall_grid(x_from=-1, x_to=1, x_res=32, y_from=-1, y_to=1, y_res=32, z_val=0,
                   device=torch.device('cuda'), x_fastest=True,
                   flattened=True) -> torch.Tensor:
    """Wall coordinates [y_res * x_res, 3] (or [y_res, x_res, 3] when not flattened)."""
    x = torch.linspace(x_from, x_to, x_res, device=device)
    y = torch.linspace(y_from, y_to, y_res, device=device)
    if x_fastest:
        y, x = torch.meshgrid(y, x, indexing='ij')
    else:
        x, y = torch.meshgrid(x, y, indexing='ij')
    z = torch.full_like(x, fill_value=z_val)
    scan_points = torch.stack((x, y, z), dim=2)
    if flattened:
        return scan_points.view(-1, 3)
    return scan_points


def merge_meshes(verts_list, faces_list):
    """Concatenates meshes [V_i, 3] / [F_i, 3] into one (totri/data/util.py:67-76)."""
    offsets = [0]
    for v in verts_list[:-1]:
        offsets.append(offsets[-1] + v.shape[-2])
    faces = torch.cat([f + o for f, o in zip(faces_list, offsets)], dim=-2)
    verts = torch.cat(verts_list, dim=-2)
    return verts, faces
