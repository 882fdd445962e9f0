"""The oracle's backward (FP64 autograd) against central finite differences
in FP64, on tiny scenes where no clamp or threshold is near its boundary.

The discrete part (culling, tile lists, depth order) is held fixed from the
unperturbed scene; the FD perturbation moves only the continuous part."""
import numpy as np
import pytest
import torch

from dmgs_gb300.camera import make_view
from helpers import oracle_camera
from oracle import raster as R


def _tiny_scene(seed, P=12):
    rng = np.random.default_rng(seed)
    means = rng.uniform(-0.3, 0.3, (P, 3)).astype(np.float32)
    scales = np.exp(rng.uniform(-2.0, -1.2, (P, 3))).astype(np.float32)
    q = rng.standard_normal((P, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    opac = rng.uniform(0.2, 0.7, (P, 1)).astype(np.float32)
    shs = np.concatenate([rng.normal(0.5, 0.2, (P, 1, 3)), rng.normal(0, 0.1, (P, 15, 3))], 1)
    view = make_view((0.3, 0.4, 3.0), (0, 0, 0), 32, 32, fovx_deg=40)
    return means, scales, q.astype(np.float32), opac, shs.astype(np.float32), view


def _image64(cam, t, fixed):
    """FP64 image from tensors `t` with the tile lists of `fixed`."""
    vals, ranges, vis = fixed
    sel = torch.as_tensor(vis)
    ndc, pix, conic, op, rgb = R.project_fp64(cam, t["means3D"], t["opacities"], t["shs"],
                                              t["colors"], t["scales"], t["rotations"], t["cov3D"], sel)
    remap = np.full(t["means3D"].shape[0], -1)
    remap[vis] = np.arange(len(vis))
    bg = torch.as_tensor(np.asarray(cam.bg, np.float64))
    gx, gy = cam.grid
    W, H = cam.width, cam.height
    tiles = []
    for tt in range(gx * gy):
        ty, tx = divmod(tt, gx)
        x0, y0 = tx * 16, ty * 16
        x1, y1 = min(x0 + 16, W), min(y0 + 16, H)
        r0, r1 = ranges[tt]
        yy, xx = torch.meshgrid(torch.arange(y0, y1, dtype=torch.float64),
                                torch.arange(x0, x1, dtype=torch.float64), indexing="ij")
        pxy = torch.stack([xx.reshape(-1), yy.reshape(-1)], 1)
        if r1 == r0:
            out = bg.view(1, 3).expand(pxy.shape[0], 3)
        else:
            g = torch.as_tensor(remap[vals[r0:r1].astype(np.int64)])
            out, _, _, _ = R._blend_tile(pxy, pix[g], conic[g], op[g], rgb[g], bg)
        tiles.append(((y0, y1, x0, x1), out))
    img = torch.zeros(3, H, W, dtype=torch.float64)
    for (y0, y1, x0, x1), out in tiles:
        img[:, y0:y1, x0:x1] = out.T.reshape(3, y1 - y0, x1 - x0)
    return img


@pytest.mark.parametrize("mode", [("shs", "sr"), ("colors", "cov")], ids=["shs-sr", "colors-cov"])
def test_oracle_backward_matches_central_differences(mode):
    means, scales, rots, opac, shs, view = _tiny_scene(0)
    cam = oracle_camera(view, bg=(0.1, 0.2, 0.3))
    rng = np.random.default_rng(1)
    P = means.shape[0]
    arrays = dict(
        means3D=means.astype(np.float64), opacities=opac.astype(np.float64),
        shs=shs.astype(np.float64) if mode[0] == "shs" else None,
        colors=rng.uniform(0, 1, (P, 3)) if mode[0] == "colors" else None,
        scales=scales.astype(np.float64) if mode[1] == "sr" else None,
        rotations=rots.astype(np.float64) if mode[1] == "sr" else None,
        cov3D=R.cov3d_from_scale_rot_f32(scales, rots, 1.0).astype(np.float64) if mode[1] == "cov" else None)
    f32 = {k: (None if v is None else v.astype(np.float32)) for k, v in arrays.items()}
    res = R.render(cam, f32["means3D"], f32["opacities"], shs=f32["shs"], colors=f32["colors"],
                   scales=f32["scales"], rotations=f32["rotations"], cov3D=f32["cov3D"])
    assert not res.ambiguous.any()
    fixed = (res.values, res.ranges, np.nonzero(res.geom["visible"])[0])
    dimg = torch.tensor(rng.standard_normal((3, 32, 32)))

    def loss(arrs, grad=False):
        t = {k: (None if v is None else torch.tensor(v, requires_grad=grad)) for k, v in arrs.items()}
        return (_image64(cam, t, fixed) * dimg).sum(), t

    L, leaves = loss(arrays, grad=True)
    L.backward()
    eps = 1e-6
    for name, leaf in leaves.items():
        if leaf is None:
            continue
        base = arrays[name]
        for fi in rng.choice(base.size, size=min(16, base.size), replace=False):
            up = {k: (None if v is None else v.copy()) for k, v in arrays.items()}
            dn = {k: (None if v is None else v.copy()) for k, v in arrays.items()}
            up[name].reshape(-1)[fi] += eps
            dn[name].reshape(-1)[fi] -= eps
            fd = (float(loss(up)[0]) - float(loss(dn)[0])) / (2 * eps)
            an = leaf.grad.numpy().reshape(-1)[fi]
            assert abs(fd - an) <= 1e-6 + 1e-5 * abs(fd), (name, int(fi), fd, an)


def test_render_backward_equals_fixed_list_autograd():
    """render().backward (the per-tile memory-bounded path) equals plain
    autograd through the same forward."""
    means, scales, rots, opac, shs, view = _tiny_scene(3, P=20)
    cam = oracle_camera(view)
    res = R.render(cam, means, opac, shs=shs, scales=scales, rotations=rots)
    rng = np.random.default_rng(4)
    dimg = rng.standard_normal((3, 32, 32))
    g = res.backward(dimg)
    fixed = (res.values, res.ranges, np.nonzero(res.geom["visible"])[0])
    arrs = dict(means3D=means, opacities=opac, shs=shs, colors=None, scales=scales,
                rotations=rots, cov3D=None)
    t = {k: (None if v is None else torch.tensor(v.astype(np.float64), requires_grad=True))
         for k, v in arrs.items()}
    (_image64(cam, t, fixed) * torch.tensor(dimg)).sum().backward()
    for k in ("means3D", "opacities", "shs", "scales", "rotations"):
        np.testing.assert_allclose(g[k], t[k].grad.numpy(), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(res.image, _image64(cam, {k: (None if v is None else torch.tensor(v.astype(np.float64))) for k, v in arrs.items()}, fixed).numpy(), atol=1e-12)
