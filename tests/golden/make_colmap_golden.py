"""Golden vectors for the real-scene (COLMAP) stage-2 path, from the
reference's own code.

Run in the build container (where the reference tree is mounted):

    python tests/golden/make_colmap_golden.py [/path/to/reference]

Imports, unmodified (device use redirected to the CPU and unused third-party
modules stubbed, as by make_golden.py; torch.jit.script is made the identity
while the model module loads, so its scripted in_frustum runs as plain
Python on the CPU):

* scene/gaussian_geo_model_mlp_flex_colmap.py — ``in_frustum`` (:31-76) for
  the whole screen, both halves and all four quarters, and
  ``renew_gaussian`` (:348-460) with ``get_covariance_dyn`` (:494-512) on a
  fixed mesh (the model's mesh source replaced by that mesh), forward and
  autograd gradients w.r.t. the vertices;
* geo/flexicubes_no_adjacent.py — ``construct_voxel_grid_vert_only``,
  ``construct_cubes`` and ``__call__`` (de_ambiguity=False, as the
  real-scene model calls it) on cube subsets chosen by those frustum masks
  and on the whole grid, in both quad-splitting modes, with autograd
  gradients of a fixed random linear loss w.r.t. the vertex positions and
  the scalar field.

Output: ``colmap_golden.npz`` next to this script.
"""
from __future__ import annotations

import math
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from tests.golden.make_golden import CpuRedirect, install_stubs, small_mesh  # noqa: E402
from tests.golden.make_flexicubes_golden import shape_sdf  # noqa: E402

PIECES = [(-1, 0), (0, 2), (1, 2), (0, 4), (1, 4), (2, 4), (3, 4)]


def camera(gfx, rng):
    """A camera outside the grid looking at it (the reference's matrices)."""
    eye = np.array([0.4, 0.9, 3.2])
    fwd = -eye / np.linalg.norm(eye)
    right = np.cross(fwd, [0.0, 1.0, 0.0])
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    c2w = np.stack([right, -up, fwd], 1)   # camera axes x right, y down, z forward
    R = c2w                                # world-to-view rotation transposed, as COLMAP stores it
    T = -c2w.T @ eye
    W2V = torch.tensor(gfx.getWorld2View2(R, T)).transpose(0, 1)
    P = gfx.getProjectionMatrix(znear=0.01, zfar=100.0, fovX=0.9, fovY=0.7).transpose(0, 1)
    return (W2V.unsqueeze(0).bmm(P.unsqueeze(0))).squeeze(0).float()


def main(ref):
    sys.path.insert(0, ref)
    install_stubs()
    rng = np.random.default_rng(77)
    out = {}
    with CpuRedirect():
        import utils.graphics_utils as gfx
        script = torch.jit.script
        torch.jit.script = lambda f: f   # in_frustum as plain Python
        try:
            import scene.gaussian_geo_model_mlp_flex_colmap as cm
        finally:
            torch.jit.script = script
        from geo.flexicubes_no_adjacent import FlexiCubes

        full = camera(gfx, rng)
        out["full_proj"] = full.numpy()
        fc = FlexiCubes(device="cpu")
        res = (20, 18, 16)
        lo, hi = [-1.1, -1.0, -1.2], [1.2, 1.1, 1.0]
        verts = fc.construct_voxel_grid_vert_only(list(res), lo, hi)
        cube_len = (hi[0] - lo[0]) / res[0]
        out.update({"res": np.array(res), "lo": np.array(lo), "hi": np.array(hi),
                    "verts": verts.numpy(), "cube_len": np.float64(cube_len)})
        for pid, npc in PIECES:
            m = cm.in_frustum(full, verts, cube_len, pid, npc)
            out[f"mask_{pid}_{npc}"] = m.numpy()
        s0 = torch.tensor(shape_sdf(verts.numpy().astype(np.float64)) + 3.7e-4, dtype=torch.float32)
        x0 = verts + torch.tensor(rng.uniform(-0.15, 0.15, verts.shape) * cube_len, dtype=torch.float32)
        out["s"] = s0.numpy()
        out["x"] = x0.numpy()
        noise = torch.tensor(rng.standard_normal(verts.shape[0]), dtype=torch.float32)
        out["noise"] = noise.numpy()
        cases = [("view", out["mask_-1_0"], s0, True), ("half", out["mask_1_2"], s0, False),
                 ("quarter", out["mask_2_4"], s0, True), ("fullnoise", None, noise, True)]
        for tag, mask, sfield, training in cases:
            if mask is None:
                cubes = fc.construct_cubes(torch.ones(verts.shape[0], dtype=torch.bool), list(res))
            else:
                cubes = fc.construct_cubes(torch.tensor(mask), list(res))
            x = x0.clone().requires_grad_(True)
            s = sfield.clone().requires_grad_(True)
            v, f, L, se = fc(x, s, cubes, list(res), training=training, de_ambiguity=False)
            gv = torch.tensor(rng.normal(0, 1, tuple(v.shape)), dtype=torch.float32)
            gl = torch.tensor(rng.normal(0, 1, tuple(L.shape)), dtype=torch.float32)
            ((v * gv).sum() + (L * gl).sum()).backward()
            out.update({f"{tag}/cubes": cubes.numpy().astype(np.int64), f"{tag}/training": np.array(training),
                        f"{tag}/v": v.detach().numpy(), f"{tag}/f": f.numpy(), f"{tag}/L": L.detach().numpy(),
                        f"{tag}/se": se.numpy(), f"{tag}/gv": gv.numpy(), f"{tag}/gl": gl.numpy(),
                        f"{tag}/dx": x.grad.numpy(), f"{tag}/ds": s.grad.numpy()})

        # binding of the real-scene model: renew_gaussian on a fixed mesh
        mverts, mfaces = small_mesh(seed=3)
        for G in (3, 6):
            for adaptive in (True, False):
                m = cm.GaussianGeoModel(3, G, 2.0)
                m.spatial_lr_scale = 2.5
                m.adaptive_cov = adaptive
                m.warm_up = False
                m.train_fg = m.train_bg = True
                vt = torch.tensor(mverts, requires_grad=True)
                ft = torch.tensor(mfaces)
                m.getMesh_full = lambda vt=vt, ft=ft: (vt, ft, torch.tensor([ft.shape[0], 0]), None, None)
                m.mlp_texture = types.SimpleNamespace(sample_noact=lambda p: torch.zeros(p.shape[0], 48))
                info = m.renew_gaussian(train_mesh=True)
                xyz, covar = info["xyz"], info["covariance"]
                gx = torch.tensor(rng.normal(0, 1, tuple(xyz.shape)), dtype=torch.float32)
                gc = torch.tensor(rng.normal(0, 1, tuple(covar.shape)), dtype=torch.float32)
                ((xyz * gx).sum() + (covar * gc).sum()).backward()
                tag = f"bind_G{G}_{'a' if adaptive else 'n'}"
                out.update({f"{tag}/bc": m.bc_coords.numpy(), f"{tag}/rad": np.float64(m.rad_base),
                            f"{tag}/xyz": xyz.detach().numpy(), f"{tag}/cov": covar.detach().numpy(),
                            f"{tag}/gxyz": gx.numpy(), f"{tag}/gcov": gc.numpy(),
                            f"{tag}/dverts": vt.grad.numpy()})
        out["mesh_verts"], out["mesh_faces"] = mverts, mfaces
    np.savez_compressed(os.path.join(HERE, "colmap_golden.npz"), **out)
    print("colmap golden vectors written to", HERE)


if __name__ == "__main__":
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMGS_REFERENCE_TREE")
    if not ref_tree:
        sys.exit(f"usage: python {os.path.basename(__file__)} <reference tree> "
                 "(or set DMGS_REFERENCE_TREE)")
    main(ref_tree)
