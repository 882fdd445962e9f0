"""Golden vectors for FlexiCubes from the reference's own class.

Run in the build container (where the reference tree is mounted):

    python tests/golden/make_flexicubes_golden.py [/path/to/reference]

Imports ``geo/flexicubes.py`` (and ``geo/tables.py``) unmodified and runs
``FlexiCubes(device='cpu')`` in float32 (the class hard-codes float32
buffers, so float64 is not possible) on small regular grids made by its own
``construct_voxel_grid_v2``.  Stores inputs, the four outputs and, for the
training-mode cases, autograd gradients of a fixed random linear loss of the
outputs w.r.t. the vertex positions, the scalar field and the three raw
weight sets.  Output: ``flexicubes_golden.npz`` next to this script, with
keys ``<case>/<name>``.

Cases
-----
shape    sphere (r 0.6) union torus (R 0.7, r 0.2) SDF on a 9x10x11 grid over
         [-1,1]^3, deformed vertices, random weights, training=True
noise    N(0,1) scalar field on a 6x7x5 grid (many ambiguous C16/C19 cubes),
         random weights, training=True
plain    the shape case without weights or deformation, training=False
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def shape_sdf(p):
    """Signed distance of sphere(0.6) union torus(R 0.7, r 0.2) about z."""
    sphere = np.linalg.norm(p, axis=1) - 0.6
    q = np.stack([np.hypot(p[:, 0], p[:, 1]) - 0.7, p[:, 2]], 1)
    torus = np.linalg.norm(q, axis=1) - 0.2
    return np.minimum(sphere, torus)


def run_case(fc, res, seed, field, weights, training, deform):
    torch.manual_seed(seed)
    rng = np.random.default_rng(seed)
    verts, cubes = fc.construct_voxel_grid_v2(list(res), [-1.0, -1.0, -1.0], [1.0, 1.0, 1.0])
    C = cubes.shape[0]
    if field == "shape":
        s = torch.tensor(shape_sdf(verts.numpy().astype(np.float64)), dtype=torch.float32)
    else:
        s = torch.tensor(rng.standard_normal(verts.shape[0]), dtype=torch.float32)
    x = verts.clone()
    if deform:
        cube = 2.0 / max(res)
        x = x + torch.tensor(rng.uniform(-0.2, 0.2, x.shape) * cube, dtype=torch.float32)
    x.requires_grad_(True)
    s.requires_grad_(True)
    out = {"res": np.array(res), "x": x.detach().numpy(), "s": s.detach().numpy(),
           "cubes": cubes.numpy().astype(np.int64), "training": np.array(training)}
    w = None
    if weights:
        w = [torch.tensor(rng.normal(0, 0.7, shp), dtype=torch.float32, requires_grad=True)
             for shp in ((C, 12), (C, 8), (C,))]
        out.update(beta=w[0].detach().numpy(), alpha=w[1].detach().numpy(), gamma=w[2].detach().numpy())
    verts_o, faces, L_dev, surf_edges = fc(x, s, cubes, list(res), *(w or (None, None, None)),
                                           training=training)
    out.update(vertices=verts_o.detach().numpy(), faces=faces.numpy().astype(np.int64),
               L_dev=L_dev.detach().numpy(), surf_edges=surf_edges.numpy().astype(np.int64))
    if training:
        gv = torch.tensor(rng.standard_normal(verts_o.shape), dtype=torch.float32)
        gl = torch.tensor(rng.standard_normal(L_dev.shape), dtype=torch.float32)
        loss = (verts_o * gv).sum() + (L_dev * gl).sum()
        inputs = [x, s] + (w or [])
        grads = torch.autograd.grad(loss, inputs, allow_unused=True)
        names = ["dx", "ds", "dbeta", "dalpha", "dgamma"]
        out.update(up_vertices=gv.numpy(), up_L_dev=gl.numpy())
        for n, g in zip(names, grads):
            out[n] = (g if g is not None else torch.zeros_like(inputs[names.index(n)])).numpy()
    return out


def main(ref):
    sys.path.insert(0, ref)
    from geo.flexicubes import FlexiCubes
    fc = FlexiCubes(device="cpu")
    cases = {
        "shape": run_case(fc, (9, 10, 11), 1, "shape", True, True, True),
        "noise": run_case(fc, (6, 7, 5), 2, "noise", True, True, True),
        "plain": run_case(fc, (9, 10, 11), 3, "shape", False, False, False),
    }
    flat = {f"{c}/{k}": v for c, d in cases.items() for k, v in d.items()}
    path = os.path.join(HERE, "flexicubes_golden.npz")
    np.savez_compressed(path, **flat)
    for c, d in cases.items():
        print(c, "vertices", d["vertices"].shape, "faces", d["faces"].shape,
              "surf_edges", d["surf_edges"].shape)
    print("wrote", path)


if __name__ == "__main__":
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMGS_REFERENCE_TREE")
    if not ref_tree:
        sys.exit(f"usage: python {os.path.basename(__file__)} <reference tree> "
                 "(or set DMGS_REFERENCE_TREE)")
    main(ref_tree)
