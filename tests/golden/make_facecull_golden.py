"""Golden vectors for the stage-3 frustum face culling from the reference's
own ``in_frustum`` (scene/gaussian_geo_model_finetune.py:33-48) applied to
face centroids as its ``renew_gaussian`` does (:405-409), run on the CPU
(float32, the reference's dtype).

    python tests/golden/make_facecull_golden.py [/path/to/reference]

The module's heavy imports are stubbed as in make_golden.py.  Mesh: 4,000
random triangles with vertices in [-2, 2]^3; cameras: three views at
distance 3 (the repository's camera helper, whose matrices follow the
reference's conventions, pinned by camera_golden.npz).  Output:
``facecull_golden.npz``: vertices, faces, per camera the full projection
matrix and the reference's face mask.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from dmgs_gb300.camera import make_view  # noqa: E402
from tests.golden.make_golden import CpuRedirect, install_stubs  # noqa: E402


def main(ref):
    sys.path.insert(0, ref)
    install_stubs()
    rng = np.random.default_rng(77)
    verts = rng.uniform(-2.0, 2.0, (3000, 3)).astype(np.float32)
    faces = rng.integers(0, len(verts), (4000, 3)).astype(np.int64)
    out = {"verts": verts, "faces": faces}
    with CpuRedirect():
        from scene.gaussian_geo_model_finetune import in_frustum
        v, f = torch.tensor(verts), torch.tensor(faces)
        centroids = v[f].mean(dim=1)
        for i, (eye, fov) in enumerate([((3.0, 0.5, 0.2), 50), ((-1.0, 2.5, 1.4), 70),
                                        ((0.3, -0.4, -3.0), 35)]):
            view = make_view(eye, (0.0, 0.0, 0.0), 320, 240, fovx_deg=fov)
            M = torch.tensor(np.asarray(view.projmatrix, np.float32))
            mask = in_frustum(M, centroids)
            out[f"proj{i}"] = M.numpy()
            out[f"mask{i}"] = mask.numpy()
            print(i, int(mask.sum()), "of", len(faces))
    np.savez_compressed(os.path.join(HERE, "facecull_golden.npz"), n=np.int64(3), **out)


if __name__ == "__main__":
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMGS_REFERENCE_TREE")
    if not ref_tree:
        sys.exit(f"usage: python {os.path.basename(__file__)} <reference tree> "
                 "(or set DMGS_REFERENCE_TREE)")
    main(ref_tree)
