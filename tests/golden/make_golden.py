"""Generate golden vectors from the reference's own Python code.

Run in the build container (where the reference tree is mounted):

    python tests/golden/make_golden.py [/path/to/reference]

The reference modules are imported unmodified.  Their hard-coded CUDA
device use is redirected to the CPU by a TorchFunctionMode, and the
third-party modules they import but this path does not use (PIL, plyfile,
trimesh, open3d, point_cloud_utils, tinycudann, torch_scatter, simple_knn,
pytorch3d) are replaced by empty stub modules.  Outputs (small .npz files
next to this script) pin:

  sh_golden.npz       utils/sh_utils.py:25-110  eval_sh, degrees 0..3
  rot_golden.npz      utils/general_utils.py:64-110  build_rotation,
                      build_scaling_rotation, strip_symmetric
  camera_golden.npz   utils/graphics_utils.py:38-71, scene/cameras.py:54-57
  binding_golden.npz  scene/gaussian_geo_model_mlp_flex.py:258-385
                      (renew_gaussian + get_covariance_dyn, forward and
                      autograd gradients w.r.t. verts and scale_factor)
  binding3_golden.npz scene/gaussian_geo_model_finetune.py:396-421,446-483
                      (renew_gaussian xyz, get_scaling, get_rot_matrix)
"""
from __future__ import annotations

import contextlib
import os
import sys
import types

import numpy as np
import torch
from torch.overrides import TorchFunctionMode

HERE = os.path.dirname(os.path.abspath(__file__))


class CpuRedirect(TorchFunctionMode):
    """Rewrites device='cuda' arguments and .cuda() calls to the CPU."""

    def __torch_function__(self, func, types_, args=(), kwargs=None):
        kwargs = dict(kwargs or {})
        if func in (torch.Tensor.cuda,):
            return args[0]
        if func is torch.Tensor.to:
            args = tuple("cpu" if (isinstance(a, (str, torch.device)) and str(a).startswith("cuda")) else a
                         for a in args)
        dev = kwargs.get("device")
        if dev is not None and str(dev).startswith("cuda"):
            kwargs["device"] = "cpu"
        return func(*args, **kwargs)


def _stub(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    return m


def install_stubs():
    @contextlib.contextmanager
    def count_time(name):
        yield
    for n in ["PIL", "PIL.Image", "plyfile", "trimesh", "open3d", "point_cloud_utils",
              "tinycudann", "torch_scatter", "simple_knn", "simple_knn._C",
              "pytorch3d", "pytorch3d.loss", "pytorch3d.structures", "pytorch3d.transforms"]:
        _stub(n)
    sys.modules["plyfile"].PlyData = object
    sys.modules["plyfile"].PlyElement = object
    sys.modules["torch_scatter"].scatter_add = None
    sys.modules["pytorch3d.loss"].mesh_laplacian_smoothing = None
    sys.modules["pytorch3d.loss"].mesh_normal_consistency = None
    sys.modules["pytorch3d.structures"].Meshes = None
    sys.modules["pytorch3d.transforms"].matrix_to_quaternion = None
    sys.modules["simple_knn._C"].distCUDA2 = None
    sys.modules["open3d"].utility = types.SimpleNamespace(
        set_verbosity_level=lambda *a: None,
        VerbosityLevel=types.SimpleNamespace(Error=0))
    eff = _stub("utils.effi_utils", count_time=count_time)
    return eff


def small_mesh(seed=0):
    """A closed, irregular triangle mesh: a subdivided icosahedron with
    jittered vertices (irregular triangles exercise the affine covariance)."""
    t = (1.0 + 5 ** 0.5) / 2
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = np.array(V, np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array(F, np.int64)
    # one level of midpoint subdivision -> 80 faces
    edge_mid = {}
    verts = list(V)
    def mid(a, b):
        k = (min(a, b), max(a, b))
        if k not in edge_mid:
            m = (verts[a] + verts[b]) / 2
            verts.append(m / np.linalg.norm(m))
            edge_mid[k] = len(verts) - 1
        return edge_mid[k]
    nf = []
    for a, b, c in F:
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
    V = np.array(verts)
    rng = np.random.default_rng(seed)
    V = V * 0.7 + rng.normal(0, 0.03, V.shape)
    return V.astype(np.float32), np.array(nf, np.int64)


def main(ref):
    sys.path.insert(0, ref)
    install_stubs()
    rng = np.random.default_rng(1234)
    with CpuRedirect():
        import utils.sh_utils as shu
        import utils.general_utils as gu
        import utils.graphics_utils as gfx
        import geo.mesh_utils as mu

        # --- SH ---
        n = 64
        sh = rng.normal(0, 0.5, (n, 3, 16)).astype(np.float32)
        dirs = rng.normal(0, 1, (n, 3))
        dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
        out = {"sh": sh, "dirs": dirs}
        for d in range(4):
            out[f"deg{d}"] = shu.eval_sh(d, torch.tensor(sh), torch.tensor(dirs)).numpy()
        np.savez(os.path.join(HERE, "sh_golden.npz"), **out)

        # --- rotation / covariance packing ---
        q = rng.normal(0, 1, (n, 4)).astype(np.float32)
        s = np.exp(rng.uniform(-3, 0, (n, 3))).astype(np.float32)
        R = gu.build_rotation(torch.tensor(q)).numpy()
        L = gu.build_scaling_rotation(torch.tensor(s), torch.nn.functional.normalize(torch.tensor(q))).numpy()
        Lt = torch.tensor(L)
        cov = gu.strip_symmetric(Lt @ Lt.transpose(1, 2)).numpy()
        np.savez(os.path.join(HERE, "rot_golden.npz"), q=q, s=s, R=R, L=L, cov=cov)

        # --- camera matrices ---
        cams = {}
        for i in range(3):
            Rm = np.linalg.qr(rng.normal(0, 1, (3, 3)))[0]
            if np.linalg.det(Rm) < 0:
                Rm[:, 0] *= -1
            T = rng.normal(0, 2, 3)
            fovx, fovy = rng.uniform(0.6, 1.2), rng.uniform(0.5, 1.0)
            W2V = torch.tensor(gfx.getWorld2View2(Rm, T)).transpose(0, 1)
            Pm = gfx.getProjectionMatrix(znear=0.01, zfar=100.0, fovX=fovx, fovY=fovy).transpose(0, 1)
            full = W2V.unsqueeze(0).bmm(Pm.unsqueeze(0)).squeeze(0)
            center = W2V.inverse()[3, :3]
            cams.update({f"R{i}": Rm, f"T{i}": T, f"fovx{i}": fovx, f"fovy{i}": fovy,
                         f"view{i}": W2V.numpy(), f"proj{i}": Pm.numpy(), f"full{i}": full.numpy(),
                         f"center{i}": center.numpy()})
        np.savez(os.path.join(HERE, "camera_golden.npz"), **cams)

        # --- stage-2 binding ---
        import scene.gaussian_geo_model_mlp_flex as flex
        verts, faces = small_mesh()
        out = {"verts": verts, "faces": faces}
        for G in (1, 3, 6):
            for adaptive in (True, False):
                m = flex.GaussianGeoModel(3, G, 2.0)
                m.spatial_lr_scale = 4.0
                m.max_scale = 2.0
                m.scale_factor = torch.nn.Parameter(torch.tensor([0.37]))
                m.adaptive_cov = adaptive
                vt = torch.tensor(verts, requires_grad=True)
                ft = torch.tensor(faces)
                m.getMesh = lambda vt=vt, ft=ft: (vt, ft, torch.zeros(()), torch.zeros(()))
                m.mlp_texture = types.SimpleNamespace(
                    sample_noact=lambda x: torch.zeros(x.shape[0], 48))
                info = m.renew_gaussian(train_mesh=True)
                xyz, covar = info["xyz"], info["covariance"]
                gx = torch.tensor(rng.normal(0, 1, tuple(xyz.shape)), dtype=torch.float32)
                gc = torch.tensor(rng.normal(0, 1, tuple(covar.shape)), dtype=torch.float32)
                loss = (xyz * gx).sum() + (covar * gc).sum()
                loss.backward()
                tag = f"G{G}_{'a' if adaptive else 'n'}"
                out.update({f"{tag}_bc": m.bc_coords.numpy(), f"{tag}_rad": np.float64(m.rad_base),
                            f"{tag}_xyz": xyz.detach().numpy(), f"{tag}_cov": covar.detach().numpy(),
                            f"{tag}_covL": info["cov3D_L"].numpy(), f"{tag}_gxyz": gx.numpy(),
                            f"{tag}_gcov": gc.numpy(), f"{tag}_dverts": vt.grad.numpy(),
                            f"{tag}_dsf": m.scale_factor.grad.numpy()})
        np.savez(os.path.join(HERE, "binding_golden.npz"), **out)

        # --- stage-3 binding (pytorch3d-free parts) ---
        import scene.gaussian_geo_model_finetune as ft3
        m = ft3.GaussianGeoModel.__new__(ft3.GaussianGeoModel)
        G = 3
        m.bc_coords, m.rad_base = mu.generate_barycentric_v2(G, "cpu")
        m.N_gs_per_face = G
        m.eval = False
        m.use_frustum = False
        m.verts = torch.tensor(verts, requires_grad=True)
        m.faces = torch.tensor(faces)
        m._rotation = torch.tensor(rng.normal(0, 1, (faces.shape[0] * G, 2)), dtype=torch.float32)
        m._scaling = torch.tensor(rng.normal(-4, 0.5, (faces.shape[0] * G, 2)), dtype=torch.float32)
        m.scaling_activation = torch.exp
        m.thin_z_scale = 1e-6
        m.gs_mask = None
        m.rot_t2w = None
        m._xyz = None
        m.renew_gaussian()
        R = m.get_rot_matrix()
        sc = m.get_scaling
        np.savez(os.path.join(HERE, "binding3_golden.npz"), verts=verts, faces=faces,
                 bc=m.bc_coords.numpy(), rotation2d=m._rotation.numpy(),
                 scaling2d=m._scaling.numpy(), xyz=m._xyz.detach().numpy(),
                 R=R.detach().numpy(), scales=sc.detach().numpy(), thin_z=1e-6)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMGS_REFERENCE_TREE")
    if not ref_tree:
        sys.exit(f"usage: python {os.path.basename(__file__)} <reference tree> "
                 "(or set DMGS_REFERENCE_TREE)")
    main(ref_tree)
