"""Camera matrices in the reference's conventions.

The reference builds ``world_view_transform = getWorld2View2(R, T).T``,
``projection_matrix = getProjectionMatrix(znear, zfar, fovX, fovY).T`` and
``full_proj_transform = world_view_transform @ projection_matrix``
(``scene/cameras.py:54-57``, ``utils/graphics_utils.py:38-71``): row-vector
(transposed) storage, camera axes x right / y down / z forward,
z-near 0.01, z-far 100.  This module produces the same matrices from a
look-at description.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def _normalize(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def look_at_rotation(eye, target, up=(0.0, 1.0, 0.0)):
    """Camera-to-world rotation (columns: right, down, forward)."""
    f = _normalize(np.asarray(target, np.float64) - np.asarray(eye, np.float64))
    r = np.cross(f, np.asarray(up, np.float64))
    if np.linalg.norm(r) < 1e-9:  # looking along `up`
        r = np.cross(f, np.array([0.0, 0.0, 1.0]))
    r = _normalize(r)
    d = np.cross(f, r)
    return np.stack([r, d, f], 1)


def world_to_view(R, eye):
    """4x4 world->view matrix [[R^T, -R^T eye], [0, 0, 0, 1]] (math convention)."""
    Rt = np.eye(4)
    Rt[:3, :3] = R.T
    Rt[:3, 3] = -R.T @ np.asarray(eye, np.float64)
    return Rt


def projection(znear, zfar, fovx, fovy):
    """Perspective matrix of the reference (math convention, z in [0, 1])."""
    P = np.zeros((4, 4))
    P[0, 0] = 1.0 / math.tan(fovx / 2)
    P[1, 1] = 1.0 / math.tan(fovy / 2)
    P[3, 2] = 1.0
    P[2, 2] = zfar / (zfar - znear)
    P[2, 3] = -(zfar * znear) / (zfar - znear)
    return P


@dataclass
class ViewSpec:
    width: int
    height: int
    fovx: float
    fovy: float
    viewmatrix: np.ndarray   # [4,4] float32, transposed storage
    projmatrix: np.ndarray   # [4,4] float32, transposed storage (full projection)
    campos: np.ndarray       # [3] float32

    @property
    def tanfovx(self):
        return math.tan(self.fovx * 0.5)

    @property
    def tanfovy(self):
        return math.tan(self.fovy * 0.5)


def make_view(eye, target, width, height, fovx_deg=None, fovy_deg=None, up=(0.0, 1.0, 0.0),
              znear=0.01, zfar=100.0) -> ViewSpec:
    """A camera at `eye` looking at `target`.  Give fovx or fovy (degrees);
    the other follows the aspect ratio through the focal length."""
    if fovx_deg is not None:
        fovx = math.radians(fovx_deg)
        focal = width / (2 * math.tan(fovx / 2))
        fovy = 2 * math.atan(height / (2 * focal))
    else:
        fovy = math.radians(fovy_deg)
        focal = height / (2 * math.tan(fovy / 2))
        fovx = 2 * math.atan(width / (2 * focal))
    R = look_at_rotation(eye, target, up)
    W2V = world_to_view(R, eye)
    Pm = projection(znear, zfar, fovx, fovy)
    view_t = W2V.T.astype(np.float32)
    full_t = (Pm @ W2V).T.astype(np.float32)
    return ViewSpec(width, height, fovx, fovy, view_t, full_t,
                    np.asarray(eye, np.float32).copy())
