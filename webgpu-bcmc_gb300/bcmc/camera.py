"""View matrices for the render pass, in the column-major float32 layout the
reference's ViewParams.proj_view has (gl-matrix's mat4.perspective,
mat4.lookAt and mat4.mul, js/bcmc.js:110-125,291), computed in float64 and
stored as float32 the way gl-matrix stores them."""
from __future__ import annotations

import math

import numpy as np


def perspective(fovy: float, aspect: float, near: float, far: float) -> np.ndarray:
    """OpenGL-style projection (depth -1..1 before WebGPU's 0..1 clip), 4x4 row-major view of a column-major array."""
    f = 1.0 / math.tan(fovy / 2.0)
    m = np.zeros(16, np.float64)
    m[0] = f / aspect
    m[5] = f
    m[10] = (far + near) / (near - far)
    m[11] = -1.0
    m[14] = 2.0 * far * near / (near - far)
    return m.astype(np.float32)


def look_at(eye, center, up) -> np.ndarray:
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    z = eye - center
    z /= np.linalg.norm(z)
    x = np.cross(up, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    m = np.zeros(16, np.float64)
    m[0], m[4], m[8] = x
    m[1], m[5], m[9] = y
    m[2], m[6], m[10] = z
    m[12], m[13], m[14] = -x @ eye, -y @ eye, -z @ eye
    m[15] = 1.0
    return m.astype(np.float32)


def mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """a * b for column-major 16-element arrays."""
    A = np.asarray(a, np.float64).reshape(4, 4).T
    B = np.asarray(b, np.float64).reshape(4, 4).T
    return (A @ B).T.reshape(16).astype(np.float32)


def default_view(width: int, height: int, eye=(0.0, 0.0, 1.0), center=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                 fovy_deg: float = 50.0):
    """The reference's starting view (js/bcmc.js:110-124): eye at +z looking at
    the origin, 50 degree vertical field of view, near 0.01, far 1000.
    Returns (proj_view[16] column-major float32, eye[3] float32)."""
    proj = perspective(fovy_deg * math.pi / 180.0, width / height, 0.01, 1000.0)
    return mul(proj, look_at(eye, center, up)), np.asarray(eye, np.float32)
