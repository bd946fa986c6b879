"""Small hand-made scenes for the render pass tests: packed vertices of a
one-block volume (dims 4x4x4, scale 2), whose world positions reach
[-0.75, 1.25] on each axis; with the identity view matrix the world position
is the clip position (w = 1), so x/y are NDC and z is the depth."""
import numpy as np

DIMS = (4, 4, 4)
SCALE = (2.0, 2.0, 2.0)
IDENTITY = np.eye(4, dtype=np.float32).reshape(16)
EYE = (0.0, 0.0, -2.0)


def q_of(w: float) -> int:
    """the 10-bit quantised in-block position whose world coordinate is nearest w"""
    q = round(((w / 2.0 + 0.5) * 4.0 - 0.5) * 1023.0 / 4.0)
    assert 0 <= q <= 1023, w
    return q


def pack(points) -> np.ndarray:
    """points: [n, 3] world positions -> [n, 2] u32 packed vertices of block 0"""
    out = np.zeros((len(points), 2), np.uint32)
    for i, (x, y, z) in enumerate(points):
        out[i, 0] = (q_of(x) << 20) | (q_of(y) << 10) | q_of(z)
    return out


def fan(n_tri: int, radius: float = 0.6, z: float = 0.5, cx: float = 0.1, cy: float = -0.05):
    """a closed polygon of n_tri triangles around a centre vertex, as a triangle list"""
    ang = np.linspace(0.0, 2 * np.pi, n_tri + 1)[:-1] + 0.1
    rim = [(cx + radius * np.cos(a), cy + radius * np.sin(a), z) for a in ang]
    pts = []
    for i in range(n_tri):
        pts += [(cx, cy, z), rim[i], rim[(i + 1) % n_tri]]
    return pack(pts)


def overlap_pair(z_first: float, z_second: float):
    """two overlapping triangles at constant depths"""
    a = [(-0.5, -0.5, z_first), (0.5, -0.5, z_first), (0.0, 0.6, z_first)]
    b = [(-0.4, 0.5, z_second), (0.6, 0.4, z_second), (0.1, -0.6, z_second)]
    return pack(a + b)


def quad(x0, y0, x1, y1, z=0.4):
    return pack([(x0, y0, z), (x1, y0, z), (x1, y1, z), (x0, y0, z), (x1, y1, z), (x0, y1, z)])
