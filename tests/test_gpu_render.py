"""The CUDA render pass (bcmc_render through the C ABI) against the oracle's
restatement: the triangle and depth buffers bit for bit, the colours within
1e-5 (the only differences are the CUDA and C library expf/powf, each within
a few ulp), on the ct44 mesh from several views, with and without fog, on
views close enough that triangles take the CTA-per-triangle path, and on the
hand-made scenes of the CPU tests."""
import os

import numpy as np
import pytest

import bcmc
import render_scenes as S
from bcmc import camera
from gpu_util import to_dev

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BG = np.uint32(0xFFFFFFFF)
COLOUR_TOL = 1e-5


def _check(ctx, oracle, verts, dims, proj, eye, w, h, scale, fog):
    want_rgba, want_depth, want_tri = oracle.render(verts, dims, proj, eye, w, h, scale, fog)
    d = to_dev(np.ascontiguousarray(verts, np.uint32).reshape(-1, 2)) if len(verts) else to_dev(
        np.zeros((1, 2), np.uint32))
    rgba, depth, tri = bcmc.render(ctx, d, len(verts), dims, proj, eye, w, h, scale, fog)
    got_tri = tri.cpu().numpy().view(np.uint32)
    assert np.array_equal(got_tri, want_tri)
    assert np.array_equal(depth.cpu().numpy().view(np.uint32), want_depth.view(np.uint32))
    got = rgba.cpu().numpy()
    assert np.isfinite(got).all()
    assert np.abs(got - want_rgba).max() <= COLOUR_TOL
    return got_tri


def _mesh(name="mc_ct44_r4.npz"):
    m = np.load(os.path.join(GOLDEN, name))
    return m["vertices_0"], tuple(int(d) for d in m["dims"])


@pytest.mark.parametrize("fog", [False, True])
@pytest.mark.parametrize("view", [((0.0, 0.0, 1.0), (1.0, 1.0, 1.0)), ((0.3, 0.4, 1.2), (1.0, 0.9, 0.8)),
                                  ((-0.9, 0.6, -0.7), (0.7, 1.3, 1.0))])
def test_render_matches_oracle(ctx, oracle, fog, view):
    verts, dims = _mesh()
    eye, scale = view
    w, h = 160, 120
    proj, eye = camera.default_view(w, h, eye=eye)
    tri = _check(ctx, oracle, verts, dims, proj, eye, w, h, scale, fog)
    assert (tri != BG).sum() > 500


def test_large_triangles_take_the_cta_path(ctx, oracle):
    """A 5 degree field of view: triangles cover up to thousands of pixels
    (more than 256 goes to one CTA per triangle)."""
    verts, dims = _mesh("mc_blobs32_r8.npz")
    w, h = 320, 240
    proj, eye = camera.default_view(w, h, eye=(0.3, 0.2, 1.0), fovy_deg=5.0)
    tri = _check(ctx, oracle, verts, dims, proj, eye, w, h, (1.0, 1.0, 1.0), True)
    ids, counts = np.unique(tri[tri != BG], return_counts=True)
    assert counts.max() > 256


def test_scenes_match_oracle(ctx, oracle):
    for verts in (S.fan(3), S.fan(13), S.quad(-0.5, -0.5, 0.5, 0.5), S.overlap_pair(0.3, 0.6),
                  S.overlap_pair(0.6, 0.3), np.concatenate([S.fan(5), S.fan(5)]), S.fan(6, z=1.1),
                  S.fan(6, z=-0.2)):
        for w, h in ((97, 71), (1, 1), (3, 200)):
            _check(ctx, oracle, verts, S.DIMS, S.IDENTITY, S.EYE, w, h, S.SCALE, False)
    flip = np.diag([1.0, 1.0, 1.0, -1.0]).astype(np.float32).reshape(16)
    tri = _check(ctx, oracle, S.fan(6), S.DIMS, flip, S.EYE, 64, 48, S.SCALE, True)
    assert (tri == BG).all()


def test_empty_and_ragged(ctx, oracle):
    _check(ctx, oracle, np.zeros((0, 2), np.uint32), S.DIMS, S.IDENTITY, S.EYE, 33, 17, S.SCALE, True)
    tri = _check(ctx, oracle, S.fan(4)[:11], S.DIMS, S.IDENTITY, S.EYE, 64, 48, S.SCALE, False)
    assert set(np.unique(tri)) <= {0, 1, 2, BG}  # the 11th and 12th vertices make no triangle


def test_bad_arguments(ctx):
    d = to_dev(S.fan(2))
    for w, h in ((0, 10), (10, 0), (20000, 10)):
        with pytest.raises(bcmc.BcmcError):
            bcmc.render(ctx, d, 6, S.DIMS, S.IDENTITY, S.EYE, w, h, S.SCALE)
    # the context stays usable
    rgba, _, _ = bcmc.render(ctx, d, 6, S.DIMS, S.IDENTITY, S.EYE, 8, 8, S.SCALE)
    assert rgba.shape == (8, 8, 4)
