"""The headless render pass on the CPU: the oracle's restatement of the
render shaders against the reference's own shaders (golden fixtures from
tests/golden/make_golden.py, and live when the reference checkout is
present), and the rasterisation rules on hand-made scenes.

Pinned bit for bit: the fog vertex stage's t_enter and the fragment shader's
colour.  The rasteriser (pixel centres, 1/256-pixel snapping, top-left rule,
"less" depth test) is the WebGPU pipeline's, not the reference's code, and is
checked through properties: watertight coverage, exactly one triangle per
pixel centre on shared edges, nearest fragment wins, earlier triangle on
ties, nothing behind the eye."""
import os

import numpy as np
import pytest

import render_scenes as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BG = np.uint32(0xFFFFFFFF)


def _golden():
    return np.load(os.path.join(GOLDEN, "render_ct44.npz")), np.load(os.path.join(GOLDEN, "mc_ct44_r4.npz"))


def test_fog_enter_matches_reference_vertex_shader(oracle):
    g, m = _golden()
    dims = tuple(int(d) for d in g["dims"])
    world = oracle.unpack_vertices(m["vertices_0"], dims, tuple(g["scale"]))
    te = oracle.fog_enter(world, g["eye"], tuple(g["scale"]))
    assert np.array_equal(te.view(np.uint32), g["t_enter_bits"])


@pytest.mark.parametrize("fog", [False, True])
def test_shading_matches_reference_fragment_shader(oracle, fog):
    g, m = _golden()
    dims = tuple(int(d) for d in g["dims"])
    world = oracle.unpack_vertices(m["vertices_0"], dims, tuple(g["scale"])).reshape(-1, 3, 3)
    want = g["frag_rgba_fog_bits" if fog else "frag_rgba_bits"]
    for i, t in enumerate(g["frag_tri"]):
        got = oracle.shade(g["frag_world"][i], g["frag_t_enter"][i], g["eye"], world[t], fog)
        assert np.array_equal(got.view(np.uint32), want[i]), i


def test_live_against_reference_render_shaders(oracle):
    import ref

    if not ref.available():
        pytest.skip("reference checkout not present (the golden fixtures cover this)")
    m = np.load(os.path.join(GOLDEN, "mc_blobs32_r8.npz"))
    verts, dims = m["vertices_0"], tuple(int(d) for d in m["dims"])
    rng = np.random.default_rng(5)
    for scale, eye in (((1.0, 1.0, 1.0), (0.0, 0.0, 1.0)), ((0.7, 1.3, 1.0), (-0.8, 0.5, -0.9))):
        world = oracle.unpack_vertices(verts, dims, scale)
        _, te_ref = ref.vert_fog(verts, dims, scale, eye)
        te = oracle.fog_enter(world, eye, scale)
        assert np.array_equal(te.view(np.uint32), te_ref.view(np.uint32))
        tri = rng.integers(0, len(verts) // 3, 200)
        bary = rng.dirichlet((1.0, 1.0, 1.0), 200).astype(np.float32)
        tw = world.reshape(-1, 3, 3)[tri]
        wp = (bary[:, :, None] * tw).sum(1).astype(np.float32)
        fte = (bary * te.reshape(-1, 3)[tri]).sum(1).astype(np.float32)
        for fog in (False, True):
            want = ref.frag(wp, fte, eye, tw[:, 1] - tw[:, 0], tw[:, 2] - tw[:, 0], fog)
            got = np.stack([oracle.shade(wp[i], fte[i], eye, tw[i], fog) for i in range(200)])
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _render(oracle, verts, w=64, h=48, fog=False, proj=S.IDENTITY):
    return oracle.render(verts, S.DIMS, proj, S.EYE, w, h, S.SCALE, fog)


def test_empty_mesh_is_background(oracle):
    rgba, depth, tri = _render(oracle, np.zeros((0, 2), np.uint32))
    assert (rgba == 1.0).all() and (depth == 1.0).all() and (tri == BG).all()
    # trailing vertices that do not make a triangle are ignored
    rgba2, _, tri2 = _render(oracle, S.fan(3)[:2])
    assert (tri2 == BG).all() and (rgba2 == 1.0).all()


@pytest.mark.parametrize("n_tri", [3, 8, 13])
def test_shared_edges_cover_each_pixel_once(oracle, n_tri):
    """Each triangle of a fan drawn alone: the masks are disjoint and their
    union is the whole fan (no pixel centre on a shared edge lost or drawn twice)."""
    verts = S.fan(n_tri)
    w, h = 97, 71
    _, _, all_tri = _render(oracle, verts, w, h)
    count = np.zeros((h, w), np.int32)
    for t in range(n_tri):
        _, _, one = _render(oracle, verts[3 * t: 3 * t + 3], w, h)
        count += one != BG
        assert np.array_equal(one != BG, all_tri == t), t  # same pixels alone as in the fan (constant depth)
    assert count.max() == 1
    assert np.array_equal(count == 1, all_tri != BG)
    # the interior of the fan is closed: every pixel whose centre lies well inside is covered
    ys, xs = np.mgrid[0:h, 0:w]
    nx, ny = (xs + 0.5) / w * 2 - 1, 1 - (ys + 0.5) / h * 2
    inner = np.hypot(nx - 0.1, ny + 0.05) < 0.6 * np.cos(np.pi / n_tri) - 3.0 / min(w, h)
    assert (all_tri[inner] != BG).all()


def test_quad_coverage_is_half_open(oracle):
    """A quad of two triangles with its edges between pixel centres covers
    exactly the pixels whose centres it contains."""
    w = h = 40
    # x in NDC from -0.5 to 0.5 -> screen 10..30: centres 10.5 .. 29.5 inside
    verts = S.quad(-0.5, -0.5, 0.5, 0.5)
    _, _, tri = _render(oracle, verts, w, h)
    cov = tri != BG
    ys, xs = np.nonzero(cov)
    assert cov.sum() == 20 * 20 and xs.min() == 10 and xs.max() == 29 and ys.min() == 10 and ys.max() == 29


@pytest.mark.parametrize("order", [0, 1])
def test_nearest_fragment_wins(oracle, order):
    verts = S.overlap_pair(0.3, 0.6) if order == 0 else S.overlap_pair(0.6, 0.3)
    _, depth, tri = _render(oracle, verts)
    near = 0 if order == 0 else 1
    a, _, ta = _render(oracle, verts[:3])
    b, _, tb = _render(oracle, verts[3:])
    both = (ta != BG) & (tb != BG)
    assert both.sum() > 20
    assert (tri[both] == near).all()
    assert np.allclose(depth[tri != BG], np.where(tri[tri != BG] == near, 0.3, 0.6), atol=2e-3)


def test_ties_go_to_the_earlier_triangle(oracle):
    t = S.overlap_pair(0.4, 0.4)[:3]
    _, _, tri = _render(oracle, np.concatenate([t, t, t]))
    assert (tri[tri != BG] == 0).all() and (tri != BG).sum() > 20


def test_behind_the_eye_and_outside_depth_range_not_drawn(oracle):
    verts = S.fan(6)
    flip = np.diag([1.0, 1.0, 1.0, -1.0]).astype(np.float32).reshape(16)  # w = -1
    _, _, tri = _render(oracle, verts, proj=flip)
    assert (tri == BG).all()
    far = S.fan(6, z=1.1)  # depth >= 1: not less than the cleared depth
    _, _, tri = _render(oracle, far)
    assert (tri == BG).all()
    near = S.fan(6, z=-0.2)  # depth < 0: clipped
    _, _, tri = _render(oracle, near)
    assert (tri == BG).all()


def test_fog_brightens_toward_white(oracle):
    g, m = _golden()
    from bcmc import camera

    dims = tuple(int(d) for d in g["dims"])
    pv, eye = camera.default_view(64, 48, eye=(0.3, 0.4, 1.2))
    plain, d0, t0 = oracle.render(m["vertices_0"], dims, pv, eye, 64, 48, tuple(g["scale"]), False)
    fogged, d1, t1 = oracle.render(m["vertices_0"], dims, pv, eye, 64, 48, tuple(g["scale"]), True)
    assert np.array_equal(t0, t1) and np.array_equal(d0.view(np.uint32), d1.view(np.uint32))
    cov = t0 != BG
    assert cov.sum() > 100
    assert (fogged[cov][:, :3] >= plain[cov][:, :3] - 1e-6).all()
    assert np.isfinite(plain).all() and (plain[cov][:, :3] <= 1.0 + 1e-6).all()
