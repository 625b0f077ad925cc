"""Oracle-level checks on the CPU: known answers and self-consistency of the
restated path (no GPU)."""
import numpy as np
import pytest

import oracle
from barney_gb300 import scenes


def test_render_deterministic_and_threads_independent():
    s = scenes.small_scene(dims=32, spp=3, width=48, height=32)
    o = oracle.Oracle(s)
    a = o.render(nthreads=1)
    b = o.render(nthreads=0)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert o.stats["density_samples"] > 0


def test_background_only_frame():
    """Known answer: a camera looking away sees bgColor with alpha bgColor.w
    on every pass (generateRays.cu:219-230; shadeRays.cu:998-1001)."""
    s = scenes.small_scene(dims=16, spp=5, width=8, height=8)
    s.cam_pos, s.cam_dir = (0.0, 0.0, 3.0), (0.0, 0.0, 1.0)
    s.bg_color = (0.25, 0.5, 0.75, 0.5)
    o = oracle.Oracle(s)
    acc = o.render()
    np.testing.assert_array_equal(acc, np.tile(np.array([1.25, 2.5, 3.75, 2.5], np.float32), (8, 8, 1)))
    img = o.tonemap(acc, 5)
    np.testing.assert_allclose(img, np.tile(np.array([0.25, 0.5, 0.75, 0.5], np.float32), (8, 8, 1)))
    rgba8 = o.tonemap(acc, 5, fmt=1)
    # make_8bit: min(255, int(c*256))
    assert rgba8[0, 0] == (64 | (128 << 8) | (192 << 16) | (128 << 24))


def test_gradient_background_when_bg_alpha_negative():
    s = scenes.small_scene(dims=16, spp=1, width=4, height=4)
    s.cam_pos, s.cam_dir = (0.0, 0.0, 3.0), (0.0, 0.0, 1.0)
    s.bg_color = (0.0, 0.0, 0.0, -1.0)
    acc = oracle.Oracle(s).render()
    t = (np.arange(4) + 0.5) / 4
    exp_r = (1 - t).astype(np.float32) * np.float32(0.9) + t.astype(np.float32) * np.float32(0.15)
    np.testing.assert_allclose(acc[:, 0, 0], exp_r, rtol=1e-6)


def test_ea_beer_lambert():
    vol = np.full((16, 16, 16), 0.5, np.float32)
    tf = np.tile(np.array([[0.2, 0.6, 0.9, 0.4]], np.float32), (4, 1))
    s = scenes.Scene(scalars=vol, tf=tf, base_density=3.0)
    views = [dict(pos=(0.0, 0.0, 2.5), dir=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0), fovy=20.0, width=8, height=8)]
    step = 0.01
    img = oracle.Oracle(s).ea_render(views, step, use_double=True).reshape(8, 8, 4)
    n = sum(1 for i in range(200) if 2.0 + (i + 0.5) * step < 3.0)
    a = 1 - np.exp(-n * 1.2 * step)
    np.testing.assert_allclose(img[3, 3, 3], a, rtol=1e-6)
    np.testing.assert_allclose(img[3, 3, :3], np.array([0.2, 0.6, 0.9]) * a, rtol=1e-6)


def test_ea_gradient_finite_differences():
    gt = scenes.ea_scene(20)
    views = scenes.fibonacci_views(2, 2.5, 20)
    step = 0.5 / 19
    tgt = oracle.Oracle(gt).ea_render(views, step, use_double=True).astype(np.float64)
    start = scenes.Scene(scalars=(0.3 + 0.2 * gt.scalars).astype(np.float32), tf=gt.tf, base_density=gt.base_density)
    o = oracle.Oracle(start)
    img = o.ea_render(views, step, use_double=True).astype(np.float64)
    gv, gtf = o.ea_backward(views, step, (2 * (img - tgt)).astype(np.float32))

    def loss(vol):
        s2 = scenes.Scene(scalars=vol, tf=start.tf, base_density=gt.base_density)
        return ((oracle.Oracle(s2).ea_render(views, step, use_double=True) - tgt) ** 2).sum()

    rng = np.random.default_rng(44)
    flat = start.scalars.reshape(-1)
    sel = np.flatnonzero(np.abs(gv.reshape(-1)) > 1e-2 * np.abs(gv).max())
    fd, an = [], []
    for v in rng.choice(sel, 6, replace=False):
        hi, lo = np.float32(flat[v] + 1e-3), np.float32(flat[v] - 1e-3)
        p, m = flat.copy(), flat.copy()
        p[v], m[v] = hi, lo
        fd.append((loss(p.reshape(start.scalars.shape)) - loss(m.reshape(start.scalars.shape))) /
                  (float(hi) - float(lo)))
        an.append(gv.reshape(-1)[v])
    fd, an = np.array(fd), np.array(an)
    assert np.linalg.norm(fd - an) <= 1e-3 * np.linalg.norm(fd)


def test_env_cdfs_monotone():
    s = scenes.small_scene(dims=8)
    s.env = scenes.env_sky(64, 32)
    cy, cx = oracle.Oracle(s).env_cdfs()
    assert np.all(np.diff(cy) >= 0) and cy[-1] == 1.0
    cx = cx.reshape(32, 64)
    assert np.all(np.diff(cx, axis=1) >= 0) and np.all(cx[:, -1] == 1.0)


def test_multi_scatter_adds_light():
    """Scattering more than once can only add energy to the single-scatter
    image in expectation (same scene, same lights)."""
    s = scenes.frame_scene(dims=32, width=24, height=24, spp=32, with_env=False)
    s.max_volume_bounces = 0
    a = oracle.Oracle(s).render()[..., :3].mean()
    s.max_volume_bounces = 4
    b = oracle.Oracle(s).render()[..., :3].mean()
    assert b > a


def test_iso_plane_of_a_linear_field():
    """v(x, y, z) = x + 0.5 on the unit cube: the iso surface v = c is the
    plane x = c - 0.5, and trilinear interpolation of a linear field is
    exact, so rays hit it at the analytic t with normal +x."""
    n = 33
    x = np.linspace(-0.5, 0.5, n, dtype=np.float64)
    vol = np.broadcast_to((x + 0.5)[None, None, :], (n, n, n)).astype(np.float32).copy()
    s = scenes.Scene(scalars=vol, tf=scenes.tf_ramp(16), cells_per_mc=8)
    o = oracle.Oracle(s)
    rng = np.random.default_rng(0)
    k = 200
    # rays from x = -0.7 that stay inside |y|, |z| < 0.5 up to the far face
    org = np.stack([np.full(k, -0.7), rng.uniform(-0.3, 0.3, k), rng.uniform(-0.3, 0.3, k)], 1)
    d = np.stack([np.ones(k), rng.uniform(-0.1, 0.1, k), rng.uniform(-0.1, 0.1, k)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((k, 8), np.float32)
    rays[:, 0:3], rays[:, 3], rays[:, 4:7] = org, 1e30, d
    for c in (0.25, 0.5, 0.8):
        h = o.iso_intersect(rays, c, ranges=o.mc_ranges())
        assert h[:, 7].all()
        t_exact = ((c - 0.5) - org[:, 0]) / d[:, 0]
        np.testing.assert_allclose(h[:, 0], t_exact, rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(h[:, 1], c - 0.5, atol=2e-6)
        np.testing.assert_allclose(h[:, 4:7], np.tile([1.0, 0.0, 0.0], (k, 1)), atol=1e-5)
    # the plane lies outside [0, 1]: no hit
    assert not o.iso_intersect(rays, 1.5, ranges=o.mc_ranges())[:, 7].any()


def test_u8_storage_form_of_the_oracle():
    """The oracle's U8 storage form: every corner is within half a step of
    its scale brick (span/510) of the voxel, so samples are too; macrocell
    ranges bound every sample inside the macrocell; a constant scale brick
    (span 0) reads back exactly."""
    s = scenes.small_scene(dims=37, spp=1, width=24, height=16)
    o, o8 = oracle.Oracle(s), oracle.Oracle(s, u8=True)
    rng = np.random.default_rng(1)
    P = rng.uniform(-0.55, 0.55, (6000, 3)).astype(np.float32)
    a, b = o.sample(P), o8.sample(P)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(a)
    v = s.scalars
    span = 0.0
    for z in range(0, 36, 8):
        for y in range(0, 36, 8):
            for x in range(0, 36, 8):
                blk = v[z:z + 9, y:y + 9, x:x + 9]
                span = max(span, float(blk.max() - blk.min()))
    assert np.abs(a[m] - b[m]).max() <= span / 510 * (1 + 1e-5) + 1e-6
    # ranges bound the U8 samples of each macrocell
    r8 = o8.mc_ranges()
    origin, spacing = s.geometry()
    cell = np.floor((P[m] - np.asarray(origin, np.float32)) / np.asarray(spacing, np.float32)).astype(int)
    M = o8.mc_dims()
    mc = np.minimum(cell // s.cells_per_mc, np.asarray(M) - 1)
    idx = mc[:, 0] + M[0] * (mc[:, 1] + M[1] * mc[:, 2])
    assert np.all(b[m] >= r8[idx, 0]) and np.all(b[m] <= r8[idx, 1])
    # constant field: span 0, every sample is the value itself
    c = scenes.Scene(scalars=np.full((17, 17, 17), 0.375, np.float32), tf=scenes.tf_ramp(16), cells_per_mc=8)
    oc = oracle.Oracle(c, u8=True)
    sc = oc.sample(rng.uniform(-0.45, 0.45, (500, 3)).astype(np.float32))
    assert np.all(sc == np.float32(0.375))
    with pytest.raises(ValueError):
        o8.render(use_double=True)


def test_oracle_bounded_sincos_equals_library_host_routine():
    """The oracle's restatement of the bounded sine/cosine (part of its
    bounded_math mode) gives the library's host results bit for bit over
    the whole angle range the renderer forms."""
    from barney_gb300 import _native as N
    x = np.concatenate([np.linspace(-np.pi / 4, 2 * np.pi + np.pi / 4, 400_001, dtype=np.float32),
                        (np.random.default_rng(7).random(200_000) * 2 * np.pi).astype(np.float32)])
    so, co = oracle.bounded_sincos(x)
    sl, cl = np.empty_like(x), np.empty_like(x)
    assert N.lib().gbv_selftest_sincos(x.ctypes.data, x.size, sl.ctypes.data, cl.ctypes.data, 0, None) == N.GBV_OK
    np.testing.assert_array_equal(so.view(np.uint32), sl.view(np.uint32))
    np.testing.assert_array_equal(co.view(np.uint32), cl.view(np.uint32))


def test_oracle_bounded_angles_equal_library_host_routine():
    """The oracle's restatement of the library's arc cosine and arc tangent
    (bounded_math mode) gives its host results bit for bit, on directions
    of the sphere, the axes, signed zeros and the ends of [-1, 1]."""
    from barney_gb300 import _native as N
    rng = np.random.default_rng(11)
    v = rng.normal(size=(300_000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    y = np.concatenate([v[:, 1], [0.0, -0.0, 0.0, -0.0, 1.0, -1.0, 0.5, -0.5]]).astype(np.float32)
    x = np.concatenate([v[:, 2], [0.0, 0.0, -0.0, -0.0, 0.0, 0.0, 1.0, -1.0]]).astype(np.float32)
    ao, to = oracle.bounded_angles(y, x)
    al, tl = np.empty_like(x), np.empty_like(x)
    assert N.lib().gbv_selftest_angles(y.ctypes.data, x.ctypes.data, x.size, al.ctypes.data, tl.ctypes.data, 0,
                                       None) == N.GBV_OK
    np.testing.assert_array_equal(ao.view(np.uint32), al.view(np.uint32))
    np.testing.assert_array_equal(to.view(np.uint32), tl.view(np.uint32))


def test_bounded_math_mode_only_replaces_the_transcendentals():
    """Paths without a sine, cosine, arc cosine or arc tangent (single
    scattering, no env map) render identically in both oracle modes; with
    multiple scattering and the env map the modes differ only where a
    last-ulp difference reaches the pixel, so most pixels stay identical."""
    s = scenes.small_scene(dims=32, spp=2, width=48, height=32)
    a = oracle.Oracle(s).render()
    b = oracle.Oracle(s, bounded_math=True).render()
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    s = scenes.frame_scene(dims=32, width=48, height=32, spp=2)
    assert s.env is not None and s.multi_scatter == 1
    a = oracle.Oracle(s).render()
    b = oracle.Oracle(s, bounded_math=True).render()
    same = float(np.mean(np.all(a.view(np.uint32) == b.view(np.uint32), axis=-1)))
    assert same > 0.5, same
