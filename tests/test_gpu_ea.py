"""Fixed-step emission-absorption march and its adjoint on the GPU.

Tolerances: forward images within 1e-5 relative (plus 1e-6 absolute for
near-zero channels) of the oracle; the FP32 adjoint within 1e-3 relative
(norm over the checked entries) of central finite differences of the FP64
GPU march (eps = 1e-3) and of the oracle's FP64 gradient.
"""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.ea import EAProblem
import oracle

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6


def small_problem(dims=48, nviews=6, size=48):
    gt = scenes.ea_scene(dims)
    views = scenes.fibonacci_views(nviews, 2.5, size)
    step = 0.5 / (dims - 1)
    return gt, views, step


def test_forward_matches_oracle(cuda):
    gt, views, step = small_problem()
    p = EAProblem(gt, views, step)
    img = p.render().cpu().numpy().reshape(-1, 4)
    o = oracle.Oracle(gt)
    ref32 = o.ea_render(views, step)
    ref64 = o.ea_render(views, step, use_double=True)
    np.testing.assert_allclose(img, ref32, rtol=RTOL, atol=ATOL)
    # FP32 against FP64: rounding of sample positions, trilinear weights and
    # steep TF segments; measured max ~3e-4 relative on 0.2% of channels
    np.testing.assert_allclose(img, ref64, rtol=1e-3, atol=1e-5)
    assert img[:, 3].max() > 0.5


def test_forward_f64_matches_oracle(cuda):
    gt, views, step = small_problem(nviews=3)
    p = EAProblem(gt, views, step)
    img = p.render_f64().cpu().numpy().reshape(-1, 4)
    ref64 = oracle.Oracle(gt).ea_render(views, step, use_double=True)
    np.testing.assert_allclose(img, ref64, rtol=1e-6, atol=1e-7)


def test_constant_density_beer_lambert(cuda):
    """Known answer: a constant field maps to constant (rgb, sigma); a pixel
    whose march takes n steps gives A = 1-exp(-n sigma dt), C = rgb*A."""
    vol = np.full((16, 16, 16), 0.5, np.float32)
    tf = np.tile(np.array([[0.2, 0.6, 0.9, 0.4]], np.float32), (4, 1))
    s = scenes.Scene(scalars=vol, tf=tf, base_density=3.0)
    views = [dict(pos=(0.0, 0.0, 2.5), dir=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0), fovy=20.0, width=8, height=8)]
    step = 0.01
    img = EAProblem(s, views, step).render().cpu().numpy().reshape(8, 8, 4)
    # central pixels: the ray runs along -z through the whole box (t0=2, t1=3)
    sigma = 0.4 * 3.0
    t0, t1 = 2.0, 3.0
    n = sum(1 for i in range(200) if t0 + (i + 0.5) * step < t1)
    a = 1 - np.exp(-n * sigma * step)
    c = img[3, 3]
    np.testing.assert_allclose(c[3], a, rtol=2e-5)
    np.testing.assert_allclose(c[:3], np.array([0.2, 0.6, 0.9]) * a, rtol=2e-5)


@pytest.mark.parametrize("tf_kind", ["ramp", "two_peaks"])
def test_adjoint_matches_oracle_and_finite_differences(cuda, tf_kind):
    """The two-peak TF has knots (slope changes) inside the data range, where a
    central difference averages two one-sided slopes; the finite-difference
    check therefore runs on the knot-free ramp TF, and both TFs are checked
    against the oracle's FP64 gradient."""
    import torch
    gt, views, step = small_problem(dims=40, nviews=4, size=40)
    if tf_kind == "ramp":
        gt.tf = scenes.tf_ramp(256, 0.9)
    p_gt = EAProblem(gt, views, step)
    target = p_gt.render()
    start = scenes.Scene(scalars=np.full_like(gt.scalars, 0.3) + 0.2 * gt.scalars, tf=gt.tf,
                         base_density=gt.base_density)
    p = EAProblem(start, views, step)
    img = p.render()
    gimg = 2.0 * (img - target)  # dL/dI of L = sum (I - target)^2
    gv, gt_tf = p.backward(img, gimg)
    gv, gt_tf = gv.cpu().numpy().astype(np.float64), gt_tf.cpu().numpy().astype(np.float64)
    # FP64 oracle gradient
    o = oracle.Oracle(start)
    ov, ot = o.ea_backward(views, step, gimg.cpu().numpy().reshape(-1, 4))
    ov = ov.reshape(-1)
    sel = np.flatnonzero(np.abs(ov) > 1e-3 * np.abs(ov).max())
    assert np.linalg.norm(gv.reshape(-1)[sel] - ov[sel]) <= 1e-3 * np.linalg.norm(ov[sel])
    assert np.linalg.norm(gt_tf - ot) <= 1e-3 * np.linalg.norm(ot)
    if tf_kind != "ramp":
        return
    # central finite differences of the FP64 march, eps = 1e-3
    rng = np.random.default_rng(44)
    tgt64 = target.double()

    def loss(pp):
        return float(((pp.render_f64() - tgt64) ** 2).sum().item())

    def fd_of(make, base, eps=1e-3):
        hi, lo = np.float32(base + eps), np.float32(base - eps)
        return (loss(make(float(hi))) - loss(make(float(lo)))) / (float(hi) - float(lo))

    vox = rng.choice(sel, size=16, replace=False)
    base = start.scalars.reshape(-1)
    fd = np.array([fd_of(lambda x, v=v: p.with_voxel(int(v), x), float(base[v])) for v in vox])
    an = gv.reshape(-1)[vox]
    assert np.linalg.norm(fd - an) <= 1e-3 * np.linalg.norm(fd) + 1e-6, (fd, an)
    tsel = np.flatnonzero(np.abs(ot.reshape(-1)) > 1e-3 * np.abs(ot).max())
    ent = rng.choice(tsel, size=min(16, tsel.size), replace=False)
    tfb = start.tf.reshape(-1)
    fd = np.array([fd_of(lambda x, e=e: p.with_tf_entry(int(e), x), float(tfb[e])) for e in ent])
    an = gt_tf.reshape(-1)[ent]
    assert np.linalg.norm(fd - an) <= 1e-3 * np.linalg.norm(fd) + 1e-6, (fd, an)


def test_autograd_function(cuda):
    import torch
    from barney_gb300.ea import ea_render_autograd
    gt, views, step = small_problem(dims=32, nviews=2, size=32)
    p = EAProblem(gt, views, step)
    vox = p.scalars.clone().requires_grad_(True)
    tf = p.tf.clone().requires_grad_(True)
    img = ea_render_autograd(vox, tf, p)
    w = torch.rand_like(img)
    (img * w).sum().backward()
    gv, gtf = p.backward(img.detach(), w)
    # the adjoint's atomics sum in no fixed order: equal up to FP32 reassociation
    torch.testing.assert_close(vox.grad.reshape(-1), gv.reshape(-1), rtol=1e-4, atol=1e-6)
    torch.testing.assert_close(tf.grad.reshape(-1), gtf.reshape(-1), rtol=1e-4, atol=1e-5)


def _rounded(v, fmt):
    if fmt == N.GBV_VOXEL_F16:
        return v.astype(np.float16).astype(np.float32)
    u = v.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("fmt,brick", [(N.GBV_VOXEL_F32, (3, 3, 3)), (N.GBV_VOXEL_F32, (4, 2, 2)),
                                       (N.GBV_VOXEL_F16, (3, 3, 3)), (N.GBV_VOXEL_BF16, (2, 2, 2))])
def test_forward_on_brick_stores(cuda, fmt, brick):
    """The forward march over a brick-corner store equals the march over the
    linear FP32 field holding the same (rounded) voxel values, bit for bit."""
    from barney_gb300.device import GpuScene
    gt, views, step = small_problem(nviews=3)
    g = GpuScene(gt, fmt=fmt, brick=brick)
    got = EAProblem(gt, views, step, store=g).render().cpu().numpy()
    rounded = gt.scalars if fmt == N.GBV_VOXEL_F32 else _rounded(gt.scalars, fmt)
    import copy
    gr = copy.copy(gt)
    gr.scalars = np.ascontiguousarray(rounded)
    ref = EAProblem(gr, views, step).render().cpu().numpy()
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_forward_on_u8_store_error_against_fp64(cuda):
    from barney_gb300.device import GpuScene
    gt, views, step = small_problem(nviews=3)
    g = GpuScene(gt, fmt=N.GBV_VOXEL_U8_SCALED)
    got = EAProblem(gt, views, step, store=g).render().cpu().numpy().reshape(-1, 4)
    ref64 = oracle.Oracle(gt).ea_render(views, step, use_double=True)
    err = np.abs(got - ref64)
    # 8-bit voxels per 8^3 cells: a few 1e-3 on the image
    assert float(np.sqrt(np.mean(err ** 2))) < 5e-3 and err.max() < 0.05, (np.sqrt(np.mean(err ** 2)), err.max())


def test_forward_on_u8_store_matches_oracle_u8_form(cuda):
    """Against the oracle's U8 storage form the U8 forward agrees as closely
    as the FP32 forward does with the FP32 oracle."""
    from barney_gb300.device import GpuScene
    gt, views, step = small_problem(nviews=3)
    g = GpuScene(gt, fmt=N.GBV_VOXEL_U8_SCALED)
    got = EAProblem(gt, views, step, store=g).render().cpu().numpy().reshape(-1, 4)
    ref = oracle.Oracle(gt, u8=True).ea_render(views, step)
    np.testing.assert_allclose(got, ref, rtol=RTOL, atol=ATOL)


def test_adjoint_rejects_brick_stores(cuda):
    import ctypes as C
    from barney_gb300.device import GpuScene, _ptr, _stream
    gt, views, step = small_problem(nviews=1)
    g = GpuScene(gt, fmt=N.GBV_VOXEL_F16)
    p = EAProblem(gt, views, step, store=g)
    rec = p.record()
    rec.d_voxels = g.voxels.data_ptr()
    rec.format, rec.layout = g.fmt, g.layout
    import torch
    img = p.render()
    gv = torch.zeros(p.scalars.numel(), device="cuda")
    gtf = torch.zeros(p.tf.numel(), device="cuda")
    st = N.lib().gbv_ea_backward(C.byref(rec), p._views_c, 1, step, _ptr(img), _ptr(img), _ptr(gv), _ptr(gtf),
                                 _stream())
    assert st == N.GBV_ERROR_UNSUPPORTED


def test_reconstruction_loop_reduces_the_loss(cuda):
    """The differentiable workload in miniature: a density grid that starts
    at a constant 0.1 and the transfer function are fitted to target views
    of a blob volume by Adam steps through the autograd wrapper (at 0.1 the
    two-peak TF is flat zero, so the first gradients reach the TF entries);
    the L2 loss falls well below its start."""
    import torch
    from barney_gb300.ea import ea_render_autograd
    gt = scenes.ea_scene(24)
    views = scenes.fibonacci_views(8, 2.5, 24)
    step = 0.5 / 23
    target = EAProblem(gt, views, step).render()
    start = scenes.Scene(scalars=np.full_like(gt.scalars, 0.1), tf=gt.tf, base_density=gt.base_density)
    p = EAProblem(start, views, step)
    vox = p.scalars.clone().requires_grad_(True)
    tf = p.tf.clone().requires_grad_(True)
    opt = torch.optim.Adam([vox, tf], lr=0.02)
    losses = []
    for _ in range(40):
        opt.zero_grad()
        img = ea_render_autograd(vox, tf, p)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        opt.step()
        with torch.no_grad():
            vox.clamp_(0.0, 1.0)
            tf.clamp_(0.0, 1.0)
        losses.append(float(loss.item()))
    assert losses[-1] < 0.3 * losses[0], losses[::8]


def test_differentiable_workload_at_its_named_size(cuda):
    """The differentiable emission-absorption workload at its own size: a
    128^3 FP32 density grid, the 256-entry two-peak TF, 32 views of 256^2 on
    a Fibonacci sphere of radius 2.5, step 0.5 voxel, L2 loss against target
    views of the seeded ground-truth blob volume.
    - forward: within 1e-5 relative (+1e-6 absolute) of the FP32 oracle;
    - adjoint: within 1e-3 relative (norm over entries above 1e-3 of the
      largest) of the oracle's FP64 gradient, voxels and TF entries;
    - central finite differences (eps = 1e-3) of the FP64 GPU march at 64
      random voxels and 64 random TF entries (seed 44): within 1e-3
      relative.  The FD check runs on the knot-free ramp TF (a central
      difference across a TF knot averages two one-sided slopes; see
      test_adjoint_matches_oracle_and_finite_differences), with the same
      grid, views, step and loss."""
    import torch
    dims = 128
    gt = scenes.ea_scene(dims)
    views = scenes.fibonacci_views(32, 2.5, 256)
    assert len(views) == 32 and all(v["width"] == v["height"] == 256 for v in views)
    step = 0.5 / (dims - 1)
    for tf_kind in ("two_peaks", "ramp"):
        truth = gt if tf_kind == "two_peaks" else scenes.Scene(scalars=gt.scalars, tf=scenes.tf_ramp(256, 0.9),
                                                                base_density=gt.base_density,
                                                                cells_per_mc=gt.cells_per_mc)
        target = EAProblem(truth, views, step).render()
        # parameters away from the truth, where every gradient term is live
        start = scenes.Scene(scalars=np.full_like(truth.scalars, 0.3) + 0.2 * truth.scalars, tf=truth.tf,
                             base_density=truth.base_density, cells_per_mc=truth.cells_per_mc)
        p = EAProblem(start, views, step)
        img = p.render()
        o = oracle.Oracle(start)
        if tf_kind == "two_peaks":
            np.testing.assert_allclose(img.cpu().numpy(), o.ea_render(views, step), rtol=RTOL, atol=ATOL)
        gimg = 2.0 * (img - target)
        gv, gtf = p.backward(img, gimg)
        torch.cuda.synchronize()
        gv = gv.cpu().numpy().astype(np.float64)
        gtf = gtf.cpu().numpy().astype(np.float64).reshape(-1)
        ov, ot = o.ea_backward(views, step, gimg.cpu().numpy().reshape(-1, 4))
        ov, ot = ov.reshape(-1), ot.reshape(-1)
        sel = np.flatnonzero(np.abs(ov) > 1e-3 * np.abs(ov).max())
        tsel = np.flatnonzero(np.abs(ot) > 1e-3 * np.abs(ot).max())
        assert sel.size > 10000 and tsel.size >= 64, (sel.size, tsel.size)
        assert np.linalg.norm(gv[sel] - ov[sel]) <= 1e-3 * np.linalg.norm(ov[sel])
        assert np.linalg.norm(gtf[tsel] - ot[tsel]) <= 1e-3 * np.linalg.norm(ot[tsel])
        if tf_kind != "ramp":
            continue
        rng = np.random.default_rng(44)
        tgt64 = target.double()

        def loss(pp):
            return float(((pp.render_f64() - tgt64) ** 2).sum().item())

        def fd_of(make, base, eps=1e-3):
            hi, lo = np.float32(base + eps), np.float32(base - eps)
            return (loss(make(float(hi))) - loss(make(float(lo)))) / (float(hi) - float(lo))

        vox = rng.choice(sel, size=64, replace=False)
        base = start.scalars.reshape(-1)
        fd = np.array([fd_of(lambda x, v=v: p.with_voxel(int(v), x), float(base[v])) for v in vox])
        an = gv[vox]
        assert np.linalg.norm(fd - an) <= 1e-3 * np.linalg.norm(fd), (fd, an)
        ent = rng.choice(tsel, size=64, replace=False)
        tfb = start.tf.reshape(-1)
        fd = np.array([fd_of(lambda x, e=e: p.with_tf_entry(int(e), x), float(tfb[e])) for e in ent])
        an = gtf[ent]
        assert np.linalg.norm(fd - an) <= 1e-3 * np.linalg.norm(fd), (fd, an)
