"""Backward of the per-pixel L2 colour loss (visibility held fixed).

CPU: central finite differences (in double, on the FP64 loss of the oracle)
check the oracle's FP64 analytic gradient on 256 seeded parameters.  The
step is h = 1e-3 for texels and vertex colours, in which the loss is
quadratic (the difference quotient is exact), and h = 1e-7 for vertex
positions: a 1e-3 step moves samples across bilinear texel cells, where the
loss is only piecewise smooth (and leaves a truncation error near 1 % even
for vertex colours); at 1e-7 the FP64 loss still resolves the quotient to
about 1e-6 relative.  GPU: ugu_gpu_backward matches the FP64 analytic gradient within
1e-4 relative (vector 2-norm per gradient array) and the finite differences
on the same 256 parameters."""
import numpy as np
import pytest

import adversarial as adv
import diffrender as dr
from ugu_gb300 import capi, scenes

H_FD = {1: 1e-3, 2: 1e-3, 3: 1e-7}  # texel, vertex colour, vertex position


def _views(subdiv, n, size):
    m, t = dr.mesh_and_target_mesh(subdiv, 256)
    cams = scenes.ring_cameras(n, 3.0, [size] * n)
    return m, t, cams


def _fp64_grads(oracle_lib, m, cams, opt, fids, targets):
    gt = np.zeros(m.textures_f32[0].size, np.float64)
    gc = np.zeros(3 * m.num_vertices, np.float64)
    gp = np.zeros(3 * m.num_vertices, np.float64)
    loss = 0.0
    for cam, fid, tg in zip(cams, fids, targets):
        loss += oracle_lib.backward_f64(m, cam, opt, fid, tg, gt, gc, gp)
    return loss, gt, gc, gp


def _fd(oracle_lib, m, cams, opt, fids, targets, kind, index):
    def L(delta):
        return sum(oracle_lib.backward_f64(m, c, opt, f, t, perturb=(kind, index, delta))
                   for c, f, t in zip(cams, fids, targets))
    h = H_FD[kind]
    return (L(h) - L(-h)) / (2 * h)


def _forward_oracle(oracle_lib, m, cam, opt):
    rc, out, _ = oracle_lib.render(m, cam, opt, outputs=("face_id",), color_f32=True)
    assert rc == 0
    return out["face_id"], out["color_f32"]


@pytest.mark.parametrize("mode", ["texture", "vertex"])
def test_fd_matches_fp64_analytic(oracle_lib, mode):
    opt = adv.option(1 if mode == "texture" else 2, 1, 1, 0, True)
    m, t, cams = _views(4, 2, (160, 120))
    fids = [_forward_oracle(oracle_lib, m, c, opt)[0] for c in cams]
    targets = [_forward_oracle(oracle_lib, t, c, opt)[1] for c in cams]
    loss, gt, gc, gp = _fp64_grads(oracle_lib, m, cams, opt, fids, targets)
    grads = {1: gt, 2: gc, 3: gp}
    checked = 0
    for kind, idx in dr.seeded_params(m):
        if (mode == "texture" and kind == 2) or (mode == "vertex" and kind == 1):
            continue
        an = grads[kind][idx]
        fd = _fd(oracle_lib, m, cams, opt, fids, targets, kind, idx)
        scale = max(abs(an), 1e-3 * np.abs(grads[kind]).max())
        assert abs(fd - an) <= 1e-4 * scale + 1e-9, (kind, idx, fd, an)
        checked += 1
    assert checked >= 150


def _gpu_case(oracle_lib, torch, ctx, m, t, cams, opt):
    from gpu_helpers import device_views, to_option
    ctx.check(ctx.set_mesh(0, m))
    ctx.check(ctx.set_option(to_option(opt)))
    fw, views = device_views(torch, cams, [0] * len(cams), outputs=("face_id", "color_f32"))
    ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS))
    ctx.check(ctx.set_mesh(1, t))
    tw, tviews = device_views(torch, cams, [1] * len(cams), outputs=("color_f32",))
    ctx.check(ctx.render_views(tviews, capi.DEVICE_POINTERS))
    torch.cuda.synchronize()
    gt = torch.zeros(m.textures_f32[0].size, dtype=torch.float32, device="cuda")
    gc = torch.zeros(3 * m.num_vertices, dtype=torch.float32, device="cuda")
    gp = torch.zeros(3 * m.num_vertices, dtype=torch.float32, device="cuda")
    loss = torch.zeros(len(cams), dtype=torch.float32, device="cuda")
    rc = ctx.backward(views, [x["color_f32"].data_ptr() for x in tw], gt.data_ptr(),
                      gc.data_ptr(), gp.data_ptr(), loss.data_ptr())
    assert rc == 0, ctx.last_error()
    torch.cuda.synchronize()
    fids = [x["face_id"].cpu().numpy() for x in fw]
    targets = [x["color_f32"].cpu().numpy() for x in tw]
    # the forward's float colour equals the oracle's bit for bit
    for cam, f, x in zip(cams, fids, fw):
        rf, rc_ = _forward_oracle(oracle_lib, m, cam, opt)
        assert np.array_equal(rf, f)
        assert np.array_equal(rc_.view(np.uint32), x["color_f32"].cpu().numpy().view(np.uint32))
    return fids, targets, gt.cpu().numpy(), gc.cpu().numpy(), gp.cpu().numpy(), loss.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["texture", "vertex"])
def test_gpu_gradients_match_fp64_and_fd(oracle_lib, gpu_lib, mode):
    torch = pytest.importorskip("torch")
    from ugu_gb300.rasterizer import Context
    opt = adv.option(1 if mode == "texture" else 2, 1, 1, 0, True)
    m, t, cams = _views(5, 4, (320, 240))
    ctx = Context(0)
    try:
        fids, targets, gt, gc, gp, loss = _gpu_case(oracle_lib, torch, ctx, m, t, cams, opt)
    finally:
        ctx.close()
    l64, et, ec, ep = _fp64_grads(oracle_lib, m, cams, opt, fids, targets)
    assert abs(loss.sum() - l64) <= 1e-4 * l64
    if mode == "texture":
        assert _rel(gt, et) <= 1e-4
        assert not gc.any()
    else:
        assert _rel(gc, ec) <= 1e-4
        assert not gt.any()
    assert _rel(gp, ep) <= 1e-4, _rel(gp, ep)
    grads = {1: gt, 2: gc, 3: gp}
    for kind, idx in dr.seeded_params(m)[:96]:
        if (mode == "texture" and kind == 2) or (mode == "vertex" and kind == 1):
            continue
        fd = _fd(oracle_lib, m, cams, opt, fids, targets, kind, idx)
        scale = max(abs(fd), 1e-3 * np.abs(grads[kind]).max())
        assert abs(grads[kind][idx] - fd) <= 1e-4 * scale + 1e-6, (kind, idx, grads[kind][idx], fd)


@pytest.mark.gpu
def test_gpu_gradients_full_size_16_views(oracle_lib, gpu_lib):
    """Icosphere-7 with a 2048^2 float texture, 16 ring views at 640x480."""
    torch = pytest.importorskip("torch")
    from ugu_gb300.rasterizer import Context
    opt = adv.option(1, 1, 1, 0, True)
    m, t = dr.mesh_and_target_mesh(7, 2048)
    cams = scenes.ring_cameras(16, 3.0, [(640, 480)] * 16)
    ctx = Context(0)
    try:
        fids, targets, gt, gc, gp, loss = _gpu_case(oracle_lib, torch, ctx, m, t, cams, opt)
    finally:
        ctx.close()
    l64, et, ec, ep = _fp64_grads(oracle_lib, m, cams, opt, fids, targets)
    assert abs(loss.sum() - l64) <= 1e-4 * l64
    assert _rel(gt, et) <= 1e-4
    assert _rel(gp, ep) <= 1e-4, _rel(gp, ep)
