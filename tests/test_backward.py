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
    rec = {"views": "16 ring views at 640x480, icosphere-7, 2048^2 float texture",
           "norm_rel_texel": _rel(gt, et), "norm_rel_position": _rel(gp, ep)}
    rec.update(_element_record("texel", gt, et))
    rec.update(_element_record("position", gp, ep))
    _report("backward_16views", rec)


def _report(name, record):
    """Writes a test's measured figures as JSON when UGU_TEST_REPORT_DIR is set."""
    import json
    import os
    d = os.environ.get("UGU_TEST_REPORT_DIR")
    if d:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, f"{name}.json"), "w") as f:
            json.dump(record, f, indent=1, default=float)


def _worst_element(g, e, floor_frac=1e-3):
    """The largest elementwise relative error |g - e| / max(|e|, floor), the
    floor being floor_frac times the largest |e| of the array (elements
    smaller than that are measured against it)."""
    floor = floor_frac * float(np.abs(e).max())
    return float((np.abs(g - e) / np.maximum(np.abs(e), floor)).max()), floor


# Element bars.  The GPU sums each gradient element in float, by atomics in
# no fixed order, while the FP64 gradient sums exactly; an element whose
# many contributions of either sign cancel keeps the absolute rounding of
# its large partial sums.  Measured on the configurations below: texels
# 1.9e-4 at a floor of 1e-3 of the largest element (3e-7 norm-wise),
# positions and vertex colours about 2e-5.
ELEMENT_BARS = ((1e-3, 5e-4), (1e-2, 1e-4))  # (floor fraction, bar)


def _element_record(name, g, e):
    rec = {}
    for frac, bar in ELEMENT_BARS:
        worst, floor = _worst_element(g, e, frac)
        rec[f"worst_element_rel_{name}_floor{frac:g}"] = worst
        rec[f"floor_{name}_{frac:g}"] = floor
        assert worst <= bar, (name, frac, worst)
    return rec


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["texture", "vertex"])
def test_gpu_gradients_c4_central_differences(oracle_lib, gpu_lib, mode):
    """The differentiable configuration's mesh and texture (icosphere-7, 2048^2
    float texels, 640x480 ring views; 4 of the 16 views keep the run time
    short): GPU gradients against the FP64 analytic gradient element by
    element (each array's worst relative error, elements below 1e-3 of its
    largest measured against that floor, at most 1e-4), and against central
    finite differences of the FP64 loss on 256 seeded parameters with a
    nonzero gradient: 170 of the colour parameters (texels or vertex
    colours, h = 1e-3, where the loss is quadratic) and 86 vertex
    coordinates (h = 1e-7, see the module docstring).  A difference quotient
    carries the rounding of the loss it differences, at most
    8 * 2^-53 * L / h here; the bar is 1e-4 |fd| plus that."""
    import concurrent.futures as cf
    import os
    torch = pytest.importorskip("torch")
    from ugu_gb300.rasterizer import Context
    opt = adv.option(1 if mode == "texture" else 2, 1, 1, 0, True)
    m, t = dr.mesh_and_target_mesh(7, 2048)
    cams = scenes.ring_cameras(16, 3.0, [(640, 480)] * 16)[::4]
    ctx = Context(0)
    try:
        fids, targets, gt, gc, gp, loss = _gpu_case(oracle_lib, torch, ctx, m, t, cams, opt)
    finally:
        ctx.close()
    l64, et, ec, ep = _fp64_grads(oracle_lib, m, cams, opt, fids, targets)
    assert abs(loss.sum() - l64) <= 1e-4 * l64
    colour_kind, gcol, ecol = (1, gt, et) if mode == "texture" else (2, gc, ec)
    cname = "texel" if mode == "texture" else "vertex_colour"
    rec = {"views": "4 ring views at 640x480, icosphere-7, 2048^2 float texture",
           "loss_fp64": float(l64), "norm_rel_" + cname: _rel(gcol, ecol),
           "norm_rel_position": _rel(gp, ep)}
    rec.update(_element_record(cname, gcol, ecol))
    rec.update(_element_record("position", gp, ep))
    # seeded parameters among those the views constrain (nonzero gradient)
    rng = np.random.default_rng(7)
    pick_col = rng.choice(np.flatnonzero(ecol), 170, replace=False)
    pick_pos = rng.choice(np.flatnonzero(ep), 86, replace=False)
    params = [(colour_kind, int(i)) for i in pick_col] + [(3, int(i)) for i in pick_pos]
    grads = {colour_kind: gcol, 3: gp}

    def fd_one(kp):
        kind, idx = kp
        return _fd(oracle_lib, m, cams, opt, fids, targets, kind, idx)

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        fds = list(ex.map(fd_one, params))
    worst_fd = 0.0
    worst_rel = 0.0
    for (kind, idx), fd in zip(params, fds):
        noise = 8.0 * 2.0 ** -53 * l64 / H_FD[kind]
        err = abs(float(grads[kind][idx]) - fd)
        worst_fd = max(worst_fd, err / (1e-4 * abs(fd) + noise))
        worst_rel = max(worst_rel, err / max(abs(fd), 1e-30))
        assert err <= 1e-4 * abs(fd) + noise, (kind, idx, grads[kind][idx], fd, noise)
    rec.update({"fd_params": len(params), "fd_h": {"colour": H_FD[colour_kind],
                                                   "position": H_FD[3]},
                "fd_worst_error_over_bar": worst_fd, "fd_worst_rel": worst_rel})
    _report(f"backward_c4_{mode}", rec)
