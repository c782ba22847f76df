"""TextureMapping (src/texturing/texture_mapper.cc: TextureMappingSimple
:924-1006, RasterizeTriangle :234-292, PaddingSimple :148-201) against the
oracle's restatement (oracle/vis_oracle.cc), texture, mask and uv bit for
bit, for the four uv types: the mesh's own uv (kUseOriginalMeshUv, through
ugu_gpu_texture_mapping), the tiled keyframe images (kGenerateSimpleTile,
the reference's default, :62-141, through ugu_gpu_tile_images), one
rectangle half per face (kGenerateSimpleTriangles, :347-440, through
ugu_gpu_texture_mapping_targets) and bin-packed charts of keyframe patches
(kGenerateSimpleCharts, :476-922, host layout and copies, as in the
reference).  The face arrays are seeded: uv triangles that
overlap heavily (a later face overwrites an earlier one), source triangles
reaching outside their keyframe images, faces without a keyframe.  Where
the reference checkout is present, the restatements are also pinned to the
reference's own texture_mapper.cc and bin_packer_2d.cc (oracle/_ref)."""
import numpy as np
import pytest

from ugu_gb300 import capi, scenes
from ugu_gb300 import visibility as vis


def overlapping_faces(n_faces=600, n_kf=3, seed=5):
    rng = np.random.default_rng(seed)
    # uv triangles of 2 to 40 texels packed into the middle of the texture
    c = rng.uniform(0.3, 0.7, (n_faces, 1, 2))
    uv = (c + rng.normal(0.0, 1.0, (n_faces, 3, 2)) * rng.uniform(0.002, 0.03, (n_faces, 1, 1)))
    uv = uv.reshape(-1, 2).astype(np.float32)
    uvi = np.arange(3 * n_faces, dtype=np.int32).reshape(-1, 3)
    sizes = [(80, 60), (64, 64), (97, 41)][:n_kf]
    imgs = [rng.integers(0, 256, (h, w, 3)).astype(np.uint8) for w, h in sizes]
    face_kf = rng.integers(-1, n_kf, n_faces).astype(np.int32)
    face_tri = np.zeros((n_faces, 3, 2), np.float32)
    for f in range(n_faces):
        w, h = sizes[max(face_kf[f], 0)]
        face_tri[f] = rng.uniform([-4, -4], [w + 4, h + 4], (3, 2))
    return uv, uvi, imgs, face_kf, face_tri


def test_oracle_single_face_copies_and_pads(oracle_lib):
    img = np.arange(8 * 8 * 3, dtype=np.uint8).reshape(8, 8, 3)
    uv = np.array([[0.0, 1.0], [1.0, 1.0], [0.0, 0.0]], np.float32)
    tri = np.array([[[-0.5, -0.5], [7.5, -0.5], [-0.5, 7.5]]], np.float32)
    rc, tex, mask = oracle_lib.texture_mapping(uv, [[0, 1, 2]], [img], [0], tri, 8, 8, 3)
    assert rc == 0
    # the uv triangle maps texel (x, y) to source point (x, y): texels copied
    assert np.array_equal(tex[0, 0], img[0, 0]) and np.array_equal(tex[2, 3], img[2, 3])
    rc, tex0, mask0 = oracle_lib.texture_mapping(uv, [[0, 1, 2]], [img], [0], tri, 8, 8, 0)
    # padded texels: inside the border, empty before, the truncated mean of
    # the 3 x 3 window's valid texels after; the border is never padded
    padded = np.argwhere((mask == 255) & (mask0 == 0))
    assert len(padded) > 0 and mask[1, 7] == 0 and mask0[1, 7] == 0
    y, x = padded[0]
    win = mask0[y - 1:y + 2, x - 1:x + 2] == 255
    mean = tex0[y - 1:y + 2, x - 1:x + 2][win].astype(np.float32).sum(0) / np.float32(win.sum())
    assert np.array_equal(tex[y, x], mean.astype(np.uint8))
    assert oracle_lib.texture_mapping(uv, [[0, 1, 2]], [img], [1], tri, 8, 8, 3)[0] == -1


def _face_info(rows):
    fi = vis.FaceInfo(visible_keyframes=[
        vis.FaceInfoPerKeyframe(k, 0, a, va, d, np.full((3, 2), k, np.float32))
        for k, a, va, d in rows])
    fi.CalcStat()
    return fi


def test_best_keyframes_by_criteria():
    info = vis.VisibilityInfo(0, 0)
    info.face_info_list = [_face_info([(0, 4.0, 0.5, 2.0), (1, 9.0, 0.2, 3.0), (2, 1.0, 0.9, 1.0)]),
                           vis.FaceInfo()]
    for crit, want in ((vis.ViewSelectionCriteria.kMaxArea, 1),
                       (vis.ViewSelectionCriteria.kMinViewingAngle, 1),
                       (vis.ViewSelectionCriteria.kMinDistance, 2)):
        fk, ft = vis.best_keyframes(info, crit)
        assert list(fk) == [want, -1] and ft[0, 0, 0] == want
    with pytest.raises(ValueError):
        vis.best_keyframes(info, 3)


def test_texture_mapping_rejected_layouts_return_false():
    m = scenes.icosphere_textured(1, 8)
    info = vis.VisibilityInfo(m.num_vertices, m.num_faces)
    tile = vis.TextureMappingOption()  # kGenerateSimpleTile, the reference's default
    assert vis.TextureMapping([], info, m, tile) is False  # no keyframe to tile
    other = vis.TextureMappingOption(type=1)  # a mapping type the reference does not implement
    assert vis.TextureMapping([], info, m, other) is False


def test_bin_packing_2d_known_answer():
    """BinPacking2D's guillotine cuts worked by hand: a 3x3 then a 2x2
    rectangle into the 8x8 free rectangle at (1, 1); the 3x3 leaves a
    5-wide strip (cut across the wider leftover: a 3-wide column first, then
    its 3-high top), and the 2x2 takes the 3x5 piece under it."""
    packed, free = vis.bin_packing_2d([(3, 3), (2, 2)], 1, 8, 1, 8)
    assert packed == [(1, 1, 3, 3), (1, 4, 2, 2)]
    assert free == [(4, 1, 5, 8), (1, 6, 3, 3), (3, 4, 1, 2)]
    assert vis.bin_packing_2d([(9, 2)], 1, 8, 1, 8) is None  # wider than the space


@pytest.mark.parametrize("seed", range(6))
def test_bin_packing_2d_pinned_to_the_reference(seed):
    """The mirror's BinPacking2D against the reference's own
    (src/discrete/bin_packer_2d.cc, built into oracle/_ref): the same packed
    and free rectangles, in the same order, or both failing.  Seeded
    rectangle lists, sorted by area as the chart atlas sorts them or not,
    into spaces from roomy to too small; runs where the reference checkout
    is present."""
    ref_build = pytest.importorskip("oracle.ref_build")
    if not ref_build.available():
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(100 + seed)
    cases = [([(3, 3), (2, 2)], (1, 8, 1, 8)), ([(9, 2)], (1, 8, 1, 8))]
    for space in (64, 128, 256):
        n = int(rng.integers(5, 60))
        rects = [(int(w), int(h)) for w, h in rng.integers(1, 40, (n, 2))]
        if seed % 2 == 0:
            rects.sort(key=lambda r: -r[0] * r[1])
        cases.append((rects, (1, space - 1, 1, space - 1)))
    for rects, (x0, x1, y0, y1) in cases:
        ok, r_packed, r_free = ref_build.bin_packing_2d([(0, 0, w, h) for w, h in rects],
                                                        x0, x1, y0, y1)
        mine = vis.bin_packing_2d(rects, x0, x1, y0, y1)
        if not ok:
            assert mine is None, (rects, x0, x1)
            continue
        assert mine is not None, (rects, x0, x1)
        assert mine[0] == r_packed
        assert mine[1] == r_free


class _Kf:
    def __init__(self, i, color):
        self.id, self.color = i, color


def _chart_case(subdiv, n_kf, size, seed, unseen=0.2):
    """Faces of an icosphere given seeded best keyframes by region (some
    unseen) and orthographic projected triangles inside size-sized images."""
    m = scenes.icosphere_textured(subdiv, 8)
    rng = np.random.default_rng(seed)
    cen = m.vertices[m.vertex_indices].mean(1)
    ang = np.arctan2(cen[:, 1], cen[:, 0])
    face_kf = (((ang + np.pi) / (2 * np.pi)) * n_kf).astype(np.int32) % n_kf
    face_kf[np.abs(cen[:, 2]) > 1.0 - unseen] = -1
    w, h = size
    tri = m.vertices[m.vertex_indices][:, :, :2]
    face_tri = np.stack([(w - 1) * 0.5 * (1 + 0.98 * tri[..., 0]),
                         (h - 1) * 0.5 * (1 + 0.98 * tri[..., 1])], -1).astype(np.float32)
    imgs = [rng.integers(0, 256, (h, w, 3), dtype=np.uint8) for _ in range(n_kf)]
    return m, face_kf, face_tri, imgs


@pytest.mark.parametrize("subdiv,n_kf,size,tex,seed", [
    (2, 3, (64, 48), 128, 1), (3, 4, (160, 120), 256, 2), (3, 2, (96, 96), 16, 3),
    (4, 6, (200, 150), 512, 4), (1, 1, (32, 32), 64, 5)])
def test_simple_charts_layout_matches_oracle(oracle_lib, subdiv, n_kf, size, tex, seed):
    """kGenerateSimpleCharts in the mirror and the oracle agree bit for bit:
    the atlas texture (patches with their replicated border, packed largest
    first, the texture grown in sqrt(2) steps when tex x tex is too small),
    the uv of every chart vertex and every face's uv indices, unseen faces on
    the shared invalid uv."""
    m, face_kf, face_tri, imgs = _chart_case(subdiv, n_kf, size, seed)
    kfs = [_Kf(i, im) for i, im in enumerate(imgs)]
    lay = vis.simple_charts_layout(m.vertex_indices, face_kf, face_tri, kfs, tex, tex)
    rc, want_t, want_uv, want_uvi = oracle_lib.simple_charts(m.vertex_indices, imgs, face_kf,
                                                             face_tri, tex, tex)
    assert rc == 0 and lay is not None
    t, uv, uvi, mask = lay
    assert np.array_equal(t, want_t)
    assert np.array_equal(uv.view(np.uint32), want_uv.view(np.uint32))
    assert np.array_equal(uvi, want_uvi)
    # every visible face's uv triangle lies on its chart's patch, unseen
    # faces all on the last three (invalid) uv
    unseen = face_kf < 0
    if unseen.any():
        assert (uvi[unseen] == np.arange(len(uv) - 3, len(uv))).all()
    seen = uvi[~unseen]
    assert seen.max() < len(uv) - 3
    H, W = t.shape[:2]
    px = np.rint(uv[seen][..., 0] * W - 0.5).astype(int)
    py = np.rint((1.0 - uv[seen][..., 1]) * H - 0.5).astype(int)
    assert (mask[py, px] == 255).all()


def test_simple_charts_rejects_what_the_reference_overruns(oracle_lib):
    """A chart whose projected triangles reach outside its keyframe image
    would make the reference copy from outside the image: both refuse."""
    m, face_kf, face_tri, imgs = _chart_case(2, 2, (64, 48), 7)
    face_tri = face_tri.copy()
    face_tri[np.flatnonzero(face_kf >= 0)[0], 0, 0] = 70.0
    kfs = [_Kf(i, im) for i, im in enumerate(imgs)]
    assert vis.simple_charts_layout(m.vertex_indices, face_kf, face_tri, kfs, 128, 128) is None
    rc, *_ = oracle_lib.simple_charts(m.vertex_indices, imgs, face_kf, face_tri, 128, 128)
    assert rc == -2


@pytest.mark.parametrize("faces,size", [(5, (64, 64)), (1, (16, 16)), (2000, (512, 384)),
                                        (301, (97, 53)), (40000, (256, 256)), (9, (7, 7)),
                                        (0, (32, 32)), (3000, (1024, 16))])
def test_simple_triangles_layout_matches_oracle(oracle_lib, faces, size):
    """The layout arithmetic of the mirror (ugu_gb300/visibility.py) and of
    the oracle agree bit for bit, including where the reference returns
    false (fewer than 6 texels per rectangle, or sq_len under 3)."""
    rng = np.random.default_rng(faces)
    face_kf = rng.integers(-1, 3, faces).astype(np.int32)
    tw, th = size
    rc, target, uv = oracle_lib.simple_triangles_layout(face_kf, tw, th)
    lay = vis.simple_triangles_layout(face_kf, tw, th)
    assert (rc == -1) == (lay is None)
    if lay is None:
        return
    assert np.array_equal(lay[0], target)
    assert np.array_equal(lay[1].view(np.uint32), uv.view(np.uint32))
    # visible faces' triangles stay inside the texture and never share a texel
    cover = np.zeros((th, tw), np.int32)
    for f in np.flatnonzero(face_kf >= 0):
        t = target[f]
        assert t.min() >= 0 and t[:, 0].max() < tw and t[:, 1].max() < th
        (x0, y0), (x1, y1) = t.min(0).astype(int), t.max(0).astype(int)
        ys, xs = np.mgrid[y0:y1 + 1, x0:x1 + 1]
        upper = f % 2 == 0  # the even face: x - x0 >= y - y0 (upper right)
        inside = (xs - x0) >= (ys - y0) if upper else (xs - x0) <= (ys - y0)
        cover[ys[inside], xs[inside]] += 1
    assert cover.max() <= 1


def test_simple_tile_layout_matches_oracle(oracle_lib):
    """The tile layout's uv (each face's projected triangle moved to its
    keyframe's tile) in the mirror and the oracle, bit for bit; an unknown
    keyframe id maps to tile 0 and a duplicated id to its first position,
    as the reference's map does; 5 keyframes (not whole rows of
    int(sqrt(5)) = 2) or images of two sizes are rejected."""
    rng = np.random.default_rng(3)
    imgs = [rng.integers(0, 256, (30, 40, 3)).astype(np.uint8) for _ in range(6)]
    ids = [7, 3, 9, 3, 12, 1]
    F = 500
    face_kf = rng.choice(ids + [-1, 99], F).astype(np.int32)
    face_tri = rng.uniform(-5, 45, (F, 3, 2)).astype(np.float32)
    kfs = [vis.Keyframe(i, None, im) for i, im in zip(ids, imgs)]
    rc, tex, uv = oracle_lib.simple_tile(ids, imgs, face_kf, face_tri)
    assert rc == 0 and tex.shape == (90, 80, 3)  # 2 x 3 tiles
    assert np.array_equal(tex[30:60, 40:80], imgs[3])
    x_tiles, y_tiles, uv2 = vis.simple_tile_layout(kfs, face_kf, face_tri)
    assert (x_tiles, y_tiles) == (2, 3)
    assert np.array_equal(uv.view(np.uint32), uv2.view(np.uint32))
    assert vis.simple_tile_layout(kfs[:5], face_kf, face_tri) is None
    assert oracle_lib.simple_tile(ids[:5], imgs[:5], face_kf, face_tri)[0] == -1
    odd = [vis.Keyframe(0, None, imgs[0]), vis.Keyframe(1, None, imgs[1][:, :20])]
    assert vis.simple_tile_layout(odd, face_kf, face_tri) is None


@pytest.mark.gpu
@pytest.mark.parametrize("size,kernel", [((256, 192), 3), ((300, 130), 5), ((128, 128), 0)])
def test_gpu_texture_mapping_matches_oracle(gpu_lib, oracle_lib, size, kernel):
    from ugu_gb300.rasterizer import Context
    uv, uvi, imgs, face_kf, face_tri = overlapping_faces()
    tw, th = size
    rc, want_t, want_m = oracle_lib.texture_mapping(uv, uvi, imgs, face_kf, face_tri, tw, th, kernel)
    assert rc == 0
    n = len(uvi)
    m = scenes.Mesh(vertices=np.zeros((3 * n, 3), np.float32), vertex_indices=uvi.copy())
    m.uv, m.uv_indices = uv, uvi
    ctx = Context(0)
    try:
        ctx.check(ctx.set_mesh(0, m))
        descs = []
        for k, img in enumerate(imgs):
            d = capi.KeyframeDesc()
            d.id = k
            d.camera = capi.camera_struct(scenes.camera_desc(img.shape[1], img.shape[0], 50.0,
                                                             50.0, 20.0, 20.0))
            d.color = img.ctypes.data
            descs.append(d)
        tex = np.zeros((th, tw, 3), np.uint8)
        mask = np.zeros((th, tw), np.uint8)
        ctx.check(ctx.texture_mapping(0, descs, face_kf, face_tri.reshape(-1, 6),
                                      capi.TextureOption(tw, th, kernel), tex, mask))
        assert np.array_equal(mask, want_m)
        bad = np.argwhere((tex != want_t).any(-1))
        assert len(bad) == 0, (len(bad), bad[:5])
        assert (want_m == 255).mean() > 0.05
        # an id past the keyframe list is an error, as an index past it is in C++
        face_kf2 = face_kf.copy()
        face_kf2[7] = len(imgs)
        assert ctx.texture_mapping(0, descs, face_kf2, face_tri.reshape(-1, 6),
                                   capi.TextureOption(tw, th, kernel), tex, mask) != 0
    finally:
        ctx.close()


@pytest.mark.gpu
def test_gpu_texture_mapping_pipeline(gpu_lib, oracle_lib):
    """VisibilityTester, then TextureMapping on the mesh's own uv: the
    texture equals the oracle's for the same best keyframes."""
    from test_visibility import keyframes, option
    m = scenes.icosphere_textured(3, 64)
    kfs = [(i, cam, im) for i, (_, cam, im) in enumerate(keyframes(oracle_lib, m, n=4))]
    vt = vis.VisibilityTester(option())
    vt.set_data(m.vertices, m.normals, m.vertex_indices)
    assert vt.PrepareData()
    info = vis.VisibilityInfo(m.num_vertices, m.num_faces)
    frames = [vis.Keyframe(kid, cam, im["color"], im["depth"], im["mask"]) for kid, cam, im in kfs]
    assert vt.Test(info, facewise=False, keyframes=frames)
    opt = vis.TextureMappingOption(uv_type=vis.TexturingOutputUvType.kUseOriginalMeshUv,
                                   tex_w=256, tex_h=256)
    face_kf, face_tri = vis.best_keyframes(info, opt.criteria)
    assert (face_kf >= 0).mean() > 0.3
    rc, want_t, want_m = oracle_lib.texture_mapping(m.uv, m.uv_indices, [f.color for f in frames],
                                                    face_kf, face_tri, 256, 256, 3)
    assert rc == 0
    assert vis.TextureMapping(frames, info, m, opt, ctx=vt._ctx, slot=1)
    assert np.array_equal(m.texture_mask, want_m)
    assert np.array_equal(m.textures[0], want_t)
    assert list(np.unique(m.material_ids)) == [0]


def _descs(imgs):
    descs = []
    for k, img in enumerate(imgs):
        d = capi.KeyframeDesc()
        d.id = k
        d.camera = capi.camera_struct(scenes.camera_desc(img.shape[1], img.shape[0], 50.0, 50.0,
                                                         20.0, 20.0))
        d.color = img.ctypes.data
        descs.append(d)
    return descs


@pytest.mark.gpu
@pytest.mark.parametrize("size", [(256, 192), (512, 512)])
def test_gpu_simple_triangles_matches_oracle(gpu_lib, oracle_lib, size):
    """Every visible face drawn into its half-rectangle on the GPU: texture
    and mask equal the oracle's (seeded faces whose projected triangles reach
    outside their keyframe images, faces without a keyframe)."""
    from ugu_gb300.rasterizer import Context
    _, _, imgs, face_kf, face_tri = overlapping_faces()
    tw, th = size
    rc, want_t, want_m, want_uv = oracle_lib.simple_triangles(imgs, face_kf, face_tri, tw, th)
    assert rc == 0
    target, uv = vis.simple_triangles_layout(face_kf, tw, th)
    assert np.array_equal(uv.view(np.uint32), want_uv.view(np.uint32))
    ctx = Context(0)
    try:
        tex = np.zeros((th, tw, 3), np.uint8)
        mask = np.zeros((th, tw), np.uint8)
        ctx.check(ctx.texture_mapping_targets(target.reshape(-1, 6), _descs(imgs), face_kf,
                                              face_tri.reshape(-1, 6),
                                              capi.TextureOption(tw, th, 3), tex, mask))
        assert np.array_equal(mask, want_m)
        assert np.array_equal(tex, want_t)
        assert (want_m == 255).mean() > 0.2
    finally:
        ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("uv_type", [vis.TexturingOutputUvType.kGenerateSimpleTile,
                                     vis.TexturingOutputUvType.kGenerateSimpleTriangles,
                                     vis.TexturingOutputUvType.kGenerateSimpleCharts])
def test_gpu_texture_mapping_atlas_pipeline(gpu_lib, oracle_lib, uv_type):
    """VisibilityTester, then TextureMapping with a generated atlas through
    the mirror: texture and uv equal the oracle's; the re-textured mesh then
    renders on the GPU bit for bit as the oracle renders it."""
    from gpu_helpers import compare, gpu_render
    from test_visibility import keyframes, option
    from ugu_gb300.rasterizer import Context, RendererCpuOption
    m = scenes.icosphere_textured(3, 64)
    base = 10 if uv_type == vis.TexturingOutputUvType.kGenerateSimpleTile else 0
    kfs = [(base + i, cam, im) for i, (_, cam, im) in enumerate(keyframes(oracle_lib, m, n=4))]
    vt = vis.VisibilityTester(option())
    vt.set_data(m.vertices, m.normals, m.vertex_indices)
    assert vt.PrepareData()
    info = vis.VisibilityInfo(m.num_vertices, m.num_faces)
    frames = [vis.Keyframe(kid, cam, im["color"], im["depth"], im["mask"]) for kid, cam, im in kfs]
    assert vt.Test(info, facewise=False, keyframes=frames)
    opt = vis.TextureMappingOption(uv_type=uv_type, tex_w=512, tex_h=512)
    face_kf, face_tri = vis.best_keyframes(info, opt.criteria)
    assert (face_kf >= 0).mean() > 0.3
    want_uvi = None
    if uv_type == vis.TexturingOutputUvType.kGenerateSimpleTile:
        rc, want_t, want_uv = oracle_lib.simple_tile([f.id for f in frames],
                                                     [f.color for f in frames], face_kf, face_tri)
        want_m = None
    elif uv_type == vis.TexturingOutputUvType.kGenerateSimpleCharts:
        rc, want_t, want_uv, want_uvi = oracle_lib.simple_charts(
            m.vertex_indices, [f.color for f in frames], face_kf, face_tri, 512, 512)
        want_m = None
    else:
        rc, want_t, want_m, want_uv = oracle_lib.simple_triangles(
            [f.color for f in frames], face_kf, face_tri, 512, 512)
    assert rc == 0
    assert vis.TextureMapping(frames, info, m, opt, ctx=vt._ctx, slot=1)
    assert np.array_equal(m.textures[0], want_t)
    assert np.array_equal(m.uv.view(np.uint32), want_uv.view(np.uint32))
    if want_m is not None:
        assert np.array_equal(m.texture_mask, want_m)
    if want_uvi is not None:
        assert np.array_equal(m.uv_indices, want_uvi)
    assert list(np.unique(m.material_ids)) == [0]
    # the atlas in use: render the re-textured mesh
    ropt = RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1, backface_culling=True)
    cam = frames[0].camera
    rc, ref, _ = oracle_lib.render(m, cam, ropt)
    assert rc == 0
    ctx = Context(0)
    try:
        rc, got = gpu_render(ctx, m, cam, ropt)
        assert rc == 0, ctx.last_error()
        compare(ref, got, "atlas render")
    finally:
        ctx.close()


@pytest.mark.parametrize("uv_type", [vis.TexturingOutputUvType.kGenerateSimpleTile,
                                     vis.TexturingOutputUvType.kUseOriginalMeshUv,
                                     vis.TexturingOutputUvType.kGenerateSimpleTriangles,
                                     vis.TexturingOutputUvType.kGenerateSimpleCharts])
@pytest.mark.parametrize("criteria", [vis.ViewSelectionCriteria.kMaxArea,
                                      vis.ViewSelectionCriteria.kMinViewingAngle])
@pytest.mark.parametrize("tex,facewise", [(256, False), (64, True)])
def test_texture_mapping_pinned_to_the_reference(oracle_lib, uv_type, criteria, tex, facewise):
    """TextureMapping against the reference's own (src/texturing/
    texture_mapper.cc after its own VisibilityTester, built into
    oracle/_ref): the oracle's restatements of each uv type, fed by the
    host mirror's VisibilityInfo (itself pinned) and best keyframes, give
    the reference's texture, uv, uv indices and material ids, bit for bit
    (a 64 x 64 texture makes the chart atlas grow).  Runs where the
    reference checkout is present."""
    ref_build = pytest.importorskip("oracle.ref_build")
    if not ref_build.available():
        pytest.skip("reference sources not present")
    from test_visibility import keyframes, oracle_run, option
    T = vis.TexturingOutputUvType
    m = scenes.icosphere_textured(3, 64)
    base = 10 if uv_type == T.kGenerateSimpleTile else 0  # other types index the list by id
    kfs = [(base + i, cam, im) for i, (_, cam, im) in enumerate(keyframes(oracle_lib, m, n=4))]
    o = option()
    tex_w = tex_h = tex
    rc, r_tex, r_uv, r_uvi, r_mat = ref_build.texture_mapping(
        m.vertices, m.normals, m.vertex_indices,
        [(kid, cam, im["color"], im["depth"], im["mask"]) for kid, cam, im in kfs], o, facewise,
        criteria, uv_type, tex_w, tex_h,
        uv=m.uv if uv_type == T.kUseOriginalMeshUv else None,
        uv_indices=m.uv_indices if uv_type == T.kUseOriginalMeshUv else None)
    assert rc in (0, 4)  # 4: the reference's TextureMapping returned false
    ref_rejects = rc == 4
    info = vis.VisibilityInfo(m.num_vertices, m.num_faces)
    vis.assemble_visibility_info(info, [kid for kid, _, _ in kfs],
                                 oracle_run(oracle_lib, m, kfs, o, facewise), m.vertex_indices,
                                 o, facewise)
    face_kf, face_tri = vis.best_keyframes(info, criteria)
    assert (face_kf >= 0).mean() > 0.3
    colors = [im["color"] for _, _, im in kfs]
    F = m.num_faces
    want_uvi = np.arange(3 * F, dtype=np.int32).reshape(-1, 3)
    if uv_type == T.kGenerateSimpleTile:
        rc, want_t, want_uv = oracle_lib.simple_tile([kid for kid, _, _ in kfs], colors,
                                                     face_kf, face_tri)
    elif uv_type == T.kGenerateSimpleCharts:
        rc, want_t, want_uv, want_uvi = oracle_lib.simple_charts(
            m.vertex_indices, colors, face_kf, face_tri, tex_w, tex_h)
    elif uv_type == T.kGenerateSimpleTriangles:
        rc, want_t, _, want_uv = oracle_lib.simple_triangles(colors, face_kf, face_tri,
                                                             tex_w, tex_h)
    else:
        rc, want_t, _ = oracle_lib.texture_mapping(m.uv, m.uv_indices, colors, face_kf,
                                                   face_tri, tex_w, tex_h)
        want_uv, want_uvi = m.uv, m.uv_indices
    if ref_rejects:  # e.g. 640 face-pair rectangles do not fit 64 x 64 texels
        assert rc != 0
        return
    assert rc == 0
    assert r_tex.shape == want_t.shape
    assert np.array_equal(r_tex, want_t), f"{(r_tex != want_t).any(-1).sum()} texels differ"
    assert np.array_equal(np.ascontiguousarray(r_uv, np.float32).view(np.uint32),
                          np.ascontiguousarray(want_uv, np.float32).view(np.uint32))
    assert np.array_equal(r_uvi, want_uvi)
    assert not r_mat.any()
