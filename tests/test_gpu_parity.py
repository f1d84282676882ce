"""CUDA path vs the CPU oracle, through the C ABI (libdoonengine.so), frame by frame.

Bar: hit voxel index, face, depth, tile states, visible flags, lastUsed, sample counts and request sets
identical; per-voxel FP32 lighting within 1e-4 relative (it is expected to be bit-identical: both sides
run the same operation sequence without FMA contraction); draw colour within 2e-6 (pow() rounding).
"""
import numpy as np
import pytest

from parity_util import Pair, compare_draw, compare_lighting, compare_tiles, draw_mats
import doonengine_gb300 as dn

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_frames_match_oracle(gpu_ready, name):
    pair = Pair(name)
    try:
        frames = 4 if name == "tiny" else 3
        for _ in range(frames):
            pair.step()
        st = pair.vol.stats()
        oc = pair.om.counters()
        # traversal counters are exact integers on both sides
        for k_gpu, k_or in (("rays", "rays"), ("primaryRays", "primary"), ("outerSteps", "outerSteps"),
                            ("chunksEntered", "chunksEntered"), ("innerSteps", "innerSteps"), ("hits", "hits"),
                            ("litVoxels", "litVoxels"), ("degenerate", "degenerate")):
            assert st[k_gpu] == oc[k_or], (k_gpu, st[k_gpu], oc[k_or])
        assert st["litVoxels"] > 0
    finally:
        pair.close()


def test_bitexact_lighting_small(gpu_ready):
    pair = Pair("small")
    try:
        for _ in range(3):
            pair.draw()
            pair.sync()
            n, nbits = pair.light()
        assert n > 0
        assert nbits == 0, "%d voxels not bit-identical" % nbits
    finally:
        pair.close()


@pytest.mark.parametrize("split", [2, 3])
def test_lighting_split(gpu_ready, split):
    pair = Pair("tiny")
    try:
        for _ in range(5):
            pair.draw()
            pair.sync(split=split)
            pair.light()
    finally:
        pair.close()


@pytest.mark.parametrize("op", [0, 1])
def test_sync_ops(gpu_ready, op):
    """DN_READ only builds requests; DN_WRITE only streams (voxel.c:756-761)."""
    pair = Pair("tiny")
    try:
        pair.step()
        pair.draw()
        pair.sync(op=op)
        pair.light()
        pair.step()
    finally:
        pair.close()


def test_edits_between_frames(gpu_ready):
    """Streaming edits: changed chunks are re-packed, their lighting and sample count restart."""
    pair = Pair("tiny")
    rng = np.random.default_rng(7)
    try:
        for f in range(6):
            pair.draw()
            pair.sync()
            pair.light()
            sx, sy, sz = pair.vol.map_size
            for _ in range(40):
                mp = (int(rng.integers(sx)), int(rng.integers(sy)), int(rng.integers(sz)))
                cp = (int(rng.integers(8)), int(rng.integers(8)), int(rng.integers(8)))
                if rng.random() < 0.4:
                    pair.vol.remove_voxel(mp, cp)
                else:
                    pair.vol.set_voxel(mp, cp, int(rng.integers(16)), (rng.normal(), rng.normal(), rng.normal()),
                                       tuple(int(x) for x in rng.integers(0, 256, 3)))
    finally:
        pair.close()


def test_transparent_and_refractive(gpu_ready):
    """Transparency accumulation and refraction in the draw (voxelShared.comp:357-409)."""
    pair = Pair("tiny")
    try:
        for m in range(0, 16, 3):
            pair.vol.set_material(m, opacity=0.5, refract=1.52, specular=0.2, reflect_type=1, shininess=3)
        for _ in range(4):
            pair.step()
    finally:
        pair.close()


def test_view_modes(gpu_ready):
    pair = Pair("tiny")
    try:
        for _ in range(3):
            pair.step()
        for mode in range(7):
            pair.vol.s.camViewMode = mode
            pair.draw()
    finally:
        pair.close()


def test_truncated_dispatch(gpu_ready):
    pair = Pair("tiny", res=(100, 70))
    try:
        pair.vol.s.truncateDispatch = 1
        for _ in range(3):
            pair.step()
    finally:
        pair.close()


def test_reference_rng_mode(gpu_ready):
    """RNG mode A: the reference's fract(sin(s)*43758.5453) with the deterministic sine."""
    pair = Pair("tiny")
    try:
        pair.vol.s.rngMode = 1
        for _ in range(4):
            pair.step(time=3.75)
    finally:
        pair.close()


def test_empty_and_single_voxel_maps(gpu_ready):
    dn.init()
    from oracle import oracle as O
    for fill in (False, True):
        vol = dn.Volume((3, 2, 4), 16)
        om = O.OracleMap(vol.map_size)
        if fill:
            vol.set_voxel((1, 0, 2), (3, 4, 5), 0, (0.0, 1.0, 0.0), (200, 100, 50))
            vol.set_material(0, specular=0.3, reflect_type=1, shininess=2)
        vol.camera(0.5, 0.9, 0.1, 30.0, 10.0)
        img = dn.Image(48, 32)
        try:
            for f in range(3):
                v, p = vol.view_proj(32 / 48)
                iv, icv, ip = draw_mats(vol, v, p)
                vol.draw(img, v, p)
                compare_draw(img.numpy(), om.draw(vol.s, iv, icv, ip, 48, 32), "fill=%s f=%d" % (fill, f))
                om.sync(vol.s)
                vol.sync()
                om.light(vol.s, 1, 1000, 2.0 + f)
                vol.update_lighting(1, 1000, 2.0 + f)
                assert vol.finish()
                compare_lighting(vol, om)
                compare_tiles(vol, om)
        finally:
            img.close()
            vol.close()
            om.close()


def test_camera_inside_map_and_host_image(gpu_ready):
    """Camera inside a full map (AABB entry skipped), drawing into pinned host memory."""
    pair = Pair("tiny", cam=(0.5, 0.25, 0.5, 10.0, 200.0))
    try:
        for _ in range(3):
            pair.step()
        host = dn.Image(pair.W, pair.H, on_device=False)
        v, p, (iv, icv, ip) = pair.matrices()
        pair.vol.draw(host, v, p)
        assert pair.vol.finish()
        compare_draw(host.numpy(), pair.om.draw(pair.vol.s, iv, icv, ip, pair.W, pair.H), "host image")
        host.close()
    finally:
        pair.close()


def test_degenerate_ray_ends_at_once(gpu_ready):
    """A primary ray whose direction has an exactly zero x component: normalize((-1e-4, 0.6, 0.8)) + EPS
    gives x = 0 in float32, so the reference's x side distance would become 0 * inf = NaN after one step and
    its loop could never finish.  Both sides end such a segment at once as a miss (D16), with the same
    pixels and the same counters: no cell visited, one degenerate segment per pixel."""
    import ctypes
    from doonengine_gb300 import _lib
    lib = dn.load()
    pair = Pair("tiny")
    try:
        pair.sync()                       # load the chunks so the ray walks through loaded ones too
        W, H = 8, 4
        iv, icv, ip = _lib.DNmat4(), _lib.DNmat4(), _lib.DNmat4()
        for c in range(4):
            icv.m[c][c] = 1.0
            iv.m[c][c] = 1.0
        iv.m[3][0], iv.m[3][1], iv.m[3][2] = 2.5, 1.5, 2.5           # camera inside the map (chunk units)
        ip.m[3][0], ip.m[3][1], ip.m[3][2], ip.m[3][3] = -1e-4, 0.6, 0.8, 1.0
        M = lib.DN_mat4_mult(icv, ip)
        p = _lib.DnDrawParams()
        p.origin[:] = [2.5, 1.5, 2.5]
        for c in range(4):
            for r in range(4):
                p.dirMat[c][r] = M.m[c][r]
        p.width, p.height = W, H
        s = pair.vol.s
        p.sunStrength[:] = s.sunStrength.tolist()
        p.skyBot[:] = s.skyGradientBot.tolist()
        p.skyTop[:] = s.skyGradientTop.tolist()
        p.emissiveStrength = s.emissiveStrength
        img = dn.Image(W, H, on_device=True)
        pair.vol.reset_stats()
        assert lib.dn_cuda_draw(s.gpu, ctypes.byref(p), ctypes.cast(s.materials, ctypes.c_void_p),
                                ctypes.cast(img.ptr.contents.color, ctypes.c_void_p),
                                ctypes.cast(img.ptr.contents.hitIndex, ctypes.c_void_p),
                                ctypes.cast(img.ptr.contents.hitFace, ctypes.c_void_p)) == 0
        assert pair.vol.finish()
        gpu = img.numpy()
        ora = pair.om.draw(s, iv, icv, ip, W, H)
        compare_draw(gpu, ora, "degenerate ray")
        st = pair.vol.stats_kind(1)
        assert st["outerSteps"] + st["innerSteps"] == 0, st
        assert st["degenerate"] == W * H and st["rays"] == W * H, st
        assert (gpu[1] == 0xFFFFFFFF).all()
        img.close()
    finally:
        pair.close()


def test_degenerate_lighting_segments_match_oracle(gpu_ready):
    """Lighting segments with an exactly zero direction component occur on their own in the batched
    workload: specular bounces (reflect() without an added EPSILON, voxelLighting.comp:132) and diffuse
    lobe directions (163).  Map 63 of the batched workload's 64 holds one in frame 2 and three by frame 4.
    Every frame must match the oracle, the degenerate-segment counter included (D16)."""
    from doonengine_gb300 import configs
    spec = configs.batched_specs(64, seed=7)[63]
    pair = Pair("small", **spec)
    pair.vol.s.mapId = 63
    try:
        for _ in range(5):
            pair.step()
        st = pair.vol.stats()
        oc = pair.om.counters()
        assert st["degenerate"] == oc["degenerate"] >= 3, (st["degenerate"], oc["degenerate"])
        assert st["rays"] == oc["rays"] and st["outerSteps"] == oc["outerSteps"]
    finally:
        pair.close()


def _window_depth(proj, t):
    """GL window depth of a point at view distance t straight ahead (z_eye = -t) under projection proj
    (column-major m[col][row]): clip z / clip w mapped from [-1, 1] to [0, 1]."""
    m = np.array([[proj.m[c][r] for r in range(4)] for c in range(4)], np.float64)
    cz = m[2][2] * -t + m[3][2]
    cw = m[2][3] * -t + m[3][3]
    return (0.5 * cz / cw + 0.5).astype(np.float32)


def _raster_scene(rng, depth_px, proj, shape):
    """Raster colour and window depth of 'shape' straddling the voxel depths of depth_px: per texel
    nothing (depth 1), a surface 0.5-1.5x as far as the voxel seen there, or one at a random distance."""
    h, w = shape
    hh, ww = depth_px.shape
    ys = (np.arange(h) * hh // h)[:, None]
    xs = (np.arange(w) * ww // w)[None, :]
    vox = depth_px[ys, xs]
    t = np.where(vox > 0, vox * rng.uniform(0.5, 1.5, (h, w)), rng.uniform(0.5, 40.0, (h, w)))
    depth = _window_depth(proj, t)
    depth = np.where(rng.random((h, w)) < 0.2, np.float32(1.0), depth).astype(np.float32)
    color = rng.random((h, w, 4), dtype=np.float32)
    return color, depth


@pytest.mark.parametrize("tex_scale,transparent", [((1, 1), False), ((2, 3), True)])
def test_raster_composition(gpu_ready, tex_scale, transparent):
    """DN_draw with raster colour / depth textures (voxelDraw.comp:86-136): raster surfaces in front of
    voxels replace them, transparent voxels in front of a raster surface tint it, texture sizes other than
    the image's wrap (GL_REPEAT) and filter (GL_LINEAR) as the oracle restates them."""
    pair = Pair("tiny")
    rng = np.random.default_rng(17)
    try:
        if transparent:
            for m in range(0, 16, 3):
                pair.vol.set_material(m, opacity=0.5, refract=1.52, specular=0.2, reflect_type=1, shininess=3)
        for _ in range(3):
            pair.step()
        v, p, (iv, icv, ip) = pair.matrices()
        plain = pair.img.numpy()[0][..., 3]
        th, tw = pair.H // tex_scale[0] + 1, pair.W // tex_scale[1] + 3
        color, depth = _raster_scene(rng, plain, p, (th, tw))
        depth2 = _raster_scene(rng, plain, p, (pair.H, pair.W))[1] if tex_scale != (1, 1) else depth
        ct = dn.Texture(tw, th, dn.Texture.RGBA32F)
        dt = dn.Texture(depth2.shape[1], depth2.shape[0], dn.Texture.DEPTH32F)
        ct.upload(color)
        dt.upload(depth2)
        pair.vol.draw(pair.img, v, p, raster=(ct, dt))
        gpu = pair.img.numpy()
        ora = pair.om.draw(pair.vol.s, iv, icv, ip, pair.W, pair.H, raster=(color, depth2))
        compare_draw(gpu, ora, "raster composition")
        compare_tiles(pair.vol, pair.om, "raster composition")
        hit_plain = plain > 0
        occluded = hit_plain & (gpu[1] == 0xFFFFFFFF)
        shown = hit_plain & (gpu[1] != 0xFFFFFFFF)
        assert occluded.sum() > 0 and shown.sum() > 0, (int(occluded.sum()), int(shown.sum()))
        # a bad handle is refused with an error and draws nothing
        before = gpu[0].copy()
        pair.vol.draw(pair.img, v, p, raster=(dt, ct))
        assert np.array_equal(pair.img.numpy()[0].view(np.uint32), before.view(np.uint32))
        # the C ABI refuses raster buffers that are not device memory, before any launch
        import ctypes
        from doonengine_gb300 import _lib
        lib = dn.load()
        host = np.zeros(64, np.float32)
        ct_ptr = lib.DN_texture_device_pointer(ct.handle, None, None)
        assert ct_ptr
        for compose, ptr in ((1, host.ctypes.data), (2, ct_ptr)):
            dp = _lib.DnDrawParams()
            dp.width, dp.height, dp.compose = 4, 4, compose
            dp.rasterColor = dp.rasterDepth = ptr
            dp.rasterColorW = dp.rasterColorH = dp.rasterDepthW = dp.rasterDepthH = 4
            rc = lib.dn_cuda_draw(pair.vol.s.gpu, ctypes.byref(dp), ctypes.cast(pair.vol.s.materials, ctypes.c_void_p),
                                  ctypes.cast(pair.img.ptr.contents.color, ctypes.c_void_p), None, None)
            assert rc == 1, (compose, rc)
        assert pair.vol.finish()
        ct.close()
        dt.close()
    finally:
        pair.close()


@pytest.mark.parametrize("K", [1, 2, 3, 5])
def test_small_fan_counts(gpu_ready, K):
    """Few direct / specular rays per voxel: the packet kernel's pools then hold more than 16 voxels
    (128 / K), so its per-pool sums take more than one round of lanes."""
    pair = Pair("tiny", K=K)
    try:
        for _ in range(3):
            pair.step()
    finally:
        pair.close()


@pytest.mark.parametrize("K", [32, 33, 48, 64])
def test_large_fan_counts(gpu_ready, K):
    """A fan of exactly one warp, just over one, and up to the maximum of 64 rays per voxel: a pool then
    holds 4, 3, 2 or 2 voxels, and a fan's rays span lanes of more than one refill."""
    pair = Pair("tiny", K=K)
    try:
        for _ in range(3):
            pair.step()
    finally:
        pair.close()


@pytest.mark.parametrize("spec,diff", [(0, 5), (1, 1), (3, 2), (4, 0)])
def test_bounce_limits(gpu_ready, spec, diff):
    """specBounceLimit 0..4 (above 2 the lighting runs the per-lane-stream kernel) and diffuseBounceLimit
    0..5, with specular, reflecting materials so that specular rays bounce"""
    pair = Pair("tiny")
    try:
        pair.vol.s.specBounceLimit = spec
        pair.vol.s.diffuseBounceLimit = diff
        for m in range(0, 16, 2):
            pair.vol.set_material(m, specular=0.6, reflect_type=1 + m % 2, shininess=2 + m % 3)
        for _ in range(3):
            pair.step()
    finally:
        pair.close()


@pytest.mark.parametrize("nd,md", [(2, 1000), (3, 2)])
def test_several_diffuse_samples(gpu_ready, nd, md):
    """numDiffuseSamples > 1 per voxel and a small maxDiffuseSamples (the running average's weight caps)"""
    pair = Pair("tiny")
    try:
        for _ in range(4):
            pair.step(num_diffuse=nd, max_diffuse=md)
    finally:
        pair.close()
