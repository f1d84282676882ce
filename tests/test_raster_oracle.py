"""The oracle's raster composition (voxelDraw.comp:24-30, 86-101, 127-136) against an independent numpy
statement of the same rules (no GPU).

On a map with no chunks, every ray that reaches the map ends in step_map's miss branch, so the pixel is
the background: the raster colour, sampled GL_LINEAR with GL_REPEAT at (x / colourWidth,
y / colourHeight) as the OpenGL 4.3 specification (section 8.14.2) defines the filter, then gamma
corrected.  The depth channel is the raster depth unprojected through the inverse projection.  Rays that
miss the map's box keep depth -1 and show the raster colour too.  Texture sizes that differ from the
image's exercise the wrap.
"""
import ctypes

import numpy as np
import pytest

from parity_util import ROOT  # noqa: F401
import doonengine_gb300 as dn
from doonengine_gb300 import _lib as L
from oracle import oracle as O


def gl_linear_repeat(tex, s, t):
    """GL_LINEAR + GL_REPEAT sample of tex (h, w, C) at texture coordinates s, t (arrays), float64."""
    h, w = tex.shape[:2]
    u = s * w - 0.5
    v = t * h - 0.5
    i0 = np.floor(u).astype(np.int64)
    j0 = np.floor(v).astype(np.int64)
    a = (u - i0)[..., None]
    b = (v - j0)[..., None]
    i1, j1 = (i0 + 1) % w, (j0 + 1) % h
    i0, j0 = i0 % w, j0 % h
    T = tex.astype(np.float64)
    return ((1 - a) * (1 - b) * T[j0, i0] + a * (1 - b) * T[j0, i1] + (1 - a) * b * T[j1, i0]
            + a * b * T[j1, i1])


@pytest.mark.parametrize("csize,dsize", [((48, 40), (48, 40)), ((17, 11), (29, 23))])
def test_oracle_composition_on_empty_map(csize, dsize):
    lib = dn.load()
    W, H = 48, 40
    vol = dn.Volume((4, 3, 5), 8, cpu_only=True)
    try:
        vol.camera(0.5, 0.5, -0.5, 0.0, 0.0)
        v, p = vol.view_proj(H / W)
        iv, icv, ip = L.DNmat4(), L.DNmat4(), L.DNmat4()
        lib.DN_draw_matrices(v, p, iv, icv, ip)
        rng = np.random.default_rng(5)
        cw, ch = csize
        dw, dh = dsize
        color = rng.random((ch, cw, 4), dtype=np.float32)
        depth = rng.uniform(0.05, 0.995, (dh, dw)).astype(np.float32)
        om = O.OracleMap(vol.map_size)
        out, hit, face = om.draw(vol.s, iv, icv, ip, W, H, raster=(color, depth))
        om.close()
    finally:
        vol.close()
    ys, xs = np.mgrid[0:H, 0:W]
    s = xs.astype(np.float32) / np.float32(cw)
    t = ys.astype(np.float32) / np.float32(ch)
    want_c = gl_linear_repeat(color, s, t)[..., :3] ** 0.4545
    d = gl_linear_repeat(depth[..., None], s, t)[..., 0] * 2.0 - 1.0
    P = np.array([[ip.m[c][r] for r in range(4)] for c in range(4)], np.float64)
    sx = xs / W * 2.0 - 1.0
    sy = ys / H * 2.0 - 1.0
    vs = [P[0][r] * sx + P[1][r] * sy + P[2][r] * d + P[3][r] for r in range(4)]
    want_d = np.sqrt((vs[0] / vs[3]) ** 2 + (vs[1] / vs[3]) ** 2 + (vs[2] / vs[3]) ** 2)
    assert (hit == 0xFFFFFFFF).all() and (face == 6).all()
    np.testing.assert_allclose(out[..., :3], want_c, rtol=2e-6, atol=2e-6)
    in_box = out[..., 3] >= 0
    assert in_box.sum() > W * H // 4 and (~in_box).sum() > 0, int(in_box.sum())
    np.testing.assert_allclose(out[..., 3][in_box], want_d[in_box], rtol=2e-6)
    assert (out[..., 3][~in_box] == -1.0).all()


def test_texture_handles_without_device():
    """Handles that name no texture are refused before any device work."""
    lib = dn.load()
    assert lib.DN_texture_format(0) == -1 and lib.DN_texture_format(-1) == -1 and lib.DN_texture_format(99999) == -1
    assert not lib.DN_texture_device_pointer(7, None, None)
    assert not lib.DN_texture_upload(3, ctypes.c_void_p(0))
