"""Parity at the headline workload's full size: 64x32x64 chunks, 1920x1080, K=32, heightfield plus 2000
boxes and spheres.  The device runs every frame; the oracle then adopts the device's tile states, lighting
and sample counts for one more frame and recomputes a seeded sample of it: pixels of the draw and request
groups of the lighting update (the oracle restates every voxel independently, so a sample checks the same
arithmetic as the whole frame).

Bar: hit index and face bit-exact, colour within 2e-6, lighting within 1e-4 relative.
"""
import numpy as np
import pytest

import doonengine_gb300 as dn
import parity_util as P
from doonengine_gb300 import configs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rows_by_tile(map_size, idx):
    """the lighting rows grouped by tile in rank order: (order of the rows, first row of each tile)"""
    sx, sy, sz = map_size
    X, Y = 8 * sx, 8 * sy
    g = idx.astype(np.int64)
    gx, gy, gz = g % X, (g // X) % Y, g // (X * Y)
    tile = gx // 8 + sx * (gy // 8 + sy * (gz // 8))
    li = gx % 8 + 8 * (gy % 8 + 8 * (gz % 8))
    order = np.lexsort((li, tile))
    start = np.searchsorted(tile[order], np.arange(sx * sy * sz + 1))
    return order, start


def test_large_frame_sampled_parity(gpu_ready):
    vol, cfg = configs.build_volume("large")
    W, H = cfg["res"]
    img = dn.Image(W, H, on_device=True)
    om = O.OracleMap(vol.map_size)
    rng = np.random.default_rng(2024)
    try:
        view, proj = vol.view_proj(H / W)
        for f in range(6):
            vol.draw(img, view, proj)
            vol.sync(dn.DN_READ_WRITE, 1)
            vol.update_lighting(1, 1000, 1.0 + 0.25 * f)
        assert vol.finish(), dn.load().dn_cuda_last_error().decode()

        # the draw of the next frame, sampled
        st, vis, _, ns = vol.export_tiles()
        idx, d, s = vol.export_lighting()
        om.import_state(vol.s, st, vis, vol.s.frameNum)
        om.import_lighting(idx, d, s)
        om.import_samples(ns)
        vol.draw(img, view, proj)
        color, hit, face = img.numpy()
        pix = rng.choice(W * H, size=16384, replace=False).astype(np.uint32)
        iv, icv, ip = P.draw_mats(vol, view, proj)
        ora = om.draw(vol.s, iv, icv, ip, W, H, pixels=pix)
        gpu = (color.reshape(-1, 4)[pix], hit.ravel()[pix], face.ravel()[pix])
        P.compare_draw(gpu, ora, "large frame draw sample")
        assert (gpu[1] != 0xFFFFFFFF).sum() > len(pix) // 10

        # its sync and lighting update, sampled
        vol.sync(dn.DN_READ_WRITE, 1)
        st, vis, _, ns = vol.export_tiles()
        reqs = vol.export_requests()
        idx, d, s = vol.export_lighting()
        om.import_state(vol.s, st, vis, vol.s.frameNum)
        om.import_lighting(idx, d, s)
        om.import_samples(ns)
        om.set_requests(reqs)
        t = 1.0 + 0.25 * 6
        params = om.light_params(vol.s, 1, 1000, t)
        vol.update_lighting(1, 1000, t)
        assert vol.finish(), dn.load().dn_cuda_last_error().decode()
        sample = rng.choice(len(reqs), size=min(len(reqs), 384), replace=False).astype(np.uint32)
        od, os_, ok = om.light_requests(vol.s, params, sample)

        gi, gd, gs = vol.export_lighting()
        order, start = rows_by_tile(vol.map_size, gi)
        checked = 0
        for j, r in enumerate(sample):
            tile, group = int(reqs[r]) >> 4, int(reqs[r]) & 15
            for lane in range(32):
                if not ok[j, lane]:
                    continue
                row = order[start[tile] + group * 32 + lane]
                assert start[tile] + group * 32 + lane < start[tile + 1]
                assert P.lighting_close(gd[row], od[j, lane]).all() and P.lighting_close(gs[row], os_[j, lane]).all(), (
                    "request %d voxel %d: device %s / %s, oracle %s / %s" % (r, lane, gd[row], gs[row], od[j, lane], os_[j, lane]))
                checked += 1
        assert checked > 5000, checked
    finally:
        om.close()
        img.close()
        vol.close()
