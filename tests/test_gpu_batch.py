"""Batched frames (DN_batch_run over the dn_cuda_batch_* C ABI) against the single-map calls.

Every map of a batch must come out exactly as if DN_draw, DN_sync_gpu and DN_update_lighting had been
called on it alone with the same arguments (the single-map path is itself checked against the oracle in
test_gpu_parity.py): images (colour with NaN positions, depth, hit index, face), tile states, visible
flags, lastUsed, sample counts, request sets and FP32 lighting, all bit for bit.  Cases: maps of uneven
size and resolution, device and host images, graph replay of repeated frames, frames that run only some
phases for some maps, edits staged between frames, autotuning between frames, a map leaving the batch.
"""
import numpy as np
import pytest

from parity_util import ROOT  # noqa: F401  (puts the repository on sys.path)
import doonengine_gb300 as dn
from doonengine_gb300 import configs

pytestmark = pytest.mark.gpu

SPECS = [
    dict(map=(5, 4, 6), seed=11, res=(96, 64), K=8),
    dict(map=(8, 5, 4), seed=12, res=(64, 48), K=12),
    dict(map=(4, 6, 5), seed=13, res=(120, 72), K=6),
    dict(map=(7, 3, 7), seed=14, res=(48, 40), K=16),
    dict(map=(3, 3, 3), seed=15, res=(32, 32), K=4),
]


def build_set(on_device_pattern=(True, False, True, False, True)):
    dn.init()
    out = []
    for spec, dev in zip(SPECS, on_device_pattern):
        vol, cfg = configs.build_volume("tiny", **spec)
        vol.s.mapId = spec["seed"]
        W, H = cfg["res"]
        img = dn.Image(W, H, on_device=dev)
        out.append((vol, img, W, H))
    return out


def frame_args(vol, W, H):
    v, p = vol.view_proj(H / W)
    return v, p


def solo_frame(maps, t, phases=None, op=2, split=1, rasters=None):
    for i, (vol, img, W, H) in enumerate(maps):
        ph = phases[i] if phases else "dsl"
        if "d" in ph:
            v, p = frame_args(vol, W, H)
            vol.draw(img, v, p, raster=rasters[i] if rasters else None)
        if "s" in ph:
            vol.sync(op, split)
        if "l" in ph:
            vol.update_lighting(1, 1000, t)
    for vol, *_ in maps:
        assert vol.finish(), dn.load().dn_cuda_last_error().decode()


def batch_frame(batch, maps, t, phases=None, op=2, split=1, rasters=None):
    items = []
    for i, (vol, img, W, H) in enumerate(maps):
        ph = phases[i] if phases else "dsl"
        if not ph:
            continue
        v, p = frame_args(vol, W, H)
        items.append(dn.Batch.item(vol, img if "d" in ph else None, v, p,
                                   sync=(op, split) if "s" in ph else None,
                                   light=(1, 1000, t) if "l" in ph else None,
                                   raster=rasters[i] if rasters else None))
    batch.run(items)
    assert batch.finish(), dn.load().dn_cuda_last_error().decode()


def same_state(a, b, where):
    (va, ia, _, _), (vb, ib, _, _) = a, b
    ca, ha, fa = ia.numpy()
    cb, hb, fb = ib.numpy()
    assert np.array_equal(ha, hb), where + ": hit index"
    assert np.array_equal(fa, fb), where + ": face"
    assert np.array_equal(ca.view(np.uint32), cb.view(np.uint32)), where + ": colour / depth bits"
    for x, y, name in zip(va.export_tiles(), vb.export_tiles(), ("state", "visible", "lastUsed", "samples")):
        assert np.array_equal(x, y), "%s: tile %s" % (where, name)
    assert np.array_equal(np.sort(va.export_requests()), np.sort(vb.export_requests())), where + ": requests"
    la, lb = va.export_lighting(), vb.export_lighting()
    assert np.array_equal(la[0], lb[0]), where + ": lit voxels"
    assert np.array_equal(la[1].view(np.uint32), lb[1].view(np.uint32)), where + ": diffuse bits"
    assert np.array_equal(la[2].view(np.uint32), lb[2].view(np.uint32)), where + ": specular bits"
    assert va.s.numLightingRequests == vb.s.numLightingRequests, where + ": numLightingRequests"


def close_all(*sets):
    for s in sets:
        for vol, img, _, _ in s:
            img.close()
            vol.close()


def test_batch_matches_single_maps(gpu_ready):
    solo, bat = build_set(), build_set()
    batch = dn.Batch([m[0] for m in bat])
    try:
        launches0 = dn.load().dn_cuda_launch_count()
        for f in range(5):       # frames 2.. repeat the composition: captured once, then replayed as a graph
            t = 1.25 + 0.5 * f
            solo_frame(solo, t)
            batch_frame(batch, bat, t)
            for i in range(len(SPECS)):
                same_state(solo[i], bat[i], "frame %d map %d" % (f, i))
        assert dn.load().dn_cuda_launch_count() > launches0
        st = batch.stats()
        assert st["rays"] > 0 and st["litVoxels"] > 0 and st["primaryRays"] > 0
    finally:
        batch.close()
        close_all(solo, bat)


def test_batch_partial_phases_and_edits(gpu_ready):
    solo, bat = build_set((True,) * 5), build_set((True,) * 5)
    batch = dn.Batch([m[0] for m in bat])
    rng = np.random.default_rng(5)
    plans = ["dsl", "ds", "sl", "l", "d", ""], ["sl", "dsl", "d", "", "dsl"], ["dsl"] * 5, ["l", "l", "dsl", "ds", "sl"]
    try:
        for f in range(8):
            phases = list(plans[f % len(plans)])[:5]
            phases += ["dsl"] * (5 - len(phases))
            t = 0.75 + 0.25 * f
            if f in (2, 5):
                # identical edits on both copies: the next sync stages the changed chunks
                for i in range(5):
                    sx, sy, sz = SPECS[i]["map"]
                    for _ in range(20):
                        mp = (int(rng.integers(sx)), int(rng.integers(sy)), int(rng.integers(sz)))
                        cp = tuple(int(c) for c in rng.integers(8, size=3))
                        mat = int(rng.integers(16))
                        for s in (solo, bat):
                            s[i][0].set_voxel(mp, cp, mat, (0.0, 1.0, 0.0), (200, 120, 40))
            solo_frame(solo, t, phases)
            batch_frame(batch, bat, t, phases)
            for i in range(5):
                same_state(solo[i], bat[i], "frame %d map %d (%s)" % (f, i, phases[i]))
    finally:
        batch.close()
        close_all(solo, bat)


def test_batch_autotune_keeps_results(gpu_ready):
    solo, bat = build_set(), build_set()
    batch = dn.Batch([m[0] for m in bat])
    try:
        for f in range(4):
            t = 2.0 + f
            solo_frame(solo, t)
            batch_frame(batch, bat, t)
            if f == 1:
                tun = batch.autotune()
                assert 1 <= tun["streamBatch"] <= 32 and tun["blocksPerSM"] >= 1
            for i in range(len(SPECS)):
                same_state(solo[i], bat[i], "frame %d map %d" % (f, i))
        batch.set_tuning(streamBatch=7, blocksPerSM=1, useGraph=0)
        for f in range(4, 6):
            t = 2.0 + f
            solo_frame(solo, t)
            batch_frame(batch, bat, t)
            for i in range(len(SPECS)):
                same_state(solo[i], bat[i], "frame %d map %d (untuned)" % (f, i))
        # the other pool size (rays a warp pulls per pool) and another diffuse compaction period
        batch.set_tuning(poolRays=64 if tun["poolRays"] == 128 else 128, diffuseBatch=5, kernel=2,
                         blocksPerSM=2, useGraph=1)
        for f in range(6, 8):
            t = 2.0 + f
            solo_frame(solo, t)
            batch_frame(batch, bat, t)
            for i in range(len(SPECS)):
                same_state(solo[i], bat[i], "frame %d map %d (pool %d)" % (f, i, batch.tuning()["poolRays"]))
    finally:
        batch.close()
        close_all(solo, bat)


def test_batch_membership_and_errors(gpu_ready):
    bat = build_set()
    solo = build_set()
    batch = dn.Batch([m[0] for m in bat[:4]])
    try:
        vol, img, W, H = bat[0]
        v, p = frame_args(vol, W, H)
        it = dn.Batch.item(vol, img, v, p, sync=(2, 1), light=(1, 1000, 1.0))
        with pytest.raises(RuntimeError):
            batch.run([it, it])                              # a map twice in one frame
        v4, p4 = frame_args(bat[4][0], bat[4][2], bat[4][3])
        with pytest.raises(RuntimeError):
            batch.run([dn.Batch.item(bat[4][0], bat[4][1], v4, p4)])   # not a member
        # a member leaves: its single-map calls run on its own stream again and stay exact
        batch.remove(bat[3][0])
        for f in range(2):
            t = 0.5 + f
            solo_frame(solo, t)
            batch_frame(batch, bat[:3], t)
            solo_frame(bat[3:], t)
            for i in range(5):
                same_state(solo[i], bat[i], "frame %d map %d" % (f, i))
    finally:
        batch.close()
        close_all(solo, bat)


def test_batch_then_delete_member(gpu_ready):
    bat = build_set()
    batch = dn.Batch([m[0] for m in bat])
    try:
        batch_frame(batch, bat, 1.0)
        vol, img, _, _ = bat.pop(2)
        img.close()
        vol.close()                  # DN_delete_volume takes the volume out of its batch
        batch.members = [m[0] for m in bat]
        batch_frame(batch, bat, 2.0)
    finally:
        batch.close()
        close_all(bat)


def test_batch_raster_composition(gpu_ready):
    """Draws composed with raster textures (DN_draw's rasterColorTexture / rasterDepthTexture) give the same
    images in a batch as alone, including graph replays that reuse the composition."""
    solo, bat = build_set(), build_set()
    batch = dn.Batch([m[0] for m in bat])
    rng = np.random.default_rng(8)
    textures = []
    try:
        rasters = []
        for k, (vol, img, W, H) in enumerate(solo):
            if k == 3:
                rasters.append(None)       # one map draws without composition
                continue
            tw, th = W // (1 + k % 2) + k, H // (1 + k % 2) + 1
            ct = dn.Texture(tw, th, dn.Texture.RGBA32F)
            dt = dn.Texture(W, H, dn.Texture.DEPTH32F)
            ct.upload(rng.random((th, tw, 4), dtype=np.float32))
            dt.upload(np.where(rng.random((H, W)) < 0.2, 1.0, rng.uniform(0.95, 1.0, (H, W))).astype(np.float32))
            textures += [ct, dt]
            rasters.append((ct, dt))
        for f in range(4):
            t = 1.25 + 0.5 * f
            solo_frame(solo, t, rasters=rasters)
            batch_frame(batch, bat, t, rasters=rasters)
            for i in range(len(SPECS)):
                same_state(solo[i], bat[i], "frame %d map %d" % (f, i))
    finally:
        batch.close()
        close_all(solo, bat)
        for x in textures:
            x.close()
