"""The serving loop (include/DoonEngine/serve.h) through its C API.

A request's results must not depend on what else is being served: a volume's request sequence gives the
same images, tile state and FP32 lighting, bit for bit, when it is served alone, when it is mixed with
concurrent traffic on other volumes (continuous batching, up to two ticks in flight), when the volume is
evicted to host memory and restored between its requests, and when the same calls are made directly
(DN_draw / DN_sync_gpu + DN_update_lighting / edits + DN_sync_gpu).
"""
import numpy as np
import pytest

from parity_util import ROOT  # noqa: F401
import doonengine_gb300 as dn
from doonengine_gb300 import configs

pytestmark = pytest.mark.gpu

SPECS = [
    dict(map=(6, 4, 5), seed=21, res=(80, 48), K=8),
    dict(map=(5, 5, 5), seed=22, res=(64, 64), K=6),
    dict(map=(8, 3, 6), seed=23, res=(96, 54), K=8),
    dict(map=(4, 4, 4), seed=24, res=(40, 30), K=4),
]


def build():
    dn.init()
    vols = []
    for sp in SPECS:
        v, cfg = configs.build_volume("tiny", **sp)
        v.s.mapId = sp["seed"]
        vols.append(v)
    return vols


def script(rng, vol_index, n, spec):
    """A request sequence for one volume: list of ('draw',) / ('relight', t) / ('edit', edits)."""
    sx, sy, sz = spec["map"]
    out = []
    for k in range(n):
        r = rng.random()
        if r < 0.5:
            out.append(("draw",))
        elif r < 0.85:
            out.append(("relight", 0.5 + 0.25 * k))
        else:
            edits = []
            for _ in range(int(rng.integers(1, 12))):
                mp = (int(rng.integers(sx)), int(rng.integers(sy)), int(rng.integers(sz)))
                cp = tuple(int(c) for c in rng.integers(8, size=3))
                edits.append((mp, cp, int(rng.integers(16)), (0.0, 1.0, 0.0), (90, 200, 60), bool(rng.random() < 0.3)))
            out.append(("edit", edits))
    return out


def to_requests(server, vi, vol, steps, images):
    W, H = SPECS[vi]["res"]
    v, p = vol.view_proj(H / W)
    reqs = []
    for k, st in enumerate(steps):
        if st[0] == "draw":
            img = dn.Image(W, H, on_device=(k % 2 == 0))
            images.append(img)
            reqs.append(server.draw_request(vi, img, v, p))
        elif st[0] == "relight":
            reqs.append(server.relight_request(vi, 1, 1000, st[1]))
        else:
            reqs.append(server.edit_request(vi, st[1]))
    return reqs


def direct(vol, vi, steps, images):
    """The same sequence as direct calls."""
    W, H = SPECS[vi]["res"]
    v, p = vol.view_proj(H / W)
    for k, st in enumerate(steps):
        if st[0] == "draw":
            img = dn.Image(W, H, on_device=(k % 2 == 0))
            images.append(img)
            vol.draw(img, v, p)
        elif st[0] == "relight":
            vol.sync(dn.DN_READ_WRITE, 1)
            vol.update_lighting(1, 1000, st[1])
        else:
            for mp, cp, mat, nrm, alb, rem in st[1]:
                if rem:
                    vol.remove_voxel(mp, cp)
                else:
                    vol.set_voxel(mp, cp, mat, nrm, alb)
            vol.sync(dn.DN_READ_WRITE, 1)
    assert vol.finish()


def snapshot(vol, images):
    imgs = [tuple(x.copy() for x in im.numpy()) for im in images]
    tiles = vol.export_tiles()
    light = vol.export_lighting()
    return imgs, tiles, light


def same(a, b, where):
    ia, ta, la = a
    ib, tb, lb = b
    assert len(ia) == len(ib), where
    for k, (x, y) in enumerate(zip(ia, ib)):
        assert np.array_equal(x[0].view(np.uint32), y[0].view(np.uint32)), "%s: draw %d colour bits" % (where, k)
        assert np.array_equal(x[1], y[1]) and np.array_equal(x[2], y[2]), "%s: draw %d hit / face" % (where, k)
    for x, y, n in zip(ta, tb, ("state", "visible", "lastUsed", "samples")):
        assert np.array_equal(x, y), "%s: tile %s" % (where, n)
    assert np.array_equal(la[0], lb[0]), where + ": lit voxels"
    assert np.array_equal(la[1].view(np.uint32), lb[1].view(np.uint32)), where + ": diffuse bits"
    assert np.array_equal(la[2].view(np.uint32), lb[2].view(np.uint32)), where + ": specular bits"


def run_served(steps_by_vol, mix_order, budget=0, replay=False):
    """Serves the scripts; mix_order: list of volume indices giving the global submission order."""
    vols = build()
    server = dn.Server(vols, budget_bytes=budget)
    images = {vi: [] for vi in range(len(vols))}
    reqs = {vi: to_requests(server, vi, vols[vi], steps_by_vol.get(vi, []), images[vi]) for vi in range(len(vols))}
    cursor = {vi: 0 for vi in reqs}
    ordered = []
    for vi in mix_order:
        ordered.append(reqs[vi][cursor[vi]])
        cursor[vi] += 1
    if replay:
        # the first requests are queued before the server starts, so the first tick carries several
        # volumes whatever the GPU's speed; the rest arrive while ticks run (continuous batching)
        head = 8
        for r in ordered[:head]:
            server.submit(r)
        server.start()
        offs = np.cumsum(np.full(len(ordered) - head, 2e-4))
        assert server.replay(ordered[head:], offs) == len(ordered) - head
    else:
        server.start()
        for r in ordered:
            server.submit(r)
    try:
        assert server.drain(300.0)
        comps = server.poll()
        st = server.stats()
    finally:
        # closing the server restores evicted volumes and hands them back: only then are they readable
        server.close()
    snaps = {vi: snapshot(vols[vi], images[vi]) for vi in range(len(vols))}
    for im in images.values():
        for x in im:
            x.close()
    for v in vols:
        v.close()
    return snaps, comps, st


def test_alone_mix_direct_agree(gpu_ready):
    rng = np.random.default_rng(3)
    steps = {vi: script(rng, vi, 14, SPECS[vi]) for vi in range(4)}
    # volume 0 alone
    alone, comps_a, _ = run_served({0: steps[0]}, [0] * len(steps[0]))
    # volume 0 mixed with the other three, submitted interleaved while the server runs
    order = []
    left = {vi: len(steps[vi]) for vi in range(4)}
    while any(left.values()):
        vi = int(rng.choice([k for k in left if left[k]]))
        order.append(vi)
        left[vi] -= 1
    mixed, comps_m, st = run_served(steps, order, replay=True)
    same(alone[0], mixed[0], "volume 0 alone vs mixed")
    assert st["completed"] == len(order) and st["failed"] == 0
    assert all(c["ok"] for c in comps_m)
    assert all(c["arrival"] <= c["admitted"] <= c["finished"] for c in comps_m)
    assert st["items"] > st["ticks"], "no tick carried more than one volume"
    # every volume against the same calls made directly
    vols = build()
    for vi in range(4):
        imgs = []
        direct(vols[vi], vi, steps[vi], imgs)
        same(snapshot(vols[vi], imgs), mixed[vi], "volume %d direct vs served" % vi)
        for x in imgs:
            x.close()
        vols[vi].close()


def test_eviction_round_trips_are_exact(gpu_ready):
    rng = np.random.default_rng(9)
    steps = {vi: script(rng, vi, 10, SPECS[vi]) for vi in range(4)}
    order = []
    for k in range(10):
        order += [0, 1, 2, 3]
    ref, _, _ = run_served(steps, order)
    # a budget a little above the largest volume: every switch of volume evicts another one
    vols = build()
    fp = max(dn.load().dn_cuda_map_footprint(v.s.gpu) for v in vols)
    for v in vols:
        v.close()
    tight, comps, st = run_served(steps, order, budget=int(fp * 1.6))
    assert st["evictions"] > 0 and st["restores"] > 0, st
    assert all(c["ok"] for c in comps)
    for vi in range(4):
        same(ref[vi], tight[vi], "volume %d with evictions" % vi)


def test_submit_rejects_bad_requests(gpu_ready):
    vols = build()
    server = dn.Server(vols[:2])
    try:
        r = server.relight_request(5)
        with pytest.raises(RuntimeError):
            server.submit(r)
        bad = dn.Server.draw_request(0, dn.Image(8, 8), *vols[0].view_proj(1.0))
        bad.output = None
        with pytest.raises(RuntimeError):
            server.submit(bad)
        # raster handles that name no texture
        img = dn.Image(8, 8)
        bad = dn.Server.draw_request(0, img, *vols[0].view_proj(1.0))
        bad.rasterColorTexture, bad.rasterDepthTexture = 4000, 4001
        with pytest.raises(RuntimeError):
            server.submit(bad)
        server.start()
        assert server.drain(10.0)
    finally:
        server.close()
        for v in vols:
            v.close()


def test_direct_eviction_behind_queued_work_is_exact(gpu_ready):
    """dn_cuda_map_evict and dn_cuda_map_restore called right behind queued draws, syncs and lighting
    launches, without waiting for them: the copies run on their own streams, ordered after the volume's work
    and before its next work.  Every other round trip restores with dn_cuda_map_restore_async and is never
    polled, so the next entry point must make the volume's stream wait by itself.  Eviction after every
    phase and a twin that never leaves the device give the same images, tile state and lighting, bit for
    bit."""
    lib = dn.load()
    trips = [0]

    def restore(g):
        trips[0] += 1
        if trips[0] % 2:
            return lib.dn_cuda_map_restore(g) == 0
        return lib.dn_cuda_map_restore_async(g) == 0 and lib.dn_cuda_map_restore_query(g) in (0, 1)
    sp = dict(SPECS[2])
    twins = []
    for _ in range(2):
        v, _ = configs.build_volume("tiny", **sp)
        v.s.mapId = sp["seed"]
        twins.append(v)
    W, H = sp["res"]
    images = [[dn.Image(W, H, on_device=True) for _ in range(6)] for _ in twins]
    try:
        for f in range(6):
            for which, vol in enumerate(twins):
                roundtrip = (lambda: (lib.dn_cuda_map_evict(vol.s.gpu) == 0 and
                                      restore(vol.s.gpu))) if which == 1 else (lambda: True)
                v, p = vol.view_proj(H / W)
                vol.draw(images[which][f], v, p)
                assert roundtrip()
                vol.sync(dn.DN_READ_WRITE, 1)
                assert roundtrip()
                vol.update_lighting(1, 1000, 0.75 + 0.5 * f)
                assert roundtrip()
                if f == 3:
                    # an evicted volume stays evicted across other work, then comes back
                    if which == 1:
                        assert lib.dn_cuda_map_evict(vol.s.gpu) == 0
                        assert lib.dn_cuda_map_is_resident(vol.s.gpu) == 0
                        assert lib.dn_cuda_map_restore_query(vol.s.gpu) == 0
                        assert lib.dn_cuda_map_restore_async(vol.s.gpu) == 0
                        import time
                        for _ in range(10000):
                            q = lib.dn_cuda_map_restore_query(vol.s.gpu)
                            if q != 0:
                                break
                            time.sleep(0.0001)
                        assert q == 1
        for vol in twins:
            assert vol.finish(), lib.dn_cuda_last_error().decode()
        same(snapshot(twins[0], images[0]), snapshot(twins[1], images[1]), "evicted twin")
    finally:
        for imgs in images:
            for im in imgs:
                im.close()
        for vol in twins:
            vol.close()
