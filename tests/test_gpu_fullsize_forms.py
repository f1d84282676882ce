"""Parity against the oracle at the full sizes of the batched, streaming-edits and serving workloads.

* Batched: the 64 maps of the batched workload (chunk dims U[8,64] per axis, 320x180..1920x1080, K=16) run
  as one batch; after the streaming ramp, one frame is split into its draw + sync batch and its lighting
  batch, and eight of the maps (the largest, a 1920x1080 one, a 320x180 one and five seeded picks) are
  checked against the oracle on a sample of their pixels and request groups.
* Streaming edits: the 128x32x128-chunk map at 1280x720 with 1-512 chunks re-rolled before every frame and
  only edited, visible chunks relit; after several edited frames one frame is checked the same way.
* Serving: eight maps of the serving workload (the largest spec of the 256, 96x32x96 chunks at most, and
  seven seeded picks) served in mixed ticks (draws, relights, edit batches); each served map must equal a
  twin driven by direct calls bit for bit, and the twin's frames are checked against the oracle.

The oracle adopts the device's state before each checked phase (tile states, visible flags, lighting,
sample counts, request list) and restates a seeded sample of the phase: it lights each voxel and shades
each pixel independently, so a sample checks the same arithmetic as the whole frame.

Bar: hit index and face bit-exact, colour within 2e-6, lighting within 1e-4 relative.
"""
import numpy as np
import pytest

import doonengine_gb300 as dn
import parity_util as P
from doonengine_gb300 import configs
from oracle import oracle as O
from test_gpu_fullsize import rows_by_tile

pytestmark = pytest.mark.gpu


def state_of(vol, with_requests=False):
    st, vis, _, ns = vol.export_tiles()
    idx, d, s = vol.export_lighting()
    out = {"st": st, "vis": vis, "ns": ns, "idx": idx, "d": d, "s": s, "frame": vol.s.frameNum}
    if with_requests:
        out["reqs"] = vol.export_requests()
    return out


def oracle_from(vol, state):
    om = O.OracleMap(vol.map_size)
    om.import_state(vol.s, state["st"], state["vis"], state["frame"])
    om.import_lighting(state["idx"], state["d"], state["s"])
    om.import_samples(state["ns"])
    if "reqs" in state:
        om.set_requests(state["reqs"])
    return om


def check_draw(vol, om, image, view, proj, rng, npix, where):
    color, hit, face = image
    H, W = hit.shape
    pix = rng.choice(W * H, size=min(W * H, npix), replace=False).astype(np.uint32)
    iv, icv, ip = P.draw_mats(vol, view, proj)
    ora = om.draw(vol.s, iv, icv, ip, W, H, pixels=pix)
    gpu = (color.reshape(-1, 4)[pix], hit.ravel()[pix], face.ravel()[pix])
    P.compare_draw(gpu, ora, where)
    return int((gpu[1] != 0xFFFFFFFF).sum())


def check_light(vol, om, reqs, params, post, rng, ngroups, where):
    """post: (idx, diff, spec) after the lighting update; returns the number of voxels checked"""
    if len(reqs) == 0:
        return 0
    sample = rng.choice(len(reqs), size=min(len(reqs), ngroups), replace=False).astype(np.uint32)
    od, os_, ok = om.light_requests(vol.s, params, sample)
    gi, gd, gs = post
    order, start = rows_by_tile(vol.map_size, gi)
    checked = 0
    for j, r in enumerate(sample):
        tile, group = int(reqs[r]) >> 4, int(reqs[r]) & 15
        for lane in range(32):
            if not ok[j, lane]:
                continue
            k = start[tile] + group * 32 + lane
            assert k < start[tile + 1], "%s: request %d lane %d has no lit row" % (where, r, lane)
            row = order[k]
            assert P.lighting_close(gd[row], od[j, lane]).all() and P.lighting_close(gs[row], os_[j, lane]).all(), (
                "%s: request %d voxel %d: device %s / %s, oracle %s / %s"
                % (where, r, lane, gd[row], gs[row], od[j, lane], os_[j, lane]))
            checked += 1
    return checked


def test_batched_workload_sampled_parity(gpu_ready):
    lib = dn.load()
    specs = configs.batched_specs(64, seed=7)
    maps = []
    batch = None
    oms = {}
    try:
        for i, sp in enumerate(specs):
            vol, cfg = configs.build_volume("small", **sp)
            vol.s.mapId = i
            W, H = cfg["res"]
            v, p = vol.view_proj(H / W)
            maps.append((vol, dn.Image(W, H, on_device=True), v, p))
        batch = dn.Batch([m[0] for m in maps])
        warm = 6
        for f in range(warm):
            t = 1.0 + 0.25 * f
            batch.run([dn.Batch.item(vol, img, v, p, sync=(dn.DN_READ_WRITE, 1), light=(1, 1000, t))
                       for vol, img, v, p in maps])
            assert batch.finish(), lib.dn_cuda_last_error().decode()
        tiles = [m[0].num_tiles for m in maps]
        rng = np.random.default_rng(77)
        picks = [int(np.argmax(tiles)),
                 next(i for i, sp in enumerate(specs) if sp["res"] == (1920, 1080)),
                 next(i for i, sp in enumerate(specs) if sp["res"] == (320, 180))]
        for i in rng.permutation(len(maps)):
            if len(picks) == 8:
                break
            if int(i) not in picks:
                picks.append(int(i))
        pre = {i: state_of(maps[i][0]) for i in picks}
        for i in picks:
            oms[i] = oracle_from(maps[i][0], pre[i])
        t = 1.0 + 0.25 * warm
        # the checked frame: its draw + sync batch, then its lighting batch, over all 64 maps
        batch.run([dn.Batch.item(vol, img, v, p, sync=(dn.DN_READ_WRITE, 1)) for vol, img, v, p in maps])
        assert batch.finish(), lib.dn_cuda_last_error().decode()
        images = {i: tuple(x.copy() for x in maps[i][1].numpy()) for i in picks}
        mid = {i: state_of(maps[i][0], with_requests=True) for i in picks}
        hits = 0
        for i in picks:
            vol, img, v, p = maps[i]
            hits += check_draw(vol, oms[i], images[i], v, p, rng, 4096, "batched map %d draw" % i)
            oms[i].close()
            oms[i] = oracle_from(vol, mid[i])
        params = {i: oms[i].light_params(maps[i][0].s, 1, 1000, t) for i in picks}
        batch.run([dn.Batch.item(vol, light=(1, 1000, t)) for vol, img, v, p in maps])
        assert batch.finish(), lib.dn_cuda_last_error().decode()
        checked = 0
        for i in picks:
            vol = maps[i][0]
            checked += check_light(vol, oms[i], mid[i]["reqs"], params[i], vol.export_lighting(), rng, 48,
                                   "batched map %d lighting" % i)
        assert hits > 4096, hits
        assert checked > 4000, checked
    finally:
        if batch is not None:
            batch.close()
        for vol, img, *_ in maps:
            img.close()
            vol.close()
        for om in oms.values():
            om.close()


def test_streaming_workload_sampled_parity(gpu_ready):
    lib = dn.load()
    seed = 31
    vol, cfg = configs.build_volume("small", map=(128, 32, 128), seed=seed, mean=0.1, amp=0.05, shapes=0,
                                    res=(1280, 720), K=16, cam=(0.1, 0.8, 0.1, 25.0, 45.0))
    W, H = cfg["res"]
    sx, sy, sz = cfg["map"]
    flags = np.array([vol.s.map[t].flag for t in range(vol.num_tiles)], np.uint8)
    occ = np.nonzero(flags)[0]
    chunk_pos = np.stack([occ % sx, (occ // sx) % sy, occ // (sx * sy)], 1).astype(np.int32)
    rng = np.random.default_rng(seed)
    img = dn.Image(W, H, on_device=True)
    split = 1 << 30
    om = None

    def edit_and_move(f):
        vol.s.camPos.x = float(0.1 * sx + 2.0 * f)
        vol.s.camPos.z = float(0.1 * sz + 1.5 * f)
        n = int(rng.integers(1, 513))
        sel = np.ascontiguousarray(chunk_pos[rng.integers(len(chunk_pos), size=n)])
        lib.dn_scene_reroll(vol.ptr, sel.ctypes.data, n, seed * 7919 + f, 14)
        return n

    try:
        warm = 6
        for f in range(warm):
            edit_and_move(f)
            v, p = vol.view_proj(H / W)
            vol.draw(img, v, p)
            vol.sync(dn.DN_READ_WRITE, split)
            vol.update_lighting(1, 1000, 1.0 + 0.25 * f)
        assert vol.finish(), lib.dn_cuda_last_error().decode()
        # the oracle adopts the state the device holds before the frame's edits are synced
        om = oracle_from(vol, state_of(vol))
        edited = edit_and_move(warm)
        v, p = vol.view_proj(H / W)
        vol.draw(img, v, p)
        assert vol.finish(), lib.dn_cuda_last_error().decode()
        hits = check_draw(vol, om, tuple(x.copy() for x in img.numpy()), v, p, rng, 16384, "streaming draw")
        om.close()
        vol.sync(dn.DN_READ_WRITE, split)
        mid = state_of(vol, with_requests=True)
        om = oracle_from(vol, mid)
        t = 1.0 + 0.25 * warm
        params = om.light_params(vol.s, 1, 1000, t)
        vol.update_lighting(1, 1000, t)
        assert vol.finish(), lib.dn_cuda_last_error().decode()
        checked = check_light(vol, om, mid["reqs"], params, vol.export_lighting(), rng, 256, "streaming lighting")
        assert edited >= 1 and hits > 1000, (edited, hits)
        assert checked > 500, checked
    finally:
        if om is not None:
            om.close()
        img.close()
        vol.close()


def test_serving_workload_maps_served_match_direct_and_oracle(gpu_ready):
    lib = dn.load()
    all_specs = configs.serving_specs(256, seed=11)
    sizes = [int(np.prod(sp["map"])) for sp in all_specs]
    rng = np.random.default_rng(5)
    pick = [int(np.argmax(sizes))] + [int(i) for i in rng.choice(len(all_specs), size=12, replace=False)
                                      if int(i) != int(np.argmax(sizes))][:7]
    specs = [all_specs[i] for i in pick]

    def build():
        out = []
        for k, sp in enumerate(specs):
            vol, cfg = configs.build_volume("small", **sp)
            vol.s.mapId = pick[k]
            out.append(vol)
        return out

    served, twins = build(), build()
    server = dn.Server(served, budget_bytes=0)
    images = []
    oms = []
    try:
        # the script of every map: draw, relight, draw, relight, [edit batch,] relight, draw
        scripts = []
        for k, sp in enumerate(specs):
            sx, sy, sz = sp["map"]
            edits = []
            if k % 2 == 0:
                for _ in range(int(rng.integers(1, 257))):
                    mp = (int(rng.integers(sx)), int(rng.integers(sy)), int(rng.integers(sz)))
                    for _ in range(4):
                        cp = tuple(int(c) for c in rng.integers(8, size=3))
                        edits.append((mp, cp, int(rng.integers(16)), (0.0, 1.0, 0.0),
                                      tuple(int(c) for c in rng.integers(40, 240, size=3)), bool(rng.random() < 0.25)))
            steps = [("draw",), ("relight", 0.75), ("draw",), ("relight", 1.0)]
            if edits:
                steps.append(("edit", edits))
            steps += [("relight", 1.25)]
            scripts.append(steps)
        # served: every map's requests interleaved into one stream, so ticks mix maps and request kinds
        reqs = []
        for n in range(max(len(s) for s in scripts)):
            for k, steps in enumerate(scripts):
                if n >= len(steps):
                    continue
                st = steps[n]
                W, H = specs[k]["res"]
                v, p = served[k].view_proj(H / W)
                if st[0] == "draw":
                    im = dn.Image(W, H, on_device=True)
                    images.append(im)
                    reqs.append(server.draw_request(k, im, v, p))
                elif st[0] == "relight":
                    reqs.append(server.relight_request(k, 1, 1000, st[1]))
                else:
                    reqs.append(server.edit_request(k, st[1]))
        server.start()
        for q in reqs:
            server.submit(q)
        assert server.drain(600.0), "the served script did not drain"
        server.poll()
        # twins: the same scripts as direct calls
        for k, steps in enumerate(scripts):
            vol = twins[k]
            W, H = specs[k]["res"]
            v, p = vol.view_proj(H / W)
            for st in steps:
                if st[0] == "draw":
                    im = dn.Image(W, H, on_device=True)
                    vol.draw(im, v, p)
                    im.close()
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
            assert vol.finish(), lib.dn_cuda_last_error().decode()
        for k in range(len(specs)):
            a, b = served[k].export_tiles(), twins[k].export_tiles()
            for x, y, name in zip(a, b, ("state", "visible", "lastUsed", "samples")):
                assert np.array_equal(x, y), "map %d: tile %s differs between served and direct" % (pick[k], name)
            la, lb = served[k].export_lighting(), twins[k].export_lighting()
            assert np.array_equal(la[0], lb[0])
            assert np.array_equal(la[1].view(np.uint32), lb[1].view(np.uint32)), "map %d diffuse" % pick[k]
            assert np.array_equal(la[2].view(np.uint32), lb[2].view(np.uint32)), "map %d specular" % pick[k]
        # one more frame on every twin, checked against the oracle
        hits = checked = 0
        for k, vol in enumerate(twins):
            W, H = specs[k]["res"]
            v, p = vol.view_proj(H / W)
            om = oracle_from(vol, state_of(vol))
            oms.append(om)
            im = dn.Image(W, H, on_device=True)
            images.append(im)
            vol.draw(im, v, p)
            assert vol.finish()
            hits += check_draw(vol, om, tuple(x.copy() for x in im.numpy()), v, p, rng, 4096,
                               "serving map %d draw" % pick[k])
            vol.sync(dn.DN_READ_WRITE, 1)
            mid = state_of(vol, with_requests=True)
            om2 = oracle_from(vol, mid)
            oms.append(om2)
            params = om2.light_params(vol.s, 1, 1000, 1.5)
            vol.update_lighting(1, 1000, 1.5)
            assert vol.finish()
            checked += check_light(vol, om2, mid["reqs"], params, vol.export_lighting(), rng, 48,
                                   "serving map %d lighting" % pick[k])
        assert hits > 4096 and checked > 2000, (hits, checked)
    finally:
        server.close()
        for om in oms:
            om.close()
        for im in images:
            im.close()
        for v in served + twins:
            v.close()
