"""DN_RESIDENCY_LRU, the reference's fixed GPU voxel buffer with least-recently-used unloading
(voxel.c:1491-1695), on the CPU: the API on a CPU-only volume and the oracle's node model.

The reference's allocator touches OpenGL on every path, so it cannot run here and the node model is
unpinned; these tests check the invariants of the reference's algorithm (the nodes tile the buffer, a
loaded chunk owns exactly one node that fits it, an unloaded one owns none) and that both of the buffer's
decisions -- unloading a stale chunk and growing -- occur in a frame sequence.
"""
import ctypes

import numpy as np

import parity_util as P
from doonengine_gb300 import configs
from oracle import oracle as O


def test_api_on_a_cpu_volume():
    vol, _ = configs.build_volume("tiny", cpu_only=True, min_chunks=8)
    try:
        assert vol.lib.DN_get_residency(vol.ptr) == 0
        cap, sizes, starts, tiles = vol.residency_nodes()
        assert cap == 0 and len(sizes) == 0
        vol.set_residency("lru")
        assert vol.lib.DN_get_residency(vol.ptr) == 1
        cap, sizes, starts, tiles = vol.residency_nodes()
        # DN_create_volume's buffer: 512 * min(tiles, minChunks) / 2 voxels in 512-voxel nodes (voxel.c:181-249)
        assert cap == 512 * 8 // 2
        assert sizes.tolist() == [512] * 4 and starts.tolist() == [0, 512, 1024, 1536] and (tiles == -1).all()
        om = O.OracleMap(vol.map_size)
        om.set_lru(8)
        ocap, osz, ost, oti = om.lru_nodes()
        assert (ocap, osz.tolist(), ost.tolist(), oti.tolist()) == (cap, sizes.tolist(), starts.tolist(), tiles.tolist())
        om.close()
        assert not vol.lib.DN_set_residency(vol.ptr, 7)          # unknown mode
        vol.set_residency("keep")
        assert vol.residency_nodes()[0] == 0
    finally:
        vol.close()


def check_nodes(om, st, where):
    cap, sizes, starts, tiles = om.lru_nodes()
    order = np.argsort(starts, kind="stable")
    s, z = starts[order].astype(np.int64), sizes[order].astype(np.int64)
    # the nodes tile [0, sum of sizes) without gaps or overlaps; only whole 512-voxel nodes are added
    assert s[0] == 0 and (s[1:] == s[:-1] + z[:-1]).all(), where + ": nodes overlap or leave a gap"
    assert z.sum() <= cap and cap - z.sum() < 512, where
    assert set(np.unique(z).tolist()) <= {16, 32, 64, 128, 256, 512}, where
    owned = tiles[tiles >= 0]
    assert len(np.unique(owned)) == len(owned), where + ": a chunk owns two nodes"
    loaded = np.nonzero(st == 2)[0]
    assert np.array_equal(np.sort(owned), loaded), where + ": owners are not the loaded chunks"


def test_oracle_lru_unloads_and_reloads():
    """frames on the 16^3-chunk map with a 64-chunk buffer; three syncs without rays age every chunk,
    then the camera moves: stale chunks lose their nodes and come back when rays request them again"""
    vol, cfg = configs.build_volume("small", cpu_only=True, min_chunks=64)
    om = O.OracleMap(vol.map_size)
    om.set_lru(64)
    W, H = 160, 90
    prev = None
    evicted, reloaded, grew = set(), 0, 0
    caps = []
    try:
        for f in range(14):
            fx, fy, fz, pitch, yaw = cfg["cam"]
            if (f // 5) % 2:
                vol.camera(0.9, fy, 0.9, pitch, yaw + 180.0)
            else:
                vol.camera(fx, fy, fz, pitch, yaw)
            v, p = vol.view_proj(H / W)
            iv, icv, ip = P.draw_mats(vol, v, p)
            om.draw(vol.s, iv, icv, ip, W, H)
            for _ in range(4 if f == 5 else 1):
                om.sync(vol.s, 2, 1)
                # the product's sync clears the CPU chunks' updated flags; this volume has no device
                for i in range(vol.s.chunkCap):
                    vol.s.chunks[i].updated = False
            st, _, _, _ = om.export_tiles()
            check_nodes(om, st, "frame %d" % f)
            caps.append(om.lru_nodes()[0])
            if prev is not None:
                reloaded += sum(1 for t in np.nonzero((prev != 2) & (st == 2))[0] if int(t) in evicted)
                evicted |= set(int(t) for t in np.nonzero((prev == 2) & (st == 1))[0])
            prev = st
            om.light(vol.s, 1, 1000, 1.25 + 0.5 * f)
        grew = sum(1 for a, b in zip(caps, caps[1:]) if b > a)
        assert len(evicted) > 0 and reloaded > 0 and grew > 0, (len(evicted), reloaded, grew)
    finally:
        om.close()
        vol.close()
