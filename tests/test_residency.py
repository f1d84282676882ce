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


class _Node(ctypes.Structure):
    _fields_ = [("size", ctypes.c_uint32), ("start", ctypes.c_uint64), ("tile", ctypes.c_int64)]


class _Nodes(ctypes.Structure):
    _fields_ = [("v", ctypes.POINTER(_Node)), ("n", ctypes.c_size_t), ("cap", ctypes.c_size_t),
                ("voxelCap", ctypes.c_uint64)]


def test_node_models_agree_on_random_sequences():
    """the product's node model (csrc/dn_residency.c, inside libdoonengine.so) and the oracle's restatement,
    driven by the same random sequences of streams, unloads, sort passes and growth"""
    import doonengine_gb300 as dn
    lib = dn.load()
    lib.dn_nodes_init.argtypes = [ctypes.POINTER(_Nodes), ctypes.c_uint64]
    lib.dn_nodes_stream.argtypes = [ctypes.POINTER(_Nodes), ctypes.c_int64, ctypes.c_uint32,
                                    ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int64)]
    lib.dn_nodes_unload.argtypes = [ctypes.POINTER(_Nodes), ctypes.c_int64]
    lib.dn_nodes_sort.argtypes = [ctypes.POINTER(_Nodes), ctypes.c_int]
    lib.dn_nodes_grow.argtypes = [ctypes.POINTER(_Nodes), ctypes.c_uint64]
    lib.dn_nodes_free.argtypes = [ctypes.POINTER(_Nodes)]
    ntiles = 96
    seen = {"evict": 0, "fail": 0, "split": 0, "merge": 0}
    for seed in range(12):
        rng = np.random.default_rng(seed)
        chunks = int(rng.integers(2, 24))
        b = _Nodes()
        assert lib.dn_nodes_init(ctypes.byref(b), chunks)
        om = O.OracleMap((4, 4, 6))
        om.set_lru(chunks)
        owned = set()
        stale_bias = rng.uniform(0.2, 0.9)
        try:
            for step in range(400):
                lu = np.where(rng.random(ntiles) < stale_bias, rng.integers(2, 9, ntiles),
                              rng.integers(0, 2, ntiles)).astype(np.uint32)
                om.lib.dno_set_last_used(om.ptr, lu.ctypes.data)
                op = rng.random()
                if op < 0.6 and len(owned) < ntiles:
                    free_tiles = [t for t in range(ntiles) if t not in owned]
                    t = int(rng.choice(free_tiles))
                    nvox = int(rng.choice([0, 1, 16, 17, 33, 100, 200, 256, 300, 511, 512]))
                    gv, ov = ctypes.c_int64(-2), ctypes.c_int64(-2)
                    gr = lib.dn_nodes_stream(ctypes.byref(b), t, nvox,
                                             lu.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(gv))
                    orr = om.lib.dno_lru_stream(om.ptr, t, nvox, ctypes.byref(ov))
                    assert gr == orr and (gr == 0 or gv.value == ov.value), (seed, step, gr, orr, gv.value, ov.value)
                    if gr:
                        seen["evict"] += gv.value >= 0
                        owned.add(t)
                        owned.discard(gv.value)
                    else:
                        seen["fail"] += 1
                    if not gr and rng.random() < 0.7:
                        cap = b.voxelCap * 2 if b.voxelCap else 512
                        lib.dn_nodes_grow(ctypes.byref(b), cap)
                        om.lib.dno_lru_grow(om.ptr, cap)
                elif op < 0.8 and owned:
                    t = int(rng.choice(sorted(owned)))
                    lib.dn_nodes_unload(ctypes.byref(b), t)
                    om.lib.dno_lru_unload(om.ptr, t)
                    owned.discard(t)
                else:
                    mc = int(rng.integers(0, 12))
                    n0 = b.n
                    lib.dn_nodes_sort(ctypes.byref(b), mc)
                    seen["merge"] += b.n < n0
                    om.lib.dno_lru_sort(om.ptr, mc)
                cap, sizes, starts, tiles = om.lru_nodes()
                seen["split"] += int((sizes < 512).any())
                assert b.voxelCap == cap and b.n == len(sizes), (seed, step)
                got = [(b.v[i].size, b.v[i].start, b.v[i].tile) for i in range(b.n)]
                assert got == list(zip(sizes.tolist(), starts.tolist(), tiles.tolist())), (seed, step)
                assert set(tiles[tiles >= 0].tolist()) == owned, (seed, step)
        finally:
            lib.dn_nodes_free(ctypes.byref(b))
            om.close()
    # every decision of the model occurred
    assert all(v > 0 for v in seen.values()), seen
