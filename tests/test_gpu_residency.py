"""DN_RESIDENCY_LRU on the device against the CPU oracle, frame by frame: tile states, lastUsed, visible
flags, sample counts, request lists, lighting, draws and the node buffer itself.

The frames make the buffer both grow and unload: three syncs without rays age every chunk, then the
camera moves and the chunks it requests take the stale chunks' nodes; the stale chunks are requested and
loaded again later.  Bar: bit-identical tile state and nodes, lighting within 1e-4 relative.
"""
import numpy as np
import pytest

import parity_util as P

pytestmark = pytest.mark.gpu


def nodes_equal(vol, om, where):
    g = vol.residency_nodes()
    o = om.lru_nodes()
    assert g[0] == o[0], "%s: buffer size %d vs oracle %d" % (where, g[0], o[0])
    for a, b, what in zip(g[1:], o[1:], ("sizes", "starts", "owners")):
        assert np.array_equal(a, b), "%s: node %s differ" % (where, what)


def test_lru_residency_matches_oracle(gpu_ready):
    pair = P.Pair("small", res=(320, 180), min_chunks=64)
    try:
        pair.vol.set_residency("lru")
        pair.om.set_lru(64)
        cfg = pair.cfg
        prev = None
        evicted, reloaded = set(), 0
        for f in range(14):
            fx, fy, fz, pitch, yaw = cfg["cam"]
            if (f // 5) % 2:
                pair.vol.camera(0.9, fy, 0.9, pitch, yaw + 180.0)
            else:
                pair.vol.camera(fx, fy, fz, pitch, yaw)
            pair.draw()
            if f == 5:
                for _ in range(3):
                    pair.sync()
            if f == 9:
                pair.sync(op=0)      # DN_READ: lastUsed advances, nothing streams
            pair.sync()
            nodes_equal(pair.vol, pair.om, "frame %d" % f)
            st = pair.vol.export_tiles()[0]
            if prev is not None:
                reloaded += sum(1 for t in np.nonzero((prev != 2) & (st == 2))[0] if int(t) in evicted)
                evicted |= set(int(t) for t in np.nonzero((prev == 2) & (st == 1))[0])
            prev = st
            pair.light()
        assert len(evicted) > 0 and reloaded > 0, (len(evicted), reloaded)
    finally:
        pair.close()


def test_lru_volume_stays_out_of_batches(gpu_ready):
    import doonengine_gb300 as dn
    from doonengine_gb300 import configs
    dn.init()
    vol, _ = configs.build_volume("tiny")
    b = dn.Batch()
    try:
        vol.set_residency("lru")
        assert not b.lib.DN_batch_add(b.ptr, vol.ptr)
        vol.sync(dn.DN_READ_WRITE, 1)
        assert not vol.lib.DN_set_residency(vol.ptr, 0)       # only before the first sync
    finally:
        b.close()
        vol.close()
