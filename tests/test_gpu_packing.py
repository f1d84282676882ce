"""Packing of staged chunks on the device (dn_cuda_sync_chunks: surface cull, occupancy mask, partial counts,
compaction, albedo linearisation and material set from the CPU map's voxels) against the packing of the
reference's voxel.c:1397-1461.

* Reference goldens: the 72 chunks the reference's own voxel.c packed (tests/golden/host_goldens.npz, made by
  tests/golden/make_golden.py) are written into a map voxel by voxel and synced once; every tile's device
  record and voxel words equal the reference's output.
* Host packing: a terrain map with see-through materials, synced and then edited over several syncs (chunks
  re-rolled, cleared, filled solid); after each sync every chunk's device record equals dn_pack_chunk of its
  CPU chunk (the host packing that the goldens pin), and its material set is the set of its words'
  materials.
* Parts: the same maps staged in 64 KiB parts (a few chunks per upload) give the same records.
* DN_HOST_PACKING=1 (packing on the host, dn_cuda_sync) gives the same records, lighting and draws.

Bar: bit-exact.
"""
import ctypes
import os

import numpy as np
import pytest

import doonengine_gb300 as dn
from doonengine_gb300 import configs

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "host_goldens.npz"))


def tile_pos(vol, t):
    sx, sy, _ = vol.map_size
    return (t % sx, (t // sx) % sy, t // (sx * sy))


def host_pack(lib, vol, ch):
    mask = np.zeros(16, np.uint32)
    part = np.zeros(3, np.uint32)
    words = np.zeros(1024, np.uint32)
    n = lib.dn_pack_chunk(vol.ptr, ctypes.byref(ch), mask.ctypes.data, part.ctypes.data, words.ctypes.data)
    return n, mask, part, words[: 2 * n].reshape(n, 2)


def material_set(words):
    s = np.zeros(8, np.uint32)
    for m in np.unique(words[:, 0] >> 24):
        s[m >> 5] |= np.uint32(1 << (int(m) & 31))
    return s


def check_against_host(lib, vol, where):
    """every chunk of the CPU map has a device record equal to the host packing of that chunk"""
    checked = 0
    for t in range(vol.num_tiles):
        ch = vol.cpu_chunk(t)
        if ch is None:
            continue
        rec = vol.export_chunk(t)
        assert rec is not None, "%s: tile %d has no record" % (where, t)
        n, mask, part, words = host_pack(lib, vol, ch)
        assert rec["nvox"] == n, "%s: tile %d count %d, host %d" % (where, t, rec["nvox"], n)
        assert np.array_equal(rec["mask"], mask), "%s: tile %d mask" % (where, t)
        assert np.array_equal(rec["partial"], part), "%s: tile %d partial counts" % (where, t)
        assert np.array_equal(rec["words"], words), "%s: tile %d voxel words" % (where, t)
        assert np.array_equal(rec["matSet"], material_set(words)), "%s: tile %d material set" % (where, t)
        assert tuple(rec["pos"]) == (ch.pos.x, ch.pos.y, ch.pos.z), "%s: tile %d position" % (where, t)
        checked += 1
    return checked


def records(vol):
    out = {}
    for t in range(vol.num_tiles):
        r = vol.export_chunk(t)
        if r is not None:
            out[t] = r
    return out


def same_records(a, b, where):
    assert sorted(a) == sorted(b), where + ": different tiles have records"
    for t in a:
        for k in a[t]:
            assert np.array_equal(np.asarray(a[t][k]), np.asarray(b[t][k])), "%s: tile %d %s" % (where, t, k)


def test_device_packing_matches_reference_goldens():
    lib = dn.load()
    dn.init()
    vol = dn.Volume((6, 3, 4), 72)
    mt = np.ascontiguousarray(G["pack_materials"], np.uint32)   # kept alive: memmove reads it below
    ctypes.memmove(vol.s.materials, mt.ctypes.data, 256 * 32)
    try:
        for k in range(len(G["pack_chunks"])):
            raw = np.ascontiguousarray(G["pack_chunks"][k], np.uint8)[24:].view(np.uint32).reshape(8, 8, 8, 2)
            mp = tile_pos(vol, k)
            for x, y, z in zip(*np.nonzero((raw[:, :, :, 0] >> 24) != 255)):
                vol.set_compressed(mp, (int(x), int(y), int(z)), int(raw[x, y, z, 0]), int(raw[x, y, z, 1]))
        vol.sync(dn.DN_READ_WRITE)
        assert vol.finish(), lib.dn_cuda_last_error().decode()
        seen = 0
        for k in range(len(G["pack_chunks"])):
            rec = vol.export_chunk(k)
            if vol.cpu_chunk(k) is None:
                assert G["pack_nvox"][k] == 0 and rec is None, k
                continue
            n = int(G["pack_nvox"][k])
            assert rec["nvox"] == n, k
            assert np.array_equal(rec["mask"], G["pack_mask"][k]), k
            if n:
                assert np.array_equal(rec["partial"], G["pack_partial"][k]), k
            assert np.array_equal(rec["words"].reshape(-1), G["pack_vox"][k].reshape(-1)[: 2 * n]), k
            seen += 1
        assert seen >= 60
    finally:
        vol.close()


def edit_sequence(lib, vol, check):
    """syncs with edits between them; 'check(where)' after each sync"""
    vol.set_material(3, opacity=0.5)
    vol.set_material(7, opacity=0.25)
    vol.sync(dn.DN_READ_WRITE)
    check("initial load")
    rng = np.random.default_rng(5)
    sx, sy, sz = vol.map_size
    for step in range(3):
        pos = np.ascontiguousarray(np.stack([rng.integers(0, s, 24) for s in (sx, sy, sz)], 1), np.int32)
        lib.dn_scene_reroll(vol.ptr, pos.ctypes.data, len(pos), 100 + step, 16)
        # one chunk filled solid (only its faces stay), one emptied but for a voxel
        fx, fy, fz = (int(v) for v in rng.integers(0, (sx, sy, sz)))
        for x in range(8):
            for y in range(8):
                for z in range(8):
                    vol.set_compressed((fx, fy, fz), (x, y, z), (5 << 24) | 0x7F7F7F, 0x80808000)
        ex, ey, ez = (int(v) for v in rng.integers(0, (sx, sy, sz)))
        for x in range(8):
            for y in range(8):
                for z in range(8):
                    if (x, y, z) != (3, 4, 5):
                        vol.remove_voxel((ex, ey, ez), (x, y, z))
        vol.set_compressed((ex, ey, ez), (3, 4, 5), (7 << 24) | 0x7F7F7F, 0x40404000)
        vol.sync(dn.DN_READ_WRITE)
        check("edit step %d" % step)


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_device_packing_matches_host_packing(name):
    lib = dn.load()
    dn.init()
    vol, _ = configs.build_volume(name)
    try:
        def check(where):
            assert vol.finish(), lib.dn_cuda_last_error().decode()
            assert check_against_host(lib, vol, "%s %s" % (name, where)) > 0
        edit_sequence(lib, vol, check)
    finally:
        vol.close()


def run_frames(vol, frames=3):
    """draw, sync and lighting frames; returns the last frame's image and the lighting"""
    img = dn.Image(320, 180, on_device=True)
    try:
        out = None
        for f in range(frames):
            v, p = vol.view_proj(180 / 320)
            vol.draw(img, v, p)
            vol.sync(dn.DN_READ_WRITE)
            vol.update_lighting(1, 1000, 1.25 + 0.5 * f)
            assert vol.finish(), dn.load().dn_cuda_last_error().decode()
            out = img.numpy()
        return out, vol.export_lighting()
    finally:
        img.close()


def test_staging_in_parts_and_host_packing_agree():
    lib = dn.load()
    dn.init()
    results = {}
    for mode in ("device", "parts", "host"):
        prev = lib.dn_cuda_stage_part_limit(64 * 1024 if mode == "parts" else 0)
        if mode == "host":
            os.environ["DN_HOST_PACKING"] = "1"
        try:
            vol, _ = configs.build_volume("small")
        finally:
            os.environ.pop("DN_HOST_PACKING", None)
        try:
            states = []

            def check(where):
                assert vol.finish(), lib.dn_cuda_last_error().decode()
                states.append(records(vol))
            edit_sequence(lib, vol, check)
            results[mode] = (states, run_frames(vol))
        finally:
            vol.close()
            lib.dn_cuda_stage_part_limit(prev)
    base_states, (base_img, base_light) = results["device"]
    for mode in ("parts", "host"):
        states, (img, light) = results[mode]
        assert len(states) == len(base_states)
        for i, (a, b) in enumerate(zip(base_states, states)):
            same_records(a, b, "%s sync %d" % (mode, i))
        for what, a, b in zip(("colour", "hit index", "face"), img, base_img):
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), "%s: draw %s" % (mode, what)
        for what, a, b in zip(("index", "diffuse", "specular"), light, base_light):
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), "%s: lighting %s" % (mode, what)
