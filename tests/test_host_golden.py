"""Host-side code and the CPU oracle against golden vectors produced by the reference's own host C
(tests/golden/make_golden.py runs src/DoonEngine/voxel.c, compiled unchanged from the reference tree).

Covered: voxel codec (voxel.c:1289-1316), chunk packing with surface culling and albedo linearisation
(voxel.c:1391-1461), camera matrices and their inverses (voxel.c:788-810, 845-853), the edit API's chunk
allocation state machine (voxel.c:659-714, 1121-1193), the CPU picking ray (voxel.c:1195-1272), the
.voxvol chunk codec (voxel.c:301-518) including the reference's demo volume, and the golden-angle
sphere against the lighting shader's fixed table (voxelLighting.comp:23).  No GPU needed.
"""
import ctypes
import os

import numpy as np
import pytest

import doonengine_gb300 as dn
from doonengine_gb300 import _lib as L
from oracle import oracle as O

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "host_goldens.npz"))


@pytest.fixture(scope="module")
def lib():
    return dn.load()


@pytest.fixture(scope="module")
def olib():
    return O.load()


def chunk_from_bytes(b):
    c = L.DNchunk()
    a = np.ascontiguousarray(b, np.uint8)   # kept alive while memmove reads it
    ctypes.memmove(ctypes.byref(c), a.ctypes.data, ctypes.sizeof(c))
    return c


def chunk_fields(b):
    """pos, numVoxels, normal words, albedo words (albedo only meaningful where the voxel is not empty)."""
    b = np.ascontiguousarray(b, np.uint8)
    pos = b[0:12].view(np.int32)
    n = int(b[16:20].view(np.uint32)[0])
    v = b[24:].view(np.uint32).reshape(512, 2)
    alb = np.where((v[:, 0] >> 24) != 255, v[:, 1], 0)
    return pos, n, v[:, 0].copy(), alb


def test_voxel_codec_product(lib):
    for i in range(len(G["codec_mat"])):
        v = L.DNvoxel(int(G["codec_mat"][i]), L.DNvec3(*G["codec_normal"][i].tolist()),
                      L.DNcolor(*[int(x) for x in G["codec_albedo"][i]]))
        c = lib.DN_compress_voxel(v)
        assert [c.normal, c.albedo] == G["codec_words"][i].tolist(), i
    for i in range(len(G["decodec_words"])):
        w = G["decodec_words"][i]
        v = lib.DN_decompress_voxel(L.DNcompressedVoxel(int(w[0]), int(w[1])))
        assert v.material == G["decodec_mat"][i]
        assert np.array_equal(np.float32([v.normal.x, v.normal.y, v.normal.z]), G["decodec_normal"][i])
        assert [v.albedo.r, v.albedo.g, v.albedo.b] == G["decodec_albedo"][i].tolist()


def test_voxel_codec_oracle(olib):
    for i in range(len(G["codec_mat"])):
        n = np.ascontiguousarray(G["codec_normal"][i], np.float32)
        a = np.ascontiguousarray(G["codec_albedo"][i], np.uint8)
        out = np.zeros(2, np.uint32)
        olib.dno_compress_voxel(int(G["codec_mat"][i]), n.ctypes.data, a.ctypes.data, out.ctypes.data)
        assert out.tolist() == G["codec_words"][i].tolist(), i
    for i in range(len(G["decodec_words"])):
        w = G["decodec_words"][i]
        m = ctypes.c_uint8()
        n = np.zeros(3, np.float32)
        a = np.zeros(3, np.uint8)
        olib.dno_decompress_voxel(int(w[0]) | (int(w[1]) << 32), ctypes.addressof(m), n.ctypes.data, a.ctypes.data)
        assert m.value == G["decodec_mat"][i] and np.array_equal(n, G["decodec_normal"][i])
        assert a.tolist() == G["decodec_albedo"][i].tolist()


def _materials_into(vol, table):
    a = np.ascontiguousarray(table, np.uint32)   # kept alive while memmove reads it
    ctypes.memmove(vol.s.materials, a.ctypes.data, 256 * 32)


def test_chunk_packing_product(lib):
    vol = dn.Volume((2, 2, 2), 4, cpu_only=True)
    _materials_into(vol, G["pack_materials"])
    for k in range(len(G["pack_chunks"])):
        ch = chunk_from_bytes(G["pack_chunks"][k])
        mask = np.zeros(16, np.uint32)
        part = np.zeros(3, np.uint32)
        words = np.zeros(1024, np.uint32)
        n = lib.dn_pack_chunk(vol.ptr, ctypes.byref(ch), mask.ctypes.data, part.ctypes.data, words.ctypes.data)
        assert n == G["pack_nvox"][k], k
        assert np.array_equal(mask, G["pack_mask"][k]), k
        if n:
            assert np.array_equal(part, G["pack_partial"][k]), k
        assert np.array_equal(words[: 2 * n], G["pack_vox"][k].reshape(-1)[: 2 * n]), k
    vol.close()


def test_chunk_packing_oracle(olib):
    class Packed(ctypes.Structure):
        _fields_ = [("mask", ctypes.c_uint32 * 16), ("partial", ctypes.c_uint32 * 3), ("nvox", ctypes.c_uint32),
                    ("vox", ctypes.c_uint32 * 1024)]
    mt = np.ascontiguousarray(G["pack_materials"], np.uint32)
    for k in range(len(G["pack_chunks"])):
        ch = np.ascontiguousarray(G["pack_chunks"][k], np.uint8)
        p = Packed()
        olib.dno_pack_chunk(ch.ctypes.data, mt.ctypes.data, ctypes.addressof(p))
        n = p.nvox
        assert n == G["pack_nvox"][k], k
        assert list(p.mask) == G["pack_mask"][k].tolist(), k
        if n:
            assert list(p.partial) == G["pack_partial"][k].tolist(), k
        assert list(p.vox)[: 2 * n] == G["pack_vox"][k].reshape(-1)[: 2 * n].tolist(), k


def test_surface_count_sizes_like_packing(lib):
    """The bit-board count that sizes a chunk's pool range before the device packs it (dn_count_surface)
    equals the reference's packed voxel count on every golden chunk, and the host packing's count on random
    chunks: opaque, see-through and empty materials, full, hollow and single-voxel chunks, every face."""
    vol = dn.Volume((2, 2, 2), 4, cpu_only=True)
    _materials_into(vol, G["pack_materials"])
    for k in range(len(G["pack_chunks"])):
        ch = chunk_from_bytes(G["pack_chunks"][k])
        assert lib.dn_count_surface(vol.ptr, ctypes.byref(ch)) == G["pack_nvox"][k], k
    rng = np.random.default_rng(7)
    mats = np.zeros((256, 8), np.uint32)
    opac = np.ones(256, np.float32)
    opac[rng.choice(255, 40, replace=False)] = rng.uniform(0.0, 0.999, 40).astype(np.float32)
    mats[:, 3] = opac.view(np.uint32)
    _materials_into(vol, mats)
    words = np.zeros(1024, np.uint32)
    mask = np.zeros(16, np.uint32)
    part = np.zeros(3, np.uint32)
    for k in range(400):
        ch = L.DNchunk()
        m = rng.integers(0, 255, 512).astype(np.uint32)
        kind = k % 5
        if kind == 0:
            m[rng.random(512) < rng.random()] = 255            # random density
        elif kind == 1:
            pass                                               # full (only the faces show, plus see-through)
        elif kind == 2:
            m[:] = 255
            m[rng.integers(0, 512)] = rng.integers(0, 255)     # one voxel
        elif kind == 3:
            g = np.indices((8, 8, 8)).reshape(3, -1)           # [x][y][z] order: a hollow shell
            m[((g > 0) & (g < 7)).all(0)] = 255
        else:
            m[:] = 255                                         # empty
        raw = np.zeros((512, 2), np.uint32)
        raw[:, 0] = (m << 24) | rng.integers(0, 1 << 24, 512).astype(np.uint32)
        raw[:, 1] = rng.integers(0, 1 << 32, 512, dtype=np.uint64).astype(np.uint32)
        ctypes.memmove(ctypes.addressof(ch.voxels), raw.ctypes.data, 4096)
        n = lib.dn_pack_chunk(vol.ptr, ctypes.byref(ch), mask.ctypes.data, part.ctypes.data, words.ctypes.data)
        assert lib.dn_count_surface(vol.ptr, ctypes.byref(ch)) == n, (k, kind)
    vol.close()


def _mat_np(m):
    return np.array([[m.m[c][r] for r in range(4)] for c in range(4)], np.float32).reshape(-1)


def test_camera_matrices(lib):
    """Restated camera maths vs the reference's compiled quickmath path: view, projection and the three
    inverses bit for bit (the inverse follows the reference's operation order)."""
    vol = dn.Volume((2, 2, 2), 4, cpu_only=True)
    for i in range(len(G["cam_params"])):
        c = G["cam_params"][i]
        vol.s.camPos.x, vol.s.camPos.y, vol.s.camPos.z = (float(x) for x in c[0:3])
        vol.s.camOrient.x, vol.s.camOrient.y, vol.s.camOrient.z = (float(x) for x in c[3:6])
        vol.s.camFOV = float(c[6])
        v, p = L.DNmat4(), L.DNmat4()
        lib.DN_set_view_projection_matrices(vol.ptr, float(c[7]), float(c[8]), 100.0, ctypes.byref(v), ctypes.byref(p))
        iv, icv, ip = L.DNmat4(), L.DNmat4(), L.DNmat4()
        lib.DN_draw_matrices(v, p, ctypes.byref(iv), ctypes.byref(icv), ctypes.byref(ip))
        got = [_mat_np(m) for m in (v, p, iv, icv, ip)]
        for j, (a, b) in enumerate(zip(got, G["cam_mats"][i])):
            a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (i, j, np.abs(a - b).max())
        d = lib.DN_cam_dir(L.DNvec3(*c[3:6].tolist()))
        assert np.abs(np.float32(d.tolist()) - G["cam_dirs"][i]).max() <= 2e-6
    vol.close()
    for i in range(len(G["norm_in"])):
        r = lib.DN_vec3_normalize(L.DNvec3(*G["norm_in"][i].tolist()))
        assert np.abs(np.float32(r.tolist()) - G["norm_out"][i]).max() <= 2e-7


def _replay_edits(lib, vol, ops):
    for op in ops:
        mp = L.DNivec3(*[int(x) for x in op[1:4]])
        cp = L.DNivec3(*[int(x) for x in op[4:7]])
        if op[0] == 0:
            n = np.array(op[8:11], np.int32).view(np.float32)
            v = L.DNvoxel(int(op[7]), L.DNvec3(*n.tolist()), L.DNcolor(*[int(x) for x in op[11:14]]))
            lib.DN_set_voxel(vol.ptr, mp, cp, v)
        else:
            lib.DN_remove_voxel(vol.ptr, mp, cp)


def test_edit_api_state_machine(lib):
    """Chunk allocation, growth, removal and voxel counts follow the reference exactly."""
    size = tuple(int(x) for x in G["edit_size"])
    vol = dn.Volume(size, 4, cpu_only=True)
    _replay_edits(lib, vol, G["edit_ops"])
    cap, nxt = (int(x) for x in G["edit_info"])
    assert vol.s.chunkCap == cap and vol.s.nextChunk == nxt
    tiles = size[0] * size[1] * size[2]
    gmap = G["edit_map"].reshape(tiles, 8)
    for t in range(tiles):
        flag = int(gmap[t, 0])
        assert vol.s.map[t].flag == flag, t
        if flag:
            assert vol.s.map[t].chunkIndex == int(gmap[t, 4:8].view(np.uint32)[0]), t
    gch = G["edit_chunks"].reshape(cap, 4120)
    raw = np.ctypeslib.as_array(ctypes.cast(vol.s.chunks, ctypes.POINTER(ctypes.c_uint8)), shape=(cap * 4120,))
    mine = raw.reshape(cap, 4120)
    for i in range(cap):
        gp, gn, gnw, galb = chunk_fields(gch[i])
        mp_, mn, mnw, malb = chunk_fields(mine[i])
        assert np.array_equal(gp, mp_), i
        if gp[0] >= 0:
            assert gn == mn and np.array_equal(gnw, mnw) and np.array_equal(galb, malb), i
    vol.close()


def test_picking_ray(lib):
    size = tuple(int(x) for x in G["edit_size"])
    vol = dn.Volume(size, 4, cpu_only=True)
    _replay_edits(lib, vol, G["edit_ops"])
    for i in range(len(G["pick_rays"])):
        r = G["pick_rays"][i]
        hp, hn = L.DNivec3(), L.DNivec3()
        hv = L.DNvoxel()
        hit = lib.DN_step_map(vol.ptr, L.DNvec3(*r[3:6].tolist()), L.DNvec3(*r[0:3].tolist()), 200,
                              ctypes.byref(hp), ctypes.byref(hv), ctypes.byref(hn))
        g = G["pick_out"][i]
        assert int(hit) == g[0], i
        assert [hn.x, hn.y, hn.z] == g[4:7].tolist(), i
        if hit:
            assert [hp.x, hp.y, hp.z] == g[1:4].tolist(), i
            c = lib.DN_compress_voxel(hv)
            assert [c.normal, c.albedo] == [int(g[7]), int(g[8])], i
    vol.close()


def _codec_case(lib, vol, chunks, lens, blob):
    off = 0
    for k in range(len(chunks)):
        want = blob[off: off + int(lens[k])]
        off += int(lens[k])
        ch = chunk_from_bytes(chunks[k])
        mem = (ctypes.c_uint8 * (2 * 4120))()
        n = lib.DN_compress_chunk(vol.ptr, ctypes.byref(ch), mem)
        assert bytes(mem[:n]) == want.tobytes(), k
        out = L.DNchunk()
        src = np.ascontiguousarray(want, np.uint8)
        assert lib.DN_decompress_chunk(vol.ptr, src.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(src),
                                       ctypes.byref(out)) == 0
        got = np.frombuffer(ctypes.string_at(ctypes.addressof(out), 4120), np.uint8)
        gp, gn, gnw, galb = chunk_fields(chunks[k])
        mp_, mn, mnw, malb = chunk_fields(got)
        assert np.array_equal(gp, mp_), k
        if gp[0] >= 0:
            assert gn == mn and np.array_equal(gnw, mnw) and np.array_equal(galb, malb), k


def test_voxvol_chunk_codec(lib):
    vol = dn.Volume(tuple(int(x) for x in G["edit_size"]), 4, cpu_only=True)
    _codec_case(lib, vol, G["vv_chunks"], G["vv_lens"], G["vv_bytes"])
    vol.close()


def test_demo_volume_chunks(lib):
    """The reference's demo volume: its decoded chunks re-encode to the reference's bytes and back."""
    vol = dn.Volume(tuple(int(x) for x in G["demo_size"]), 4, cpu_only=True)
    _codec_case(lib, vol, G["demo_chunks"], G["demo_lens"], G["demo_bytes"])
    vol.close()


def test_decoder_rejects_malformed_input(lib):
    vol = dn.Volume((4, 4, 4), 4, cpu_only=True)
    out = L.DNchunk()
    ok = np.zeros(12 + 2, np.uint8)          # pos (0,0,0), empty palettes, then nothing
    bad_run = np.concatenate([ok, np.array([255, 0], np.uint8)])          # zero-length run
    truncated = np.concatenate([ok, np.array([1, 10], np.uint8)])         # run without voxel data
    for b in (bad_run, truncated, ok[:5]):
        b = np.ascontiguousarray(b)
        assert lib.DN_decompress_chunk(vol.ptr, b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(b),
                                       ctypes.byref(out)) == -1
    vol.close()


def test_sphere_points_match_shader_table(olib):
    pts = np.zeros((15, 3), np.float32)
    olib.dno_sphere_points(15, pts.ctypes.data)
    assert np.abs(pts - G["sphere15"]).max() < 2e-6


def test_deterministic_sine(olib):
    xs = np.linspace(-3000.0, 3000.0, 20011, dtype=np.float32)
    got = np.array([olib.dno_sin(float(x)) for x in xs[::7]], np.float64)
    want = np.sin(xs[::7].astype(np.float64))
    assert np.abs(got - want).max() < 2e-4     # the reduction keeps absolute error small over this range
