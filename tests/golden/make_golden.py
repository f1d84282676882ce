"""Generates tests/golden/host_goldens.npz from the reference's own host C.

The reference's src/DoonEngine/voxel.c is compiled unchanged from the reference tree into
oracle/_ref/libdnref.so (oracle/ref/Makefile; no GL code is linked) and driven here through ctypes on
seeded inputs.  The outputs are the golden vectors the CPU tests check the product's host code and the
CPU oracle against.  x86-64 only (the reference's vendored math header forces SSE).

    python tests/golden/make_golden.py [/path/to/reference]
"""
import ctypes
import os
import sys
from ctypes import POINTER, c_float, c_int, c_int32, c_uint8, c_uint32, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

CHUNK_BYTES = 4120


def load_ref(ref_root):
    path = O.build_reference(ref_root)
    if not path:
        raise SystemExit("the reference host C builds only on x86-64 with the reference tree present")
    lib = ctypes.CDLL(path)
    sigs = {
        "ref_sizeof_chunk": (c_uint32, []),
        "ref_compress_voxel": (None, [c_uint8, c_void_p, c_void_p, c_void_p]),
        "ref_decompress_voxel": (None, [c_void_p, c_void_p, c_void_p, c_void_p]),
        "ref_chunk_to_gpu": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
        "ref_view_projection": (None, [c_void_p, c_void_p, c_float, c_float, c_float, c_float] + [c_void_p] * 5),
        "ref_cam_dir": (None, [c_void_p, c_void_p]),
        "ref_vec3_normalize": (None, [c_void_p, c_void_p]),
        "ref_volume_new": (c_void_p, [c_uint32, c_uint32, c_uint32, c_uint32]),
        "ref_volume_free": (None, [c_void_p]),
        "ref_volume_info": (None, [c_void_p, c_void_p]),
        "ref_volume_map": (c_void_p, [c_void_p]),
        "ref_volume_chunks": (c_void_p, [c_void_p]),
        "ref_set_voxel": (None, [c_void_p, c_void_p, c_void_p, c_uint8, c_void_p, c_void_p]),
        "ref_remove_voxel": (None, [c_void_p, c_void_p, c_void_p]),
        "ref_step_map": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
        "ref_compress_chunk": (c_uint32, [c_void_p, c_void_p, c_void_p]),
        "ref_decompress_chunk": (None, [c_void_p, c_void_p, c_void_p]),
    }
    for n, (r, a) in sigs.items():
        f = getattr(lib, n)
        f.restype = r
        f.argtypes = a
    assert lib.ref_sizeof_chunk() == CHUNK_BYTES
    return lib


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def make_chunk(rng, density, nmat, pos=(0, 0, 0)):
    """DNchunk bytes: pos, updated, numVoxels, numVoxelsGpu, voxels[x][y][z] (normal word, albedo word)."""
    vox = np.zeros((8, 8, 8, 2), np.uint32)
    vox[..., 0] = 0xFFFFFFFF
    fill = rng.random((8, 8, 8)) < density
    n = int(fill.sum())
    mats = rng.integers(0, nmat, n).astype(np.uint32)
    nb = rng.integers(0, 256, (n, 3)).astype(np.uint32)
    ab = rng.integers(0, 256, (n, 3)).astype(np.uint32)
    vox[fill, 0] = (mats << 24) | (nb[:, 0] << 16) | (nb[:, 1] << 8) | nb[:, 2]
    vox[fill, 1] = (ab[:, 0] << 24) | (ab[:, 1] << 16) | (ab[:, 2] << 8)
    buf = np.zeros(CHUNK_BYTES, np.uint8)
    buf[0:12] = np.array(pos, np.int32).view(np.uint8)
    buf[16:20] = np.array([n], np.uint32).view(np.uint8)
    buf[24:] = vox.reshape(-1).view(np.uint8)
    return buf


def materials_table(rng, n=256):
    m = np.zeros((n, 8), np.uint32)
    mf = m.view(np.float32)
    mf[:, 3] = np.where(rng.random(n) < 0.25, rng.uniform(0.1, 0.9, n), 1.0).astype(np.float32)   # opacity
    mf[:, 4] = 1.0
    mf[:, 5] = rng.uniform(0, 1, n).astype(np.float32)
    return m


def main():
    ref_root = O.reference_root(sys.argv[1] if len(sys.argv) > 1 else None)
    if ref_root is None:
        sys.exit("usage: %s REFERENCE_ROOT (or set DN_REFERENCE_ROOT)" % sys.argv[0])
    lib = load_ref(ref_root)
    rng = np.random.default_rng(20261203)
    out = {}

    # A. voxel codec (voxel.c:1289-1316)
    n = 600
    mats = rng.integers(0, 256, n).astype(np.uint8)
    normals = rng.uniform(-1.3, 1.3, (n, 3)).astype(np.float32)
    normals[:40] = np.array([[1, 0, -1], [-1, -1, -1], [0, 0, 0], [1, 1, 1]], np.float32)[np.arange(40) % 4]
    albedo = rng.integers(0, 256, (n, 3)).astype(np.uint8)
    words = np.zeros((n, 2), np.uint32)
    for i in range(n):
        w = (c_uint32 * 2)()
        lib.ref_compress_voxel(int(mats[i]), f32(normals[i]).ctypes.data, albedo[i].ctypes.data, w)
        words[i] = list(w)
    out["codec_mat"], out["codec_normal"], out["codec_albedo"], out["codec_words"] = mats, normals, albedo, words
    dw = rng.integers(0, 2**32, (n, 2), dtype=np.uint64).astype(np.uint32)
    dmat = np.zeros(n, np.uint8); dnorm = np.zeros((n, 3), np.float32); dalb = np.zeros((n, 3), np.uint8)
    for i in range(n):
        m = c_uint8(); nn = (c_float * 3)(); aa = (c_uint8 * 3)()
        lib.ref_decompress_voxel(np.ascontiguousarray(dw[i]).ctypes.data, ctypes.byref(m), nn, aa)
        dmat[i], dnorm[i], dalb[i] = m.value, list(nn), list(aa)
    out["decodec_words"], out["decodec_mat"], out["decodec_normal"], out["decodec_albedo"] = dw, dmat, dnorm, dalb

    # B. chunk packing: surface cull, mask, partial counts, linear albedo (voxel.c:1391-1461)
    mt = materials_table(rng)
    out["pack_materials"] = mt
    chunks, masks, partials, nvoxs, pvox = [], [], [], [], []
    for k in range(72):
        density = [0.0, 0.02, 0.1, 0.3, 0.6, 0.95, 1.0, 0.5][k % 8]
        ch = make_chunk(rng, density, [1, 3, 8, 256][k % 4])
        mask = (c_uint32 * 16)(); part = (c_uint32 * 3)(); nv = c_uint32(); vv = (c_uint32 * 1024)()
        lib.ref_chunk_to_gpu(ch.ctypes.data, mt.ctypes.data, mask, part, ctypes.byref(nv), vv)
        chunks.append(ch); masks.append(list(mask)); partials.append(list(part)); nvoxs.append(nv.value)
        pv = np.zeros((512, 2), np.uint32)
        pv.reshape(-1)[: 2 * nv.value] = np.array(vv[: 2 * nv.value], np.uint32)
        pvox.append(pv)
    out["pack_chunks"] = np.stack(chunks); out["pack_mask"] = np.array(masks, np.uint32)
    out["pack_partial"] = np.array(partials, np.uint32); out["pack_nvox"] = np.array(nvoxs, np.uint32)
    out["pack_vox"] = np.stack(pvox)

    # C. camera (voxel.c:788-810, inverses 845-853), cam dir (1283-1287), normalize (942)
    ncam = 40
    cams = np.zeros((ncam, 9), np.float32)
    cams[:, 0:3] = rng.uniform(-20, 60, (ncam, 3))
    cams[:, 3] = rng.uniform(-89, 89, ncam)
    cams[:, 4] = rng.uniform(0, 360, ncam)
    cams[:, 5] = np.where(rng.random(ncam) < 0.5, 0.0, rng.uniform(-30, 30, ncam))
    cams[:, 6] = rng.uniform(30, 120, ncam)
    cams[:, 7] = np.array([0.5625, 1.0, 1.7778, 0.75, 2.0, 0.3])[np.arange(ncam) % 6]
    cams[:, 8] = rng.uniform(0.05, 1.0, ncam)
    mats_out = np.zeros((ncam, 5, 16), np.float32)
    dirs = np.zeros((ncam, 3), np.float32)
    for i in range(ncam):
        c = cams[i]
        ms = [(c_float * 16)() for _ in range(5)]
        lib.ref_view_projection(f32(c[0:3]).ctypes.data, f32(c[3:6]).ctypes.data, float(c[6]), float(c[7]),
                                float(c[8]), 100.0, *ms)
        for j in range(5):
            mats_out[i, j] = list(ms[j])
        d = (c_float * 3)()
        lib.ref_cam_dir(f32(c[3:6]).ctypes.data, d)
        dirs[i] = list(d)
    out["cam_params"], out["cam_mats"], out["cam_dirs"] = cams, mats_out, dirs
    vecs = rng.uniform(-5, 5, (100, 3)).astype(np.float32)
    nv = np.zeros((100, 3), np.float32)
    for i in range(100):
        d = (c_float * 3)()
        lib.ref_vec3_normalize(f32(vecs[i]).ctypes.data, d)
        nv[i] = list(d)
    out["norm_in"], out["norm_out"] = vecs, nv

    # D. edit API state machine (voxel.c:659-714, 1121-1193) and the CPU picking ray (1195-1272)
    size = (5, 4, 3)
    vol = lib.ref_volume_new(*size, 4)
    ops = []
    for i in range(4000):
        mp = rng.integers(0, size).astype(np.int32)
        cp = rng.integers(0, 8, 3).astype(np.int32)
        kind = rng.random()
        if kind < 0.55:
            mat = int(rng.integers(0, 6)) if rng.random() < 0.9 else 255
            nrm = rng.uniform(-1, 1, 3).astype(np.float32)
            alb = rng.integers(0, 256, 3).astype(np.uint8)
            lib.ref_set_voxel(vol, mp.ctypes.data, cp.ctypes.data, mat, nrm.ctypes.data, alb.ctypes.data)
            ops.append([0, *mp, *cp, mat, *nrm.view(np.int32), *alb.astype(np.int32)])
        elif kind < 0.8:
            # remove only where a chunk exists (the reference does not check, voxel.h:313-318)
            mapb = np.ctypeslib.as_array(ctypes.cast(lib.ref_volume_map(vol), POINTER(c_uint8)), shape=(60 * 8,))
            t = mp[0] + size[0] * (mp[1] + size[1] * mp[2])
            if mapb[t * 8] == 0:
                continue
            lib.ref_remove_voxel(vol, mp.ctypes.data, cp.ctypes.data)
            ops.append([1, *mp, *cp, 0, 0, 0, 0, 0, 0, 0])
        else:
            # a dense block, so that chunks fill and empty out again
            for dz in range(2):
                for dy in range(2):
                    for dx in range(2):
                        c2 = np.minimum(cp + np.array([dx, dy, dz], np.int32), 7).astype(np.int32)
                        nrm = np.array([0, 1, 0], np.float32)
                        alb = np.array([9, 9, 9], np.uint8)
                        lib.ref_set_voxel(vol, mp.ctypes.data, c2.ctypes.data, 3, nrm.ctypes.data, alb.ctypes.data)
                        ops.append([0, *mp, *c2, 3, *nrm.view(np.int32), 9, 9, 9])
    info = (c_uint64 * 3)()
    lib.ref_volume_info(vol, info)
    cap = int(info[0])
    tiles = size[0] * size[1] * size[2]
    mapb = np.ctypeslib.as_array(ctypes.cast(lib.ref_volume_map(vol), POINTER(c_uint8)), shape=(tiles * 8,)).copy()
    chb = np.ctypeslib.as_array(ctypes.cast(lib.ref_volume_chunks(vol), POINTER(c_uint8)), shape=(cap * CHUNK_BYTES,)).copy()
    out["edit_size"] = np.array(size, np.int32)
    out["edit_ops"] = np.array(ops, np.int32)
    out["edit_info"] = np.array([cap, int(info[1])], np.uint64)
    out["edit_map"] = mapb
    out["edit_chunks"] = chb
    # picking rays through the edited volume
    nray = 400
    rays = np.zeros((nray, 6), np.float32)
    rays[:, 0:3] = rng.uniform(-1, np.array(size) + 1, (nray, 3))
    d = rng.normal(size=(nray, 3)).astype(np.float32)
    d[:60] = np.array([[1, 0, 0], [0, -1, 0], [0, 0, 1], [-1, 0, 0], [1, 1, 0], [0.5, -1, 0.25]], np.float32)[np.arange(60) % 6]
    rays[:, 3:6] = d
    pick = np.zeros((nray, 9), np.int64)
    for i in range(nray):
        hp = (c_int32 * 3)(); hv = (c_uint32 * 2)(); hn = (c_int32 * 3)()
        r = lib.ref_step_map(vol, f32(rays[i, 3:6]).ctypes.data, f32(rays[i, 0:3]).ctypes.data, 200, hp, hv, hn)
        pick[i] = [r, *hp, *hn, *hv] if r else [0, 0, 0, 0, *hn, 0, 0]
    out["pick_rays"], out["pick_out"] = rays, pick

    # E. .voxvol chunk codec (voxel.c:301-518): random chunks through the reference encoder
    enc, encb = [], []
    for k in range(48):
        inb = k % 6 != 5
        pos = tuple(int(x) for x in rng.integers(0, size)) if inb else (-1, -1, -1)
        ch = make_chunk(rng, [0.01, 0.2, 0.5, 0.97, 1.0, 0.05][k % 6], [1, 2, 6][k % 3], pos)
        if k % 4 == 0:
            # few distinct normals / albedos: the palette path
            v = ch[24:].view(np.uint32).reshape(8, 8, 8, 2)
            full = v[..., 0] != 0xFFFFFFFF
            v[full, 0] = (v[full, 0] & 0xFF000000) | 0x00804080
            v[full, 1] = 0x20406000
        mem = (c_uint8 * (2 * CHUNK_BYTES))()
        nbytes = lib.ref_compress_chunk(vol, ch.ctypes.data, mem)
        enc.append(ch)
        encb.append(np.frombuffer(bytes(mem)[:nbytes], np.uint8))
    out["vv_chunks"] = np.stack(enc)
    out["vv_lens"] = np.array([len(b) for b in encb], np.uint32)
    out["vv_bytes"] = np.concatenate(encb)
    lib.ref_volume_free(vol)

    # F. the reference's demo volume, decoded by the reference decoder and re-encoded by its encoder
    demo = os.path.join(ref_root, "assets", "volumes", "demo.voxvol")
    raw = open(demo, "rb").read()
    msize = np.frombuffer(raw[0:12], np.uint32)
    dcap = int(np.frombuffer(raw[12:20], np.uint64)[0])
    dvol = lib.ref_volume_new(int(msize[0]), int(msize[1]), int(msize[2]), 1)
    off = 20
    dchunks, dbytes, dlens = [], [], []
    for i in range(dcap):
        sz = int(np.frombuffer(raw[off:off + 2], np.uint16)[0])
        blob = np.frombuffer(raw[off + 2: off + 2 + sz], np.uint8).copy()
        off += 2 + sz
        ch = np.zeros(CHUNK_BYTES, np.uint8)
        lib.ref_decompress_chunk(dvol, blob.ctypes.data, ch.ctypes.data)
        mem = (c_uint8 * (2 * CHUNK_BYTES))()
        nbytes = lib.ref_compress_chunk(dvol, ch.ctypes.data, mem)
        dchunks.append(ch)
        dbytes.append(np.frombuffer(bytes(mem)[:nbytes], np.uint8))
        dlens.append(nbytes)
    lib.ref_volume_free(dvol)
    out["demo_size"] = msize.astype(np.uint32)
    out["demo_chunks"] = np.stack(dchunks)
    out["demo_lens"] = np.array(dlens, np.uint32)
    out["demo_bytes"] = np.concatenate(dbytes)

    # G. the fixed sphere-point table of the lighting shader (voxelLighting.comp:23), read from the shader text
    import re
    src = open(os.path.join(ref_root, "assets", "shaders", "voxelLighting.comp")).read()
    line = [ln for ln in src.splitlines() if "spherePoints[15]" in ln][0]
    pts = [[float(v) for v in m.split(",")] for m in re.findall(r"vec3\(([^)]*)\)", line)]
    out["sphere15"] = np.array(pts, np.float32)

    dst = os.path.join(HERE, "host_goldens.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
