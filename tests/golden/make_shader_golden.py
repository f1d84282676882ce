"""Generates tests/golden/shader_goldens.npz: outputs of the reference's own compute shaders, run on the
CPU, for the oracle pin in tests/test_shader_pin.py.

The shaders (assets/shaders/voxelShared.comp, voxelDraw.comp, voxelLighting.comp) are translated to C++
by oracle/ref/glsl_to_cpp.py and executed per invocation by oracle/ref/pin_harness.cpp; the scenes are
built with the reference's own edit API and packed by its own _DN_chunk_to_gpu (oracle/ref/dnref_shim.c).
Stored: the scene inputs (CPU chunks, materials, lighting history, sample counts, request words, camera
matrices, parameters) and the shaders' outputs (draw RGBA and tile flags per camera and view mode; the
FP32 specular and diffuse light of every lit voxel, captured before quantisation).

    python tests/golden/make_shader_golden.py [/path/to/reference]
"""
import ctypes
import os
import re
import subprocess
import sys
from ctypes import POINTER, Structure, c_float, c_uint8, c_uint32, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import load_ref, CHUNK_BYTES  # noqa: E402
from oracle import oracle as O  # noqa: E402

INV255 = np.float32(0.00392156862)
INV65535 = np.float32(0.0000152590219)


class PinMap(Structure):
    _fields_ = [("sx", c_uint32), ("sy", c_uint32), ("sz", c_uint32), ("handles", c_void_p), ("chunks", c_void_p),
                ("voxels", c_void_p), ("nvox", c_uint32), ("materials", c_void_p), ("skyBot", c_float * 3),
                ("skyTop", c_float * 3), ("sunStrength", c_float * 3), ("ambient", c_float * 3)]


def load_pin(ref_root):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "pin", "REF=" + ref_root], check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libglslpin.so"))
    lib.pin_draw.argtypes = [POINTER(PinMap), c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p]
    lib.pin_light.argtypes = [POINTER(PinMap), c_void_p, c_uint32, c_float, c_uint32, c_uint32, c_uint32, c_uint32,
                              c_void_p, c_float, c_void_p, c_void_p, c_void_p, c_void_p]
    return lib


def materials(kind):
    m = np.zeros((256, 8), np.uint32)
    f = m.view(np.float32)
    f[:, 3] = 1.0   # opacity
    f[:, 4] = 1.0   # refract index
    # 0 diffuse, 1 specular sky-reflecting, 2 specular no sky, 3 emissive, 4 transparent, 5 highlight-only,
    # 6 transparent specular, 7 mostly specular
    f[1, 5], m[1, 6], m[1, 7] = 0.4, 1, 3
    f[2, 5], m[2, 6], m[2, 7] = 0.25, 0, 2
    m[3, 2] = 1
    f[4, 3], f[4, 4] = 0.5, 1.3
    f[5, 5], m[5, 6], m[5, 7] = 0.5, 2, 4
    f[6, 3], f[6, 4], f[6, 5], m[6, 6], m[6, 7] = 0.35, 1.52, 0.3, 1, 2
    f[7, 5], m[7, 6], m[7, 7] = 0.9, 1, 8
    if kind == "opaque":
        f[4, 3] = 1.0
        f[6, 3] = 1.0
    return m


def build_scene(lib, rng, size, kind):
    vol = lib.ref_volume_new(*size, 8)
    X, Y, Z = size[0] * 8, size[1] * 8, size[2] * 8

    def put(x, y, z, mat, n):
        mp = np.array([x // 8, y // 8, z // 8], np.int32)
        cp = np.array([x % 8, y % 8, z % 8], np.int32)
        nn = np.asarray(n, np.float32)
        al = rng.integers(20, 256, 3).astype(np.uint8)
        lib.ref_set_voxel(vol, mp.ctypes.data, cp.ctypes.data, int(mat), nn.ctypes.data, al.ctypes.data)

    for z in range(Z):
        for x in range(X):
            h = int(Y * 0.25 + 3 * np.sin(x / 5.0) + 3 * np.cos(z / 7.0))
            for y in range(max(1, h)):
                put(x, y, z, rng.integers(0, 3) if y < h - 1 else rng.integers(0, 8), (0.1 * np.sin(x), 1.0, 0.1 * np.cos(z)))
    for _ in range(10):
        c = rng.integers(2, [X - 3, Y - 3, Z - 3])
        r = int(rng.integers(1, 4))
        mat = int(rng.integers(0, 8))
        for dz in range(-r, r + 1):
            for dy in range(-r, r + 1):
                for dx in range(-r, r + 1):
                    if dx * dx + dy * dy + dz * dz <= r * r:
                        put(c[0] + dx, c[1] + dy, c[2] + dz, mat, (dx, dy, dz) if (dx or dy or dz) else (0, 1, 0))
    tiles = size[0] * size[1] * size[2]
    info = (ctypes.c_uint64 * 3)()
    lib.ref_volume_info(vol, info)
    cap = int(info[0])
    mapb = np.ctypeslib.as_array(ctypes.cast(lib.ref_volume_map(vol), POINTER(c_uint8)), shape=(tiles * 8,)).copy()
    chb = np.ctypeslib.as_array(ctypes.cast(lib.ref_volume_chunks(vol), POINTER(c_uint8)), shape=(cap * CHUNK_BYTES,)).copy()
    lib.ref_volume_free(vol)
    return mapb.reshape(tiles, 8), chb.reshape(cap, CHUNK_BYTES)


def gpu_buffers(ref, size, mapb, chb, mats, rng, history):
    """The reference's GPU layout: handles, dense per-tile chunk records, voxels with quantised lighting."""
    tiles = size[0] * size[1] * size[2]
    handles = np.zeros((tiles, 3), np.uint32)
    chunks = np.zeros((tiles, 23), np.uint32)
    vox = []
    base = np.full(tiles, 0xFFFFFFFF, np.uint32)
    samples = rng.choice([0, 0, 3, 7], tiles).astype(np.uint32)
    hist_rows = []
    n = 0
    for t in range(tiles):
        if not mapb[t, 0]:
            continue
        ci = int(mapb[t, 4:8].view(np.uint32)[0])
        ch = np.ascontiguousarray(chb[ci])
        mask = (c_uint32 * 16)(); part = (c_uint32 * 3)(); nv = c_uint32(); vv = (c_uint32 * 1024)()
        ref.ref_chunk_to_gpu(ch.ctypes.data, mats.ctypes.data, mask, part, ctypes.byref(nv), vv)
        x, y, z = t % size[0], (t // size[0]) % size[1], t // (size[0] * size[1])
        handles[t] = [2, 0, n]
        base[t] = n
        chunks[t, 0:3] = np.array([x, y, z], np.int32).view(np.uint32)
        chunks[t, 3] = samples[t]
        chunks[t, 4:7] = list(part)
        chunks[t, 7:23] = list(mask)
        rank = 0
        for li in range(512):
            if not (mask[li >> 5] >> (li & 31)) & 1:
                continue
            nw, aw = vv[2 * rank], vv[2 * rank + 1]
            if history:
                sq = rng.integers(0, 256, 3).astype(np.uint32)
                dq = rng.integers(0, 65536, 3).astype(np.uint32)
            else:
                sq = np.zeros(3, np.uint32); dq = np.zeros(3, np.uint32)
            w1 = (aw & 0xFFFFFF00) | int(sq[0])
            w2 = (int(sq[1]) << 24) | (int(sq[2]) << 16) | int(dq[0])
            w3 = (int(dq[1]) << 16) | int(dq[2])
            vox.append([nw, w1, w2, w3])
            gx, gy, gz = x * 8 + (li & 7), y * 8 + ((li >> 3) & 7), z * 8 + (li >> 6)
            hist_rows.append([gx + size[0] * 8 * (gy + size[1] * 8 * gz), *dq, *sq])
            rank += 1
        n += rank
    return handles, chunks, np.array(vox, np.uint32), base, samples, np.array(hist_rows, np.uint32)


def requests_for(size, mapb, chunks):
    words = []
    for t in range(size[0] * size[1] * size[2]):
        if not mapb[t, 0]:
            continue
        nvox = sum(bin(int(w)).count("1") for w in chunks[t, 7:23])
        for i in range(0, nvox, 32):
            words.append((t << 4) | (i // 32))
    return np.array(words, np.uint32)


def main():
    ref_root = O.reference_root(sys.argv[1] if len(sys.argv) > 1 else None)
    if ref_root is None:
        sys.exit("usage: %s REFERENCE_ROOT (or set DN_REFERENCE_ROOT)" % sys.argv[0])
    ref = load_ref(ref_root)
    pin = load_pin(ref_root)
    src = open(os.path.join(ref_root, "assets", "shaders", "voxelLighting.comp")).read()
    line = [ln for ln in src.splitlines() if "spherePoints[15]" in ln][0]
    sphere = np.array([[float(v) for v in m.split(",")] for m in re.findall(r"vec3\(([^)]*)\)", line)], np.float32)
    rng = np.random.default_rng(7)
    out = {"sphere15": sphere}
    sky_bot = np.float32([0.71, 0.85, 0.90]); sky_top = np.float32([0.00, 0.45, 0.74])
    sun = np.float32([0.6, 0.6, 0.6]); amb = np.float32([0.01, 0.01, 0.01])
    scenes = [("opaque", (4, 3, 4), False), ("transparent", (3, 3, 4), True)]
    for si, (kind, size, history) in enumerate(scenes):
        mats = materials(kind)
        mapb, chb = build_scene(ref, rng, size, kind)
        handles, chunks, vox, base, samples, hist = gpu_buffers(ref, size, mapb, chb, mats, rng, history)
        reqs = requests_for(size, mapb, chunks)
        pre = "s%d_" % si
        out[pre + "size"] = np.array(size, np.uint32)
        out[pre + "map"] = mapb
        out[pre + "chunks"] = chb
        out[pre + "materials"] = mats
        out[pre + "samples"] = samples
        out[pre + "history"] = hist
        out[pre + "requests"] = reqs
        pm = PinMap()
        pm.sx, pm.sy, pm.sz = size
        pm.chunks = chunks.ctypes.data
        pm.voxels = vox.ctypes.data
        pm.nvox = len(vox)
        pm.materials = mats.ctypes.data
        pm.skyBot[:], pm.skyTop[:], pm.sunStrength[:], pm.ambient[:] = sky_bot, sky_top, sun, amb
        # draw: two cameras (outside looking in, inside the map), view modes 0 and 5
        cams = [((-0.5, 2.9, -0.7), (28.0, 40.0, 0.0), 80.0), ((1.6, 1.4, 2.1), (10.0, 200.0, 5.0), 95.0)]
        W, H = 64, 48
        draw_h = handles.copy()
        pm.handles = draw_h.ctypes.data
        cam_mats, draws, flags = [], [], []
        for ci, (pos, orient, fov) in enumerate(cams):
            ms = [(c_float * 16)() for _ in range(5)]
            pos_a, orient_a = np.float32(pos), np.float32(orient)     # keep both arrays alive across the call
            ref.ref_view_projection(pos_a.ctypes.data, orient_a.ctypes.data, fov, H / W, 0.1, 100.0, *ms)
            inv = [np.array(list(m), np.float32) for m in ms[2:5]]
            cam_mats.append(np.stack(inv))
            for vm in (0, 5):
                rgba = np.zeros((H, W, 4), np.float32)
                fl = np.zeros(len(handles), np.uint32)
                pin.pin_draw(ctypes.byref(pm), inv[0].ctypes.data, inv[1].ctypes.data, inv[2].ctypes.data, W, H, vm,
                             rgba.ctypes.data, fl.ctypes.data)
                draws.append(rgba)
                flags.append(fl)
        out[pre + "cam_mats"] = np.stack(cam_mats)
        out[pre + "draw_rgba"] = np.stack(draws)
        out[pre + "draw_flags"] = np.stack(flags)
        # lighting: two parameter sets
        light_h = handles.copy()
        light_h[light_h[:, 0] == 2, 0] = 6   # loaded and visible
        pm.handles = light_h.ctypes.data
        lp = [(1.75, 1), (3.1, 2)]
        sunDir = np.float32([0.4, 1.0, 0.25])
        ln = np.sqrt(np.float32(np.float32(np.float32(sunDir[0] * sunDir[0]) + np.float32(sunDir[1] * sunDir[1])) + np.float32(sunDir[2] * sunDir[2])))
        sunDir = (sunDir * np.float32(np.float32(1.0) / ln)).astype(np.float32)
        cam = np.float32([-0.5, 2.9, -0.7])
        lspec, ldiff, lvalid = [], [], []
        for t, nd in lp:
            sp = np.zeros((len(vox), 3), np.float32); df = np.zeros((len(vox), 3), np.float32); vd = np.zeros(len(vox), np.uint8)
            pin.pin_light(ctypes.byref(pm), reqs.ctypes.data, len(reqs), t, nd, 1000, 5, 2, sunDir.ctypes.data, 10.0,
                          cam.ctypes.data, sp.ctypes.data, df.ctypes.data, vd.ctypes.data)
            lspec.append(sp); ldiff.append(df); lvalid.append(vd)
        out[pre + "light_params"] = np.array([[t, nd] for t, nd in lp], np.float32)
        out[pre + "light_sun"] = sunDir
        out[pre + "light_cam"] = cam
        # pool index -> global voxel index, in the reference's layout
        gidx = np.zeros(len(vox), np.uint32)
        for t in range(len(base)):
            if base[t] == 0xFFFFFFFF:
                continue
            x, y, z = t % size[0], (t // size[0]) % size[1], t // (size[0] * size[1])
            r = 0
            for li in range(512):
                if (chunks[t, 7 + (li >> 5)] >> (li & 31)) & 1:
                    gx, gy, gz = x * 8 + (li & 7), y * 8 + ((li >> 3) & 7), z * 8 + (li >> 6)
                    gidx[base[t] + r] = gx + size[0] * 8 * (gy + size[1] * 8 * gz)
                    r += 1
        out[pre + "light_gidx"] = gidx
        out[pre + "light_spec"] = np.stack(lspec)
        out[pre + "light_diff"] = np.stack(ldiff)
        out[pre + "light_valid"] = np.stack(lvalid)
        print(kind, "voxels", len(vox), "requests", len(reqs), "lit", [int(v.sum()) for v in lvalid],
              "draw hits", [int((d[..., 3] > 0).sum()) for d in draws])
    dst = os.path.join(HERE, "shader_goldens.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
