"""Generates tests/golden/shape_goldens.npz from the reference's own shape functions.

The reference's src/DoonEngine/voxel.c and voxelShapes.c are compiled unchanged from the reference tree
into oracle/_ref/libdnref.so (oracle/ref/Makefile; no GL code is linked).  Each script below is a seeded
sequence of DN_shape_* calls on a CPU map of 6x4x6 chunks; the golden is the map's voxels afterwards
(normal and albedo words, tile flags) plus each call's quaternion, transform and inverse.  x86-64 only.

    python tests/golden/make_shape_golden.py [/path/to/reference]
"""
import ctypes
import os
import sys
from ctypes import c_uint32, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

MAP = (6, 4, 6)

# ref_shape_op of oracle/ref/dnref_shim.c
OP = np.dtype([("kind", "<i4"), ("flip", "<i4"), ("transform", "<i4"), ("material", "u1"), ("albedo", "u1", 3),
               ("normal", "<f4", 3), ("c", "<f4", 3), ("v", "<f4", 3), ("a", "<f4"), ("b", "<f4"),
               ("euler", "<f4", 3)], align=True)


def q(x, step=0.25):
    return np.round(np.asarray(x, np.float64) / step) * step


def op(kind, c, v=(0, 0, 0), a=0.0, b=0.0, euler=(0, 0, 0), material=1, albedo=(200, 120, 60), flip=0,
       transform=0, normal=(0.0, 1.0, 0.0)):
    r = np.zeros((), OP)
    r["kind"], r["flip"], r["transform"], r["material"] = kind, flip, transform, material
    r["albedo"], r["normal"], r["c"], r["v"] = albedo, normal, c, v
    r["a"], r["b"], r["euler"] = a, b, euler
    return r


def bowl_script(rng):
    """the reference's cereal-bowl recipe (main.c:70-122) at this map's scale"""
    c = (24.5, 18.25, 24.75)
    ops = [op(0, c, a=14.0, material=1, albedo=(230, 230, 220)),
           op(0, c, a=9.0, material=255, flip=1),
           op(1, (c[0], c[1] + 7.0, c[2]), v=(14.0, 7.0, 14.0), material=255, flip=1)]
    for k in range(14):
        p = (c[0] + rng.integers(-6, 7), c[1] - rng.integers(0, 6), c[2] + rng.integers(-6, 7))
        e = tuple(float(x) for x in rng.integers(0, 360, 3))
        alb = tuple(int(x) for x in rng.integers(0, 256, 3))
        kind = (3, 0, 1)[k % 3]
        if kind == 3:
            ops.append(op(3, p, a=3.0, b=1.5, euler=e, material=2, albedo=alb))
        elif kind == 0:
            ops.append(op(0, p, a=2.5, material=3, albedo=alb))
        else:
            ops.append(op(1, p, v=(2.0, 2.0, 2.0), euler=e, material=4, albedo=alb))
    return ops


def kinds_script(rng, transform):
    """every kind, placed and removed (with and without flipped normals), rotated, partly outside the map"""
    X, Y, Z = (8 * s for s in MAP)
    ops = []
    for rep in range(3):
        for kind in range(8):
            c = q(rng.uniform((-4, -4, -4), (X + 4, Y + 4, Z + 4)))
            e = tuple(float(x) for x in rng.integers(0, 360, 3)) if rep else (0.0, 0.0, 0.0)
            v = q(rng.uniform(2.0, 9.0, 3))
            a, b = float(q(rng.uniform(2.0, 8.0))), float(q(rng.uniform(1.0, 7.0)))
            if kind == 3:
                b = min(b, a - 0.5)
            alb = tuple(int(x) for x in rng.integers(0, 256, 3))
            ops.append(op(kind, c, v=v, a=a, b=b, euler=e, material=int(rng.integers(0, 8)), albedo=alb,
                          transform=transform))
            if rng.random() < 0.45:
                c2 = c + q(rng.uniform(-3.0, 3.0, 3))
                k2 = int(rng.integers(0, 8))
                ops.append(op(k2, c2, v=v * 0.75, a=a * 0.75, b=b * 0.75, euler=e, material=255,
                              flip=int(rng.random() < 0.7), transform=transform))
    # a shape wholly outside the map, and one covering the map's corner
    ops.append(op(0, (-40.0, -40.0, -40.0), a=5.0))
    ops.append(op(1, (X - 1.0, Y - 1.0, Z - 1.0), v=(4.0, 4.0, 4.0), euler=(30.0, 45.0, 60.0), material=6))
    return ops


def run(lib, ops):
    vol = lib.ref_volume_new(MAP[0], MAP[1], MAP[2], 16)
    mats = []
    for o in ops:
        buf = np.ascontiguousarray(o.reshape(1))
        qv = np.zeros(4, np.float32)
        t = np.zeros(16, np.float32)
        it = np.zeros(16, np.float32)
        lib.ref_shape_matrices(buf.ctypes.data, qv.ctypes.data, t.ctypes.data, it.ctypes.data)
        mats.append(np.concatenate([qv, t, it]))
        lib.ref_shape_run(vol, buf.ctypes.data)
    n = 8 * MAP[0] * 8 * MAP[1] * 8 * MAP[2]
    nw = np.zeros(n, np.uint32)
    aw = np.zeros(n, np.uint32)
    tf = np.zeros(MAP[0] * MAP[1] * MAP[2], np.uint8)
    lib.ref_export_voxels(vol, nw.ctypes.data, aw.ctypes.data, tf.ctypes.data)
    lib.ref_volume_free(vol)
    return np.stack(mats), nw, aw, tf


def main():
    ref_root = O.reference_root(sys.argv[1] if len(sys.argv) > 1 else None)
    if ref_root is None:
        sys.exit("usage: %s REFERENCE_ROOT (or set DN_REFERENCE_ROOT)" % sys.argv[0])
    path = O.build_reference(ref_root)
    if not path:
        raise SystemExit("the reference host C builds only on x86-64 with the reference tree present")
    lib = ctypes.CDLL(path)
    for name, restype, argtypes in (("ref_volume_new", c_void_p, [c_uint32] * 4), ("ref_volume_free", None, [c_void_p]),
                                    ("ref_shape_run", None, [c_void_p, c_void_p]),
                                    ("ref_shape_matrices", None, [c_void_p] * 4),
                                    ("ref_export_voxels", None, [c_void_p] * 4)):
        getattr(lib, name).restype = restype
        getattr(lib, name).argtypes = argtypes
    rng = np.random.default_rng(2024)
    scripts = {"bowl": bowl_script(rng), "kinds": kinds_script(rng, 0), "transform": kinds_script(rng, 1)}
    out = {"map": np.array(MAP, np.uint32)}
    for name, ops in scripts.items():
        arr = np.array(ops, OP)
        mats, nw, aw, tf = run(lib, arr)
        out[name + "_ops"] = arr.view(np.uint8).reshape(len(arr), OP.itemsize)
        out[name + "_mats"] = mats
        out[name + "_normal"] = nw
        out[name + "_albedo"] = aw
        out[name + "_tiles"] = tf
        print(name, len(arr), "ops,", int((nw >> 24 != 255).sum()), "solid voxels,", int(tf.sum()), "chunks")
    np.savez_compressed(os.path.join(HERE, "shape_goldens.npz"), **out)


if __name__ == "__main__":
    main()
