"""Helpers of the shape tests: the reference goldens (tests/golden/shape_goldens.npz, made by
tests/golden/make_shape_golden.py from the reference's own voxelShapes.c), the test transform function,
and runners for the product and the oracle."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np

from parity_util import ROOT
import doonengine_gb300 as dn
from doonengine_gb300 import _lib as L
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "shape_goldens.npz")
SCRIPTS = ("bowl", "kinds", "transform")

# ref_shape_op of oracle/ref/dnref_shim.c, as stored in the goldens
OP = np.dtype([("kind", "<i4"), ("flip", "<i4"), ("transform", "<i4"), ("material", "u1"), ("albedo", "u1", 3),
               ("normal", "<f4", 3), ("c", "<f4", 3), ("v", "<f4", 3), ("a", "<f4"), ("b", "<f4"),
               ("euler", "<f4", 3)], align=True)

_cb = None


def goldens():
    return np.load(GOLDEN)


def script(g, name):
    ops = np.ascontiguousarray(g[name + "_ops"]).view(OP).reshape(-1)
    return ops, g[name + "_mats"]


def transform_func():
    """pointer to dn_test_shape_transform (tests/shape_transform.c), compiled once per process"""
    global _cb
    if _cb is None:
        out = os.path.join(tempfile.mkdtemp(prefix="dnshape"), "libshapecb.so")
        subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "shape_transform.c"), "-o", out, "-lm"], check=True)
        lib = ctypes.CDLL(out)
        _cb = (lib, ctypes.cast(lib.dn_test_shape_transform, ctypes.c_void_p).value)
    return _cb[1]


def product_matrices(o):
    """the quaternion, transform and inverse the product builds for a shape call (as the shim exports them)"""
    lib = dn.load()
    q = lib.DN_quaternion_from_euler(L.DNvec3(*[float(x) for x in o["euler"]]))
    rot = lib.DN_quaternion_to_mat4(q)
    at = L.DNvec3(*[float(x) for x in o["c"]])
    if o["kind"] == 6:
        # the cone's transform is placed at its apex: base + (rot * (0, 1, 0, 1)).xyz * h
        up = lib.DN_mat4_mult_vec4(rot, L.DNvec4(0.0, 1.0, 0.0, 1.0))
        at = lib.DN_vec3_add(at, lib.DN_vec3_scale(L.DNvec3(up.x, up.y, up.z), float(o["b"])))
    t = lib.DN_mat4_mult(lib.DN_mat4_translate(at), rot)
    it = lib.DN_mat4_inv(t)
    flat = lambda mm: np.array([mm.m[c][r] for c in range(4) for r in range(4)], np.float32)
    return np.concatenate([np.array([q.x, q.y, q.z, q.w], np.float32), flat(t), flat(it)])


def oracle_op(o, mats):
    t = mats[4:20].reshape(4, 4)
    it = mats[20:36].reshape(4, 4)
    return O.DenseShapes.op(int(o["kind"]), int(o["flip"]), int(o["material"]), o["albedo"], o["normal"], o["c"],
                            o["v"], float(o["a"]), float(o["b"]), t, it)


def run_oracle(map_size, ops, mats):
    d = O.DenseShapes(map_size)
    for o, m in zip(ops, mats):
        d.apply(oracle_op(o, m))
    return d.normal, d.albedo, d.tile_flags()


def run_product(map_size, ops, host_apply_only=False, mats=None):
    """the ops through the product on a CPU-only volume: DN_shape_* (GPU evaluation), or, with
    host_apply_only, the oracle's evaluated hits through the product's host half (dn_shape_apply)"""
    lib = dn.load()
    vol = dn.Volume(map_size, 16, cpu_only=True)
    try:
        for k, o in enumerate(ops):
            func = transform_func() if o["transform"] else None
            voxel = (int(o["material"]), [float(x) for x in o["normal"]], [int(x) for x in o["albedo"]])
            if not host_apply_only:
                vol.shape(int(o["kind"]), voxel, [float(x) for x in o["c"]], [float(x) for x in o["v"]], float(o["a"]),
                          float(o["b"]), [float(x) for x in o["euler"]], bool(o["flip"]), func)
                continue
            d = O.DenseShapes(map_size)
            oo = oracle_op(o, mats[k])
            ev = d.evaluate(oo)
            if ev is None:
                continue
            cmin, cmax, counts, hits = ev
            mn, mx = d.bounds(oo)
            vox = L.DNvoxel()
            vox.material = voxel[0]
            vox.normal = L.DNvec3(*voxel[1])
            vox.albedo = L.DNcolor(*voxel[2])
            inv = L.DNmat4()
            it = mats[k][20:36].reshape(4, 4)
            for c in range(4):
                for r in range(4):
                    inv.m[c][r] = float(it[c][r])
            hits = np.ascontiguousarray(hits) if len(hits) else np.zeros(1, O.SHAPE_HIT)
            lib.dn_shape_apply(vol.ptr, vox, bool(o["flip"]), int(o["kind"]) == 0, func, None, L.DNvec3(*mn.tolist()),
                               L.DNvec3(*mx.tolist()), inv, cmin.ctypes.data, cmax.ctypes.data, counts.ctypes.data,
                               hits.ctypes.data)
        return vol.export_voxels()
    finally:
        vol.close()


def same_map(a, b, where):
    (na, aa, ta), (nb, ab, tb) = a, b
    assert np.array_equal(ta, tb), "%s: tile flags differ at %s" % (where, np.where(ta != tb)[0][:8])
    bad = np.where(na != nb)[0]
    assert len(bad) == 0, "%s: %d normal words differ, first voxel %d: %08x vs %08x" % (
        where, len(bad), bad[0], na[bad[0]], nb[bad[0]])
    bad = np.where(aa != ab)[0]
    assert len(bad) == 0, "%s: %d albedo words differ, first voxel %d: %08x vs %08x" % (
        where, len(bad), bad[0], aa[bad[0]], ab[bad[0]])
