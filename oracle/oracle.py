"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (oracle/dn_oracle.c), the plain-C restatement of
the reference shaders and host packing that the CUDA path is checked against.  Only tests, the smoke
check and the benchmark's CPU-baseline leg use it; the product never imports it.

``OracleMap`` mirrors one volume's device state.  It reads the CPU-side map, chunks, materials and
parameters of a product ``DNvolume`` (public struct fields) and derives the per-launch parameters itself,
as the reference's host code does (voxel.c:883-952): latched time on frame 0 of the lighting split,
normalised sun direction, K-point golden-angle sphere.
"""
import ctypes
import os
import platform
import subprocess
from ctypes import POINTER, Structure, c_float, c_int, c_int32, c_uint8, c_uint16, c_uint32, c_uint64, c_void_p, c_size_t

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libdn_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libdnref.so")

RNG_HASH, RNG_SIN, PERSIST_TRANSPARENCY, REFERENCE_SHADOW = 0, 1, 2, 4


class LightParams(Structure):
    _fields_ = [("sunDir", c_float * 3), ("sunStrength", c_float * 3), ("ambient", c_float * 3), ("camPos", c_float * 3),
                ("skyBot", c_float * 3), ("skyTop", c_float * 3), ("shadowSoftness", c_float), ("time", c_float),
                ("emissiveStrength", c_float), ("numDiffuse", c_uint32), ("maxDiffuse", c_uint32),
                ("diffuseBounceLimit", c_uint32), ("specBounceLimit", c_uint32), ("K", c_uint32), ("flags", c_uint32),
                ("mapId", c_uint32), ("useSpherePoints", c_uint32), ("spherePts", (c_float * 3) * 64)]


class DrawParams(Structure):
    _fields_ = [("invView", (c_float * 4) * 4), ("invCenteredView", (c_float * 4) * 4), ("invProj", (c_float * 4) * 4),
                ("width", c_uint32), ("height", c_uint32), ("viewMode", c_uint32), ("truncate16", c_uint32),
                ("sunStrength", c_float * 3), ("skyBot", c_float * 3), ("skyTop", c_float * 3),
                ("emissiveStrength", c_float), ("pixels", POINTER(c_uint32)), ("npixels", c_uint32),
                ("compose", c_uint32), ("rasterColor", POINTER(c_float)), ("rasterDepth", POINTER(c_float)),
                ("rasterColorW", c_uint32), ("rasterColorH", c_uint32), ("rasterDepthW", c_uint32),
                ("rasterDepthH", c_uint32)]


class Counters(Structure):
    _fields_ = [("rays", c_uint64), ("primary", c_uint64), ("outerSteps", c_uint64), ("chunksEntered", c_uint64),
                ("innerSteps", c_uint64), ("hits", c_uint64), ("litVoxels", c_uint64), ("degenerate", c_uint64)]


class ShapeOp(Structure):
    """dno_shape_op of dn_oracle.h"""
    _fields_ = [("kind", c_int32), ("flip", c_int32), ("material", c_uint8), ("albedo", c_uint8 * 3),
                ("normal", c_float * 3), ("c", c_float * 3), ("v", c_float * 3), ("a", c_float), ("b", c_float),
                ("transform", (c_float * 4) * 4), ("invTransform", (c_float * 4) * 4)]


# dno_shape_hit of dn_oracle.h (the layout of the product's dn_shape_hit)
SHAPE_HIT = np.dtype([("local", "<u2"), ("inside", "u1"), ("pad", "u1"), ("normal", "<f4", 3)])


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def reference_root(arg=None):
    """The reference tree's root: an explicit argument, else the DN_REFERENCE_ROOT environment variable;
    None when neither names an existing directory."""
    root = arg or os.environ.get("DN_REFERENCE_ROOT")
    return root if root and os.path.isdir(root) else None


def build_reference(ref_root=None):
    """Compile the reference's own host C into oracle/_ref (x86-64 only; needs the reference tree, named by
    ref_root or DN_REFERENCE_ROOT).  Returns the library path, or None when it cannot be built here."""
    ref_root = reference_root(ref_root)
    if platform.machine() not in ("x86_64", "AMD64") or ref_root is None:
        return None
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + ref_root], check=True)
    return REF_LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    srcs = [os.path.join(HERE, f) for f in ("dn_oracle.c", "dno_shapes.c", "dn_oracle.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(LIB) < os.path.getmtime(p) for p in srcs):
        build()
    lib = ctypes.CDLL(LIB)
    sigs = [
        ("dno_create", c_void_p, [c_uint32, c_uint32, c_uint32]),
        ("dno_destroy", None, [c_void_p]),
        ("dno_sync", None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int]),
        ("dno_light", None, [c_void_p, c_void_p, POINTER(LightParams), c_int]),
        ("dno_draw", None, [c_void_p, c_void_p, POINTER(DrawParams), c_void_p, c_void_p, c_void_p, c_int]),
        ("dno_light_requests", None, [c_void_p, c_void_p, POINTER(LightParams), c_void_p, c_uint32, c_void_p, c_void_p,
                                      c_void_p, c_int]),
        ("dno_num_requests", c_uint32, [c_void_p]),
        ("dno_requests", POINTER(c_uint32), [c_void_p]),
        ("dno_frame_num", c_uint32, [c_void_p]),
        ("dno_get_counters", None, [c_void_p, POINTER(Counters)]),
        ("dno_reset_counters", None, [c_void_p]),
        ("dno_export_tiles", None, [c_void_p, c_void_p, c_void_p, c_void_p]),
        ("dno_set_lru", None, [c_void_p, c_uint64]),
        ("dno_set_chunk_cap", None, [c_void_p, c_uint64]),
        ("dno_lru_nodes", c_size_t, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t]),
        ("dno_lru_stream", c_int, [c_void_p, ctypes.c_int64, c_uint32, c_void_p]),
        ("dno_lru_unload", None, [c_void_p, ctypes.c_int64]),
        ("dno_lru_sort", None, [c_void_p, c_int]),
        ("dno_lru_grow", None, [c_void_p, c_uint64]),
        ("dno_set_last_used", None, [c_void_p, c_void_p]),
        ("dno_export_lighting", c_uint64, [c_void_p, c_void_p, c_void_p, c_void_p]),
        ("dno_export_samples", None, [c_void_p, c_void_p]),
        ("dno_import_lighting", None, [c_void_p, c_uint64, c_void_p, c_void_p, c_void_p]),
        ("dno_import_samples", None, [c_void_p, c_void_p]),
        ("dno_pack_chunk", None, [c_void_p, c_void_p, c_void_p]),
        ("dno_import_state", None, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_uint32]),
        ("dno_set_requests", None, [c_void_p, c_void_p, c_uint32]),
        ("dno_compress_voxel", None, [c_uint8, c_void_p, c_void_p, c_void_p]),
        ("dno_decompress_voxel", None, [c_uint64, c_void_p, c_void_p, c_void_p]),
        ("dno_sin", c_float, [c_float]),
        ("dno_hash32", c_uint32, [c_uint32]),
        ("dno_sphere_points", None, [c_uint32, c_void_p]),
        ("dno_shape_bounds", None, [POINTER(ShapeOp), c_void_p, c_void_p]),
        ("dno_shape_range", c_int, [POINTER(ShapeOp), c_void_p, c_void_p, c_void_p]),
        ("dno_shape_eval", c_uint64, [POINTER(ShapeOp), c_void_p, c_void_p, c_void_p, c_void_p, c_uint64]),
        ("dno_shape_apply", None, [POINTER(ShapeOp), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p]),
    ]
    for n, r, a in sigs:
        f = getattr(lib, n)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


def _f32(x):
    return np.float32(x)


def normalize_like_reference(v):
    """v * (1 / |v|) in float32 steps (the reference normalises sunDir this way on the host, voxel.c:942)."""
    x, y, z = (_f32(c) for c in v)
    ln = np.sqrt(np.float32(np.float32(np.float32(x * x) + np.float32(y * y)) + np.float32(z * z)))
    if ln == 0:
        return [0.0, 0.0, 0.0]
    inv = np.float32(np.float32(1.0) / ln)
    return [float(np.float32(x * inv)), float(np.float32(y * inv)), float(np.float32(z * inv))]


class OracleMap:
    def __init__(self, map_size):
        self.lib = load()
        self.map_size = tuple(map_size)
        self.ptr = self.lib.dno_create(*self.map_size)
        if not self.ptr:
            raise MemoryError("dno_create")
        self.frame = 0
        self.last_time = 123.456   # reference default, voxel.c:278
        self.lru = False

    def close(self):
        if self.ptr:
            self.lib.dno_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_tiles(self):
        x, y, z = self.map_size
        return x * y * z

    def set_lru(self, num_chunks):
        """the reference's node buffer with least-recently-used unloading, for num_chunks = min(tiles, minChunks)"""
        self.lib.dno_set_lru(self.ptr, num_chunks)
        self.lru = True

    def lru_nodes(self):
        """(buffer size in voxels, node sizes, first voxels, owning tiles or -1)"""
        cap = c_uint64(0)
        n = self.lib.dno_lru_nodes(self.ptr, ctypes.byref(cap), None, None, None, 0)
        sizes = np.zeros(max(n, 1), np.uint32)
        starts = np.zeros(max(n, 1), np.uint64)
        tiles = np.zeros(max(n, 1), np.int64)
        self.lib.dno_lru_nodes(self.ptr, ctypes.byref(cap), sizes.ctypes.data, starts.ctypes.data, tiles.ctypes.data, n)
        return int(cap.value), sizes[:n], starts[:n], tiles[:n]

    def sync(self, vol_s, op=2, split=1):
        """vol_s: a product DNvolume struct (ctypes); reads map / chunks / materials before the product's sync."""
        if self.lru:
            self.lib.dno_set_chunk_cap(self.ptr, vol_s.chunkCap)
        self.lib.dno_sync(self.ptr, ctypes.cast(vol_s.map, c_void_p), ctypes.cast(vol_s.chunks, c_void_p),
                          ctypes.cast(vol_s.materials, c_void_p), op, split)
        self.frame = self.lib.dno_frame_num(self.ptr)

    def light_params(self, vol_s, num_diffuse, max_diffuse, time, flags=RNG_HASH, sphere_points=None):
        if self.frame == 0:
            self.last_time = float(np.float32(time))
        p = LightParams()
        p.sunDir[:] = normalize_like_reference(vol_s.sunDir.tolist())
        p.sunStrength[:] = vol_s.sunStrength.tolist()
        p.ambient[:] = vol_s.ambientLightStrength.tolist()
        p.camPos[:] = vol_s.camPos.tolist()
        p.skyBot[:] = vol_s.skyGradientBot.tolist()
        p.skyTop[:] = vol_s.skyGradientTop.tolist()
        p.shadowSoftness = vol_s.shadowSoftness
        p.time = self.last_time
        p.emissiveStrength = vol_s.emissiveStrength
        p.numDiffuse = max(0, num_diffuse)
        p.maxDiffuse = max(0, max_diffuse)
        p.diffuseBounceLimit = vol_s.diffuseBounceLimit
        p.specBounceLimit = vol_s.specBounceLimit
        p.K = min(64, max(1, vol_s.numDirectRays))
        p.flags = flags | (RNG_SIN if vol_s.rngMode == 1 else 0)
        p.mapId = vol_s.mapId
        if sphere_points is not None:
            p.useSpherePoints = 1
            for k, pt in enumerate(sphere_points):
                p.spherePts[k][:] = pt
            p.K = len(sphere_points)
        return p

    def light(self, vol_s, num_diffuse=1, max_diffuse=1000, time=0.0, nthreads=0, flags=RNG_HASH, sphere_points=None):
        p = self.light_params(vol_s, num_diffuse, max_diffuse, time, flags, sphere_points)
        self.lib.dno_light(self.ptr, ctypes.cast(vol_s.materials, c_void_p), ctypes.byref(p), nthreads)
        return p

    def light_requests(self, vol_s, params, req_idx, nthreads=0):
        req_idx = np.ascontiguousarray(req_idx, dtype=np.uint32)
        n = len(req_idx)
        d = np.zeros((n, 32, 3), np.float32)
        s = np.zeros((n, 32, 3), np.float32)
        v = np.zeros((n, 32), np.uint8)
        self.lib.dno_light_requests(self.ptr, ctypes.cast(vol_s.materials, c_void_p), ctypes.byref(params),
                                    req_idx.ctypes.data, n, d.ctypes.data, s.ctypes.data, v.ctypes.data, nthreads)
        return d, s, v

    def draw(self, vol_s, inv_view, inv_cview, inv_proj, width, height, pixels=None, nthreads=0, raster=None):
        """raster: None, or (colour (h, w, 4) float32, depth (h, w) float32) composed as DN_draw does with
        raster textures"""
        p = DrawParams()
        for M, dst in ((inv_view, p.invView), (inv_cview, p.invCenteredView), (inv_proj, p.invProj)):
            for c in range(4):
                for r in range(4):
                    dst[c][r] = M.m[c][r]
        p.width, p.height = width, height
        p.viewMode = vol_s.camViewMode
        p.truncate16 = vol_s.truncateDispatch
        p.sunStrength[:] = vol_s.sunStrength.tolist()
        p.skyBot[:] = vol_s.skyGradientBot.tolist()
        p.skyTop[:] = vol_s.skyGradientTop.tolist()
        p.emissiveStrength = vol_s.emissiveStrength
        if raster is not None:
            rc = np.ascontiguousarray(raster[0], dtype=np.float32)
            rd = np.ascontiguousarray(raster[1], dtype=np.float32)
            assert rc.ndim == 3 and rc.shape[2] == 4 and rd.ndim == 2
            p.compose = 1
            p.rasterColor = rc.ctypes.data_as(POINTER(c_float))
            p.rasterDepth = rd.ctypes.data_as(POINTER(c_float))
            p.rasterColorH, p.rasterColorW = rc.shape[:2]
            p.rasterDepthH, p.rasterDepthW = rd.shape
        if pixels is not None:
            pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
            p.pixels = pixels.ctypes.data_as(POINTER(c_uint32))
            p.npixels = len(pixels)
            n = len(pixels)
        else:
            n = width * height
        color = np.zeros((n, 4), np.float32)
        hit = np.zeros(n, np.uint32)
        face = np.zeros(n, np.uint8)
        self.lib.dno_draw(self.ptr, ctypes.cast(vol_s.materials, c_void_p), ctypes.byref(p), color.ctypes.data,
                          hit.ctypes.data, face.ctypes.data, nthreads)
        if pixels is None:
            return color.reshape(height, width, 4), hit.reshape(height, width), face.reshape(height, width)
        return color, hit, face

    def counters(self):
        c = Counters()
        self.lib.dno_get_counters(self.ptr, ctypes.byref(c))
        return {k: int(getattr(c, k)) for k, _ in Counters._fields_}

    def reset_counters(self):
        self.lib.dno_reset_counters(self.ptr)

    def requests(self):
        n = self.lib.dno_num_requests(self.ptr)
        if n == 0:
            return np.zeros(0, np.uint32)
        return np.ctypeslib.as_array(self.lib.dno_requests(self.ptr), shape=(n,)).copy()

    def export_tiles(self):
        n = self.num_tiles
        st = np.empty(n, np.uint8)
        vis = np.empty(n, np.uint8)
        lu = np.empty(n, np.uint32)
        self.lib.dno_export_tiles(self.ptr, st.ctypes.data, vis.ctypes.data, lu.ctypes.data)
        ns = np.empty(n, np.uint32)
        self.lib.dno_export_samples(self.ptr, ns.ctypes.data)
        return st, vis, lu, ns

    def export_lighting(self):
        n = self.lib.dno_export_lighting(self.ptr, None, None, None)
        idx = np.empty(n, np.uint32)
        d = np.empty((n, 3), np.float32)
        s = np.empty((n, 3), np.float32)
        if n:
            self.lib.dno_export_lighting(self.ptr, idx.ctypes.data, d.ctypes.data, s.ctypes.data)
        return idx, d, s

    def import_lighting(self, idx, diff, spec):
        idx = np.ascontiguousarray(idx, np.uint32)
        diff = np.ascontiguousarray(diff, np.float32)
        spec = np.ascontiguousarray(spec, np.float32)
        self.lib.dno_import_lighting(self.ptr, len(idx), idx.ctypes.data, diff.ctypes.data, spec.ctypes.data)

    def import_state(self, vol_s, state, vis, frame_num):
        state = np.ascontiguousarray(state, np.uint8)
        vis = np.ascontiguousarray(vis, np.uint8)
        self.lib.dno_import_state(self.ptr, ctypes.cast(vol_s.map, c_void_p), ctypes.cast(vol_s.chunks, c_void_p),
                                  ctypes.cast(vol_s.materials, c_void_p), state.ctypes.data, vis.ctypes.data, frame_num)
        self.frame = frame_num
        self.last_time = float(vol_s.lastTime)

    def set_requests(self, words):
        words = np.ascontiguousarray(words, np.uint32)
        self.lib.dno_set_requests(self.ptr, words.ctypes.data, len(words))

    def import_samples(self, samples):
        samples = np.ascontiguousarray(samples, np.uint32)
        self.lib.dno_import_samples(self.ptr, samples.ctypes.data)


class DenseShapes:
    """A dense CPU map (normal / albedo words per voxel, voxel count per tile) edited by the oracle's
    restatement of the reference's shape functions."""

    def __init__(self, map_size):
        self.lib = load()
        self.size = np.array(map_size, np.uint32)
        n = int(8 * self.size[0] * 8 * self.size[1] * 8 * self.size[2])
        self.normal = np.full(n, 0xFFFFFFFF, np.uint32)
        self.albedo = np.zeros(n, np.uint32)
        self.count = np.zeros(int(self.size.prod()), np.int32)

    @staticmethod
    def op(kind, flip, material, albedo, normal, c, v, a, b, transform, inv):
        o = ShapeOp()
        o.kind, o.flip, o.material = kind, flip, material
        o.albedo[:], o.normal[:], o.c[:], o.v[:] = list(albedo), list(normal), list(c), list(v)
        o.a, o.b = a, b
        t = np.asarray(transform, np.float32).reshape(4, 4)
        it = np.asarray(inv, np.float32).reshape(4, 4)
        for col in range(4):
            o.transform[col][:] = t[col].tolist()
            o.invTransform[col][:] = it[col].tolist()
        return o

    def bounds(self, o):
        mn = np.zeros(3, np.float32)
        mx = np.zeros(3, np.float32)
        self.lib.dno_shape_bounds(ctypes.byref(o), mn.ctypes.data, mx.ctypes.data)
        return mn, mx

    def evaluate(self, o):
        """(cmin, cmax, counts, hits) of the shape on this map, or None when it covers no chunk"""
        cmin = np.zeros(3, np.int32)
        cmax = np.zeros(3, np.int32)
        if not self.lib.dno_shape_range(ctypes.byref(o), self.size.ctypes.data, cmin.ctypes.data, cmax.ctypes.data):
            return None
        nch = int(np.prod(cmax - cmin + 1))
        counts = np.zeros(nch, np.uint32)
        total = self.lib.dno_shape_eval(ctypes.byref(o), cmin.ctypes.data, cmax.ctypes.data, counts.ctypes.data, None, 0)
        hits = np.zeros(max(1, total), SHAPE_HIT)
        self.lib.dno_shape_eval(ctypes.byref(o), cmin.ctypes.data, cmax.ctypes.data, counts.ctypes.data,
                                hits.ctypes.data, total)
        return cmin, cmax, counts, hits[:total]

    def apply(self, o):
        ev = self.evaluate(o)
        if ev is None:
            return None
        cmin, cmax, counts, hits = ev
        hits = np.ascontiguousarray(hits) if len(hits) else np.zeros(1, SHAPE_HIT)
        self.lib.dno_shape_apply(ctypes.byref(o), self.size.ctypes.data, cmin.ctypes.data, cmax.ctypes.data,
                                 counts.ctypes.data, hits.ctypes.data, self.normal.ctypes.data, self.albedo.ctypes.data,
                                 self.count.ctypes.data)
        return ev

    def tile_flags(self):
        return (self.count != 0).astype(np.uint8)
