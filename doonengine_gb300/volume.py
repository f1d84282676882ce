"""Python mirror of the DN_* API: a thin object wrapper over libdoonengine.so for tests, benchmarks and
tools.  Every call goes through the C ABI; nothing here computes lighting or traverses rays."""
import ctypes
from ctypes import POINTER, byref, c_double, c_float, c_int64, c_size_t, c_uint8, c_uint32, c_uint64, c_void_p

import numpy as np

from . import _lib as L

DN_READ, DN_WRITE, DN_READ_WRITE = 0, 1, 2

_callback_keepalive = []
_messages = []


def install_message_callback(store=True, echo=False):
    """Set g_DN_message_callback to collect (type, severity, text) tuples in ``messages()``."""
    lib = L.load()

    def cb(t, s, m):
        txt = m.decode(errors="replace") if m else ""
        if store:
            _messages.append((t, s, txt))
        if echo:
            print("[DN %d/%d] %s" % (t, s, txt))

    f = L.MESSAGE_CALLBACK(cb)
    _callback_keepalive.append(f)
    ptr = ctypes.c_void_p.in_dll(lib, "g_DN_message_callback")
    ptr.value = ctypes.cast(f, ctypes.c_void_p).value
    return f


def messages():
    return _messages


def init():
    lib = L.load()
    if not lib.DN_init():
        raise RuntimeError("DN_init failed: %s" % lib.dn_cuda_last_error().decode())
    return lib


def mat_to_np(m):
    """DNmat4 -> 4x4 numpy array indexed [col][row]."""
    return np.array([[m.m[c][r] for r in range(4)] for c in range(4)], dtype=np.float32)


class Image:
    """A DNimage (device or pinned host memory)."""

    def __init__(self, width, height, on_device=True, hit_info=True):
        self.lib = L.load()
        self.ptr = self.lib.DN_image_create(width, height, 1 if on_device else 0, 1 if hit_info else 0)
        if not self.ptr:
            raise RuntimeError("DN_image_create failed")
        self.width, self.height, self.on_device = width, height, on_device

    def close(self):
        if self.ptr:
            self.lib.DN_image_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def numpy(self):
        """(color [h,w,4] float32, hit [h,w] uint32, face [h,w] uint8) copied to the host."""
        n = self.width * self.height
        img = self.ptr.contents
        # device work runs on per-volume non-blocking streams: wait for it before reading the image
        self.lib.dn_cuda_device_sync()
        color = np.empty((self.height, self.width, 4), np.float32)
        hit = np.empty((self.height, self.width), np.uint32)
        face = np.empty((self.height, self.width), np.uint8)
        if self.on_device:
            self.lib.dn_cuda_memcpy_d2h(color.ctypes.data, ctypes.cast(img.color, c_void_p), n * 16)
            if img.hitIndex:
                self.lib.dn_cuda_memcpy_d2h(hit.ctypes.data, ctypes.cast(img.hitIndex, c_void_p), n * 4)
            if img.hitFace:
                self.lib.dn_cuda_memcpy_d2h(face.ctypes.data, ctypes.cast(img.hitFace, c_void_p), n)
        else:
            ctypes.memmove(color.ctypes.data, img.color, n * 16)
            if img.hitIndex:
                ctypes.memmove(hit.ctypes.data, img.hitIndex, n * 4)
            if img.hitFace:
                ctypes.memmove(face.ctypes.data, img.hitFace, n)
        return color, hit, face


class Texture:
    """A raster texture (DN_texture_create): RGBA32F colour or DEPTH32F window depth, in device memory."""

    RGBA32F, DEPTH32F = 0, 1

    def __init__(self, width, height, fmt):
        self.lib = L.load()
        self.handle = self.lib.DN_texture_create(width, height, fmt)
        if self.handle <= 0:
            raise RuntimeError("DN_texture_create failed")
        self.width, self.height, self.fmt = width, height, fmt

    def upload(self, texels):
        """texels: (height, width, 4) for colour, (height, width) for depth; converted to float32."""
        shape = (self.height, self.width, 4) if self.fmt == self.RGBA32F else (self.height, self.width)
        a = np.ascontiguousarray(texels, dtype=np.float32)
        if a.shape != shape:
            raise ValueError("texture data of shape %s, expected %s" % (a.shape, shape))
        if not self.lib.DN_texture_upload(self.handle, a.ctypes.data):
            raise RuntimeError("DN_texture_upload failed")

    def close(self):
        if self.handle > 0:
            self.lib.DN_texture_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _raster_handles(raster):
    """(colour Texture, depth Texture) or None -> the two DN_draw handles"""
    if raster is None:
        return -1, -1
    return raster[0].handle, raster[1].handle


class Volume:
    """Owns one DNvolume."""

    def __init__(self, map_size, min_chunks=256, cpu_only=False, _ptr=None):
        self.lib = L.load()
        if _ptr is not None:
            self.ptr = _ptr
        else:
            ms = L.DNuvec3(*map_size)
            self.ptr = (self.lib.DN_create_volume_cpu if cpu_only else self.lib.DN_create_volume)(ms, min_chunks)
        if not self.ptr:
            raise RuntimeError("DN_create_volume failed: %s" % self.lib.dn_cuda_last_error().decode())

    @classmethod
    def load(cls, path, min_chunks=256):
        lib = L.load()
        p = lib.DN_load_volume(path.encode(), min_chunks)
        if not p:
            raise RuntimeError("DN_load_volume failed for %s" % path)
        return cls(None, _ptr=p)

    def save(self, path):
        return bool(self.lib.DN_save_volume(path.encode(), self.ptr))

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.DN_delete_volume(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def s(self):
        return self.ptr.contents

    @property
    def map_size(self):
        m = self.s.mapSize
        return (m.x, m.y, m.z)

    @property
    def num_tiles(self):
        x, y, z = self.map_size
        return x * y * z

    # ---- edits
    def set_voxel(self, mp, cp, material, normal, albedo):
        v = L.DNvoxel(material, L.DNvec3(*normal), L.DNcolor(*albedo))
        self.lib.DN_set_voxel(self.ptr, L.DNivec3(*mp), L.DNivec3(*cp), v)

    def set_compressed(self, mp, cp, normal_word, albedo_word):
        self.lib.DN_set_compressed_voxel(self.ptr, L.DNivec3(*mp), L.DNivec3(*cp), L.DNcompressedVoxel(normal_word, albedo_word))

    def remove_voxel(self, mp, cp):
        self.lib.DN_remove_voxel(self.ptr, L.DNivec3(*mp), L.DNivec3(*cp))

    def get_compressed(self, mp, cp):
        c = self.lib.DN_get_compressed_voxel(self.ptr, L.DNivec3(*mp), L.DNivec3(*cp))
        return c.normal, c.albedo

    def set_material(self, i, emissive=0, opacity=1.0, refract=1.0, specular=0.0, reflect_type=0, shininess=1):
        m = self.s.materials[i]
        m.emissive, m.opacity, m.refractIndex = emissive, opacity, refract
        m.specular, m.reflectType, m.shininess = specular, reflect_type, shininess

    def nonempty_chunks(self):
        return sum(1 for t in range(self.num_tiles) if self.s.map[t].flag)

    # ---- frame
    def view_proj(self, aspect, near=0.1, far=100.0):
        v, p = L.DNmat4(), L.DNmat4()
        self.lib.DN_set_view_projection_matrices(self.ptr, aspect, near, far, byref(v), byref(p))
        return v, p

    def draw(self, image, view, proj, raster=None):
        """raster: None, or (colour Texture, depth Texture) to compose with"""
        self.lib.DN_draw(self.ptr, image.ptr, view, proj, *_raster_handles(raster))

    def sync(self, op=DN_READ_WRITE, split=1):
        self.lib.DN_sync_gpu(self.ptr, op, split)

    def update_lighting(self, num_diffuse=1, max_diffuse=1000, time=0.0):
        self.lib.DN_update_lighting(self.ptr, num_diffuse, max_diffuse, time)

    def finish(self):
        return bool(self.lib.DN_finish(self.ptr))

    def stats(self):
        s = L.DNstats()
        if not self.lib.DN_get_stats(self.ptr, byref(s)):
            raise RuntimeError("DN_get_stats failed: %s" % self.lib.dn_cuda_last_error().decode())
        return {k: int(getattr(s, k)) for k, _ in L.DNstats._fields_}

    def stats_kind(self, kind):
        """kind 0: all kernels, 1: draw, 2: lighting (k_light + k_commit)."""
        s = L.DNstats()
        if self.lib.dn_cuda_stats_kind(self.s.gpu, kind, ctypes.byref(s)) != 0:
            raise RuntimeError("dn_cuda_stats_kind failed: %s" % self.lib.dn_cuda_last_error().decode())
        return {k: int(getattr(s, k)) for k, _ in L.DNstats._fields_}

    def reset_stats(self):
        self.lib.DN_reset_stats(self.ptr)

    def export_lighting(self):
        n = self.lib.DN_export_lighting(self.ptr, None, None, None, 0)
        idx = np.empty(n, np.uint32)
        diff = np.empty((n, 3), np.float32)
        spec = np.empty((n, 3), np.float32)
        if n:
            got = self.lib.DN_export_lighting(self.ptr, idx.ctypes.data_as(POINTER(c_uint32)),
                                              diff.ctypes.data_as(POINTER(c_float)), spec.ctypes.data_as(POINTER(c_float)), n)
            assert got == n
        return idx, diff, spec

    def export_tiles(self):
        n = self.num_tiles
        st = np.empty(n, np.uint8)
        vis = np.empty(n, np.uint8)
        lu = np.empty(n, np.uint32)
        ns = np.empty(n, np.uint32)
        ok = self.lib.DN_export_tiles(self.ptr, st.ctypes.data_as(POINTER(c_uint8)), vis.ctypes.data_as(POINTER(c_uint8)),
                                      lu.ctypes.data_as(POINTER(c_uint32)), ns.ctypes.data_as(POINTER(c_uint32)))
        if not ok:
            raise RuntimeError("DN_export_tiles failed: %s" % self.lib.dn_cuda_last_error().decode())
        return st, vis, lu, ns

    def set_residency(self, mode):
        """DN_set_residency: "keep" (default) or "lru" (the reference's fixed voxel buffer with least-recently-used
        unloading); before the volume's first sync"""
        m = {"keep": 0, "lru": 1}[mode]
        if not self.lib.DN_set_residency(self.ptr, m):
            raise RuntimeError("DN_set_residency(%s) failed" % mode)

    def residency_nodes(self):
        """DN_RESIDENCY_LRU: (buffer size in voxels, node sizes, first voxels, owning tiles or -1)"""
        cap = c_size_t(0)
        n = self.lib.DN_residency_nodes(self.ptr, ctypes.byref(cap), None, None, None, 0)
        sizes = np.zeros(max(n, 1), np.uint32)
        starts = np.zeros(max(n, 1), np.uint64)
        tiles = np.zeros(max(n, 1), np.int64)
        self.lib.DN_residency_nodes(self.ptr, ctypes.byref(cap), sizes.ctypes.data_as(POINTER(c_uint32)),
                                    starts.ctypes.data_as(POINTER(c_uint64)), tiles.ctypes.data_as(POINTER(c_int64)), n)
        return int(cap.value), sizes[:n], starts[:n], tiles[:n]

    def export_requests(self):
        n = self.lib.DN_export_requests(self.ptr, None, 0)
        out = np.empty(max(n, 1), np.uint32)
        if n:
            self.lib.DN_export_requests(self.ptr, out.ctypes.data_as(POINTER(c_uint32)), n)
        return out[:n]

    def stream(self):
        return self.lib.dn_cuda_stream(self.s.gpu)

    # ---- scenes
    def palette(self, seed, n_materials=16, n_emissive=2, albedo_lo=0.1, albedo_hi=0.9, spec_max=0.5):
        self.lib.dn_scene_palette(self.ptr, seed, n_materials, n_emissive, albedo_lo, albedo_hi, spec_max)

    def terrain(self, seed, mean_frac, amp_frac, n_materials=16, n_emissive=2):
        self.lib.dn_scene_terrain(self.ptr, seed, mean_frac, amp_frac, n_materials, n_emissive)

    def shapes(self, seed, n, min_size, max_size, n_materials=14, y_lo=0.0, y_hi=0.5):
        self.lib.dn_scene_shapes(self.ptr, seed, n, min_size, max_size, n_materials, y_lo, y_hi)

    # shapes (include/DoonEngine/voxelShapes.h); voxel = (material, normal, albedo), orient = Euler degrees
    _SHAPES = {"sphere": 0, "box": 1, "rounded_box": 2, "torus": 3, "ellipsoid": 4, "cylinder": 5, "cone": 6,
               "pyramid": 7}

    def shape(self, kind, voxel, c, v=(0.0, 0.0, 0.0), a=0.0, b=0.0, orient=(0.0, 0.0, 0.0), flip=False, func=None,
              user=None):
        """DN_shape_<kind>: sphere (c, a=r), box (c, v=len), rounded_box (c, v=len, a=r), torus (c, a=ra, b=rb),
        ellipsoid (c, v=radii), cylinder (c, a=r, b=h), cone (base c, a=r, b=h), pyramid (base c, v=len);
        func: a C VoxelTransformFunc pointer (or None)"""
        vox = L.DNvoxel()
        vox.material = voxel[0]
        vox.normal = L.DNvec3(*voxel[1])
        vox.albedo = L.DNcolor(*voxel[2])
        q = self.lib.DN_quaternion_from_euler(L.DNvec3(*orient))
        cv, vv = L.DNvec3(*c), L.DNvec3(*v)
        k = kind if isinstance(kind, int) else self._SHAPES[kind]
        f = self.lib
        args = {0: (f.DN_shape_sphere, (cv, a)), 1: (f.DN_shape_box, (cv, vv)), 2: (f.DN_shape_rounded_box, (cv, vv, a)),
                3: (f.DN_shape_torus, (cv, a, b)), 4: (f.DN_shape_ellipsoid, (cv, vv)),
                5: (f.DN_shape_cylinder, (cv, a, b)), 6: (f.DN_shape_cone, (cv, a, b)), 7: (f.DN_shape_pyramid, (cv, vv))}
        fn, rest = args[k]
        fn(self.ptr, vox, bool(flip), *rest, q, func, user)

    def export_chunk(self, tile):
        """The device record of a loaded tile (dn_cuda_export_chunk): dict of mask (16 words), partial (3),
        nvox, pos, voxBase, matSet (8 words) and words (nvox x 2: normal word, linear albedo word), or None
        when the tile has no record"""
        rec = np.zeros(24, np.uint32)
        mats = np.zeros(8, np.uint32)
        words = np.zeros(1024, np.uint32)
        rc = self.lib.dn_cuda_export_chunk(self.s.gpu, int(tile), rec.ctypes.data, mats.ctypes.data, words.ctypes.data)
        if rc != 0:
            return None
        n = int(rec[19])
        return {"mask": rec[:16].copy(), "partial": rec[16:19].copy(), "nvox": n, "pos": rec[20:23].view(np.int32).copy(),
                "voxBase": int(rec[23]), "matSet": mats, "words": words[: 2 * n].reshape(n, 2).copy()}

    def cpu_chunk(self, tile):
        """The CPU map's chunk of a tile (a DNchunk), or None when the tile has none"""
        h = self.s.map[int(tile)]
        return self.s.chunks[h.chunkIndex] if h.flag else None

    def export_voxels(self):
        """(normal words, albedo words, tile flags) of the CPU map, dense"""
        sx, sy, sz = self.map_size
        n = 512 * sx * sy * sz
        nw = np.zeros(n, np.uint32)
        aw = np.zeros(n, np.uint32)
        tf = np.zeros(sx * sy * sz, np.uint8)
        self.lib.DN_export_voxels(self.ptr, nw.ctypes.data, aw.ctypes.data, tf.ctypes.data)
        return nw, aw, tf

    def camera(self, fx, fy, fz, pitch, yaw, fov=90.0):
        self.lib.dn_scene_camera(self.ptr, fx, fy, fz, pitch, yaw, fov)


class Batch:
    """A DNbatch: frames of many volumes as batched kernels (DN_batch_*)."""

    def __init__(self, volumes=()):
        self.lib = L.load()
        self.ptr = self.lib.DN_batch_create()
        if not self.ptr:
            raise RuntimeError("DN_batch_create failed: %s" % self.lib.dn_cuda_last_error().decode())
        self.members = []
        for v in volumes:
            self.add(v)

    def add(self, vol):
        if not self.lib.DN_batch_add(self.ptr, vol.ptr):
            raise RuntimeError("DN_batch_add failed: %s" % self.lib.dn_cuda_last_error().decode())
        self.members.append(vol)

    def remove(self, vol):
        if not self.lib.DN_batch_remove(self.ptr, vol.ptr):
            raise RuntimeError("DN_batch_remove failed")
        self.members.remove(vol)

    def close(self):
        if self.ptr:
            self.lib.DN_batch_destroy(self.ptr)
            self.ptr = None
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def item(vol, image=None, view=None, proj=None, sync=None, light=None, raster=None):
        """One DNbatchItem: draw into image with (view, proj) composed with raster=(colour, depth) Textures;
        sync=(op, split); light=(numDiffuse, maxDiffuse, time)."""
        it = L.DNbatchItem()
        it.vol = vol.ptr
        ph = 0
        if image is not None:
            ph |= L.PHASE_DRAW
            it.output = image.ptr
            it.view, it.projection = view, proj
            it.rasterColorTexture, it.rasterDepthTexture = _raster_handles(raster)
        if sync is not None:
            ph |= L.PHASE_SYNC
            it.op, it.lightingSplit = sync
        if light is not None:
            ph |= L.PHASE_LIGHT
            it.numDiffuseSamples, it.maxDiffuseSamples, it.time = light
        it.phases = ph
        return it

    def run(self, items):
        arr = (L.DNbatchItem * len(items))(*items)
        if not self.lib.DN_batch_run(self.ptr, arr, len(items)):
            raise RuntimeError("DN_batch_run failed: %s" % self.lib.dn_cuda_last_error().decode())

    def finish(self):
        return bool(self.lib.DN_batch_finish(self.ptr))

    def stats(self):
        s = L.DNstats()
        if not self.lib.DN_batch_get_stats(self.ptr, byref(s)):
            raise RuntimeError("DN_batch_get_stats failed: %s" % self.lib.dn_cuda_last_error().decode())
        return {k: int(getattr(s, k)) for k, _ in L.DNstats._fields_}

    def reset_stats(self):
        self.lib.DN_batch_reset_stats(self.ptr)

    def autotune(self):
        if not self.lib.DN_batch_autotune(self.ptr):
            raise RuntimeError("DN_batch_autotune failed: %s" % self.lib.dn_cuda_last_error().decode())
        return self.tuning()

    def _gpu(self):
        # struct DNbatch starts with its struct DNgpuBatch pointer
        return ctypes.cast(self.ptr, POINTER(c_void_p))[0]

    def tuning(self):
        t = L.DnBatchTuning()
        if self.lib.dn_cuda_batch_get_tuning(self._gpu(), byref(t)) != 0:
            raise RuntimeError("dn_cuda_batch_get_tuning failed")
        return {k: int(getattr(t, k)) for k, _ in L.DnBatchTuning._fields_}

    def set_tuning(self, streamBatch=None, blocksPerSM=None, useGraph=None, kernel=None, poolRays=None,
                   diffuseBatch=None):
        cur = self.tuning()
        t = L.DnBatchTuning(streamBatch if streamBatch is not None else cur["streamBatch"],
                            blocksPerSM if blocksPerSM is not None else cur["blocksPerSM"],
                            useGraph if useGraph is not None else cur["useGraph"],
                            kernel if kernel is not None else cur["kernel"],
                            poolRays if poolRays is not None else cur["poolRays"],
                            diffuseBatch if diffuseBatch is not None else cur["diffuseBatch"])
        if self.lib.dn_cuda_batch_set_tuning(self._gpu(), byref(t)) != 0:
            raise RuntimeError("dn_cuda_batch_set_tuning failed: %s" % self.lib.dn_cuda_last_error().decode())

    def stream(self):
        return self.lib.dn_cuda_batch_stream(self._gpu())


class Server:
    """A DNserver (include/DoonEngine/serve.h): requests on many volumes served in batched ticks by the
    server's own thread, with whole-volume eviction under a device budget."""

    def __init__(self, volumes, budget_bytes=0, max_volumes_per_tick=0, ticks_in_flight=2):
        self.lib = L.load()
        cfg = L.DNserveConfig(budget_bytes, max_volumes_per_tick, ticks_in_flight)
        self.ptr = self.lib.DN_server_create(byref(cfg))
        if not self.ptr:
            raise RuntimeError("DN_server_create failed: %s" % self.lib.dn_cuda_last_error().decode())
        self.volumes = list(volumes)
        for v in self.volumes:
            if self.lib.DN_server_add_volume(self.ptr, v.ptr) < 0:
                raise RuntimeError("DN_server_add_volume failed")
        self._keep = []

    def start(self):
        if not self.lib.DN_server_start(self.ptr):
            raise RuntimeError("DN_server_start failed")

    @staticmethod
    def draw_request(volume, image, view, proj, user=0, raster=None):
        r = L.DNrequest()
        r.kind, r.volume, r.output, r.view, r.projection, r.user = L.REQUEST_DRAW, volume, image.ptr, view, proj, user
        r.rasterColorTexture, r.rasterDepthTexture = _raster_handles(raster)
        return r

    @staticmethod
    def relight_request(volume, num_diffuse=1, max_diffuse=1000, time=0.0, user=0):
        r = L.DNrequest()
        r.kind, r.volume, r.user = L.REQUEST_RELIGHT, volume, user
        r.numDiffuseSamples, r.maxDiffuseSamples, r.time = num_diffuse, max_diffuse, time
        return r

    def edit_request(self, volume, edits, user=0):
        """edits: iterable of (mapPos, chunkPos, material, normal, albedo, remove)."""
        arr = (L.DNvoxelEdit * max(1, len(edits)))()
        for i, (mp, cp, mat, nrm, alb, rem) in enumerate(edits):
            arr[i].mapPos, arr[i].chunkPos = L.DNivec3(*mp), L.DNivec3(*cp)
            arr[i].voxel = L.DNvoxel(mat, L.DNvec3(*nrm), L.DNcolor(*alb))
            arr[i].remove = 1 if rem else 0
        self._keep.append(arr)
        r = L.DNrequest()
        r.kind, r.volume, r.user = L.REQUEST_EDIT, volume, user
        r.edits, r.numEdits = ctypes.cast(arr, POINTER(L.DNvoxelEdit)), len(edits)
        return r

    def submit(self, req):
        rid = self.lib.DN_server_submit(self.ptr, byref(req))
        if not rid:
            raise RuntimeError("DN_server_submit rejected the request")
        return rid

    def replay(self, reqs, offsets):
        arr = (L.DNrequest * len(reqs))(*reqs)
        off = np.ascontiguousarray(offsets, np.float64)
        return self.lib.DN_server_replay(self.ptr, arr, off.ctypes.data_as(POINTER(ctypes.c_double)), len(reqs))

    def drain(self, timeout=600.0):
        return bool(self.lib.DN_server_drain(self.ptr, timeout))

    def poll(self, cap=1 << 16):
        out = []
        buf = (L.DNcompletion * cap)()
        while True:
            n = self.lib.DN_server_poll(self.ptr, buf, cap)
            out += [dict(id=buf[i].id, user=buf[i].user or 0, kind=buf[i].kind, volume=buf[i].volume,
                         arrival=buf[i].arrival, admitted=buf[i].admitted, finished=buf[i].finished, ok=buf[i].ok)
                    for i in range(n)]
            if n < cap:
                return out

    def stats(self):
        st = L.DNserveStats()
        self.lib.DN_server_get_stats(self.ptr, byref(st))
        return {k: (float if t is c_double else int)(getattr(st, k)) for k, t in L.DNserveStats._fields_}

    def batch_stats(self):
        s = L.DNstats()
        self.lib.DN_batch_get_stats(self.lib.DN_server_batch(self.ptr), byref(s))
        return {k: int(getattr(s, k)) for k, _ in L.DNstats._fields_}

    def close(self):
        if self.ptr:
            self.lib.DN_server_destroy(self.ptr)
            self.ptr = None
            self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
