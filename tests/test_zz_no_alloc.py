"""dn_cuda_light_noalloc: the lighting update without any allocation, against dn_cuda_light.

Some callers cannot let the lighting pass allocate device memory while a frame is in flight: a render
loop that runs under a fixed device-memory budget, or a host engine whose own allocator hands out all
device memory and forbids ad-hoc cudaMalloc / cudaFree.  dn_cuda_light keeps its per-request scratch in
the volume and grows it with cudaMalloc; dn_cuda_light_noalloc keeps it in a fixed array inside the
library instead.  These tests drive two identical volumes through the same frames and, for two calls in
a row, light one with each entry point through the C ABI: the lighting must agree within the parity
tolerance, and the library's allocation count and the volume's device footprint must not change across
the call.  The limit is checked at the boundary (a list of exactly the limit is lit, one group more is
not) and at the real size of the array.  This file is collected last so that a stop-at-first-failure run
has already run every other test.
"""
import ctypes
import math

import numpy as np
import pytest

import doonengine_gb300 as dn
from doonengine_gb300 import _lib as L, configs
from parity_util import lighting_close

pytestmark = pytest.mark.gpu

DN_CUDA_ERR_CAPACITY = 6


def light_params(vol_s, time):
    """The per-launch parameters DN_update_lighting derives from the volume (voxel.c:883-952)."""
    p = L.DnLightParams()
    x, y, z = (np.float32(c) for c in vol_s.sunDir.tolist())
    ln = np.sqrt(np.float32(np.float32(np.float32(x * x) + np.float32(y * y)) + np.float32(z * z)))
    inv = np.float32(np.float32(1.0) / ln)
    p.sunDir[:] = [float(np.float32(x * inv)), float(np.float32(y * inv)), float(np.float32(z * inv))]
    p.sunStrength[:] = vol_s.sunStrength.tolist()
    p.ambient[:] = vol_s.ambientLightStrength.tolist()
    p.camPos[:] = vol_s.camPos.tolist()
    p.skyBot[:] = vol_s.skyGradientBot.tolist()
    p.skyTop[:] = vol_s.skyGradientTop.tolist()
    p.shadowSoftness = vol_s.shadowSoftness
    p.time = time
    p.emissiveStrength = vol_s.emissiveStrength
    p.numDiffuse, p.maxDiffuse = 1, 1000
    p.diffuseBounceLimit = vol_s.diffuseBounceLimit
    p.specBounceLimit = vol_s.specBounceLimit
    K = min(64, max(1, vol_s.numDirectRays))
    p.K = K
    p.rngMode = vol_s.rngMode
    p.mapId = vol_s.mapId
    ga = math.pi * (3.0 - math.sqrt(5.0))
    for k in range(K):
        yk = 1.0 - 2.0 * k / (K - 1) if K > 1 else 1.0
        r = math.sqrt(max(0.0, 1.0 - yk * yk))
        p.spherePts[k][:] = [math.cos(ga * k) * r, yk, math.sin(ga * k) * r]
    return p


def frame(vol, img, view, proj, t):
    vol.draw(img, view, proj)
    vol.sync()
    vol.update_lighting(1, 1000, t)
    assert vol.finish()


def test_noalloc_matches_regular_entry_point(gpu_ready):
    lib = dn.load()
    a, cfg = configs.build_volume("tiny")
    b, _ = configs.build_volume("tiny")
    W, H = cfg["res"]
    img = dn.Image(W, H)
    view, proj = a.view_proj(H / W)
    try:
        for f in range(3):           # identical warm-up: chunks load and become visible on both
            for v in (a, b):
                frame(v, img, view, proj, 1.5 + f)
        lit_total = 0
        for call in range(2):        # two calls in a row of each entry point
            for v in (a, b):
                v.draw(img, view, proj)
                v.sync()
            p = light_params(a.s, 4.5 + call)
            mats_a = ctypes.cast(a.s.materials, ctypes.c_void_p)
            mats_b = ctypes.cast(b.s.materials, ctypes.c_void_p)
            assert lib.dn_cuda_light(a.s.gpu, ctypes.byref(p), mats_a) == 0, lib.dn_cuda_last_error()
            allocs, footprint = lib.dn_cuda_alloc_count(), lib.dn_cuda_map_footprint(b.s.gpu)
            rc = lib.dn_cuda_light_noalloc(b.s.gpu, ctypes.byref(p), mats_b)
            assert rc == 0, lib.dn_cuda_last_error()
            assert a.finish() and b.finish()
            assert lib.dn_cuda_alloc_count() == allocs, "the no-allocation entry point allocated"
            assert lib.dn_cuda_map_footprint(b.s.gpu) == footprint
            ia, da, sa = a.export_lighting()
            ib, db, sb = b.export_lighting()
            assert np.array_equal(ia, ib)
            assert lighting_close(da, db).all() and lighting_close(sa, sb).all()
            lit_total += len(ia)
        assert lit_total > 0
    finally:
        img.close()
        a.close()
        b.close()


def finish_rc(lib, vol):
    n = ctypes.c_uint64()
    return lib.dn_cuda_finish(vol.s.gpu, ctypes.byref(n))


def test_noalloc_limit_boundary(gpu_ready):
    """A request list of exactly the limit is lit like dn_cuda_light; one group above it is not lit at all,
    leaves the volume unchanged and is reported by the next finish; the call itself never fails."""
    lib = dn.load()
    a, cfg = configs.build_volume("tiny")
    b, _ = configs.build_volume("tiny")
    W, H = cfg["res"]
    img = dn.Image(W, H)
    view, proj = a.view_proj(H / W)
    try:
        for f in range(3):
            for v in (a, b):
                frame(v, img, view, proj, 1.5 + f)
        for call, over in enumerate((False, True)):
            for v in (a, b):
                v.draw(img, view, proj)
                v.sync()
                assert v.finish()
            n = b.s.numLightingRequests
            assert n > 1
            p = light_params(a.s, 4.5 + call)
            before = b.export_lighting() + (b.export_tiles()[3],)
            lib.dn_cuda_light_noalloc_set_limit(n - 1 if over else n)
            try:
                rc = lib.dn_cuda_light_noalloc(b.s.gpu, ctypes.byref(p), ctypes.cast(b.s.materials, ctypes.c_void_p))
                assert rc == 0, lib.dn_cuda_last_error()
                frc = finish_rc(lib, b)
            finally:
                lib.dn_cuda_light_noalloc_set_limit(0)
            if over:
                assert frc == DN_CUDA_ERR_CAPACITY
                assert b"exceeded the fixed scratch" in lib.dn_cuda_last_error()
                after = b.export_lighting() + (b.export_tiles()[3],)
                for x, y in zip(before, after):
                    assert np.array_equal(x, y)
                assert finish_rc(lib, b) == 0            # the flag is reported once
            else:
                assert frc == 0, lib.dn_cuda_last_error()
                assert lib.dn_cuda_light(a.s.gpu, ctypes.byref(p), ctypes.cast(a.s.materials, ctypes.c_void_p)) == 0
                assert a.finish()
                ia, da, sa = a.export_lighting()
                ib, db, sb = b.export_lighting()
                assert np.array_equal(ia, ib)
                assert lighting_close(da, db).all() and lighting_close(sa, sb).all()
    finally:
        img.close()
        a.close()
        b.close()


def test_noalloc_rejects_request_lists_beyond_its_scratch(gpu_ready):
    lib = dn.load()
    vol, cfg = configs.build_volume("large")
    W, H = 1280, 720
    img = dn.Image(W, H)
    view, proj = vol.view_proj(H / W)
    try:
        for f in range(9):
            frame(vol, img, view, proj, 1.0 + f)
        vol.draw(img, view, proj)
        vol.sync()
        assert vol.finish()
        assert vol.s.numLightingRequests > 8192
        p = light_params(vol.s, 9.0)
        allocs = lib.dn_cuda_alloc_count()
        rc = lib.dn_cuda_light_noalloc(vol.s.gpu, ctypes.byref(p), ctypes.cast(vol.s.materials, ctypes.c_void_p))
        assert rc == 0, lib.dn_cuda_last_error()
        assert finish_rc(lib, vol) == DN_CUDA_ERR_CAPACITY
        assert b"exceeded the fixed scratch of 8192 groups" in lib.dn_cuda_last_error()
        assert lib.dn_cuda_alloc_count() == allocs
    finally:
        img.close()
        vol.close()
