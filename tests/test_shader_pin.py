"""Pins the CPU oracle to the reference's own compute shaders.

tests/golden/make_shader_golden.py ran voxelDraw.comp and voxelLighting.comp (translated to C++ by
oracle/ref/glsl_to_cpp.py, executed per invocation by oracle/ref/pin_harness.cpp) on scenes built with the
reference's own edit API and packed by its own _DN_chunk_to_gpu.  Here the oracle runs the same scenes in
its reference-faithful modes -- sin-fract RNG (voxelLighting.comp:29-57), transparency state carried over
the rays of one invocation (voxelShared.comp:321-325), one jittered shadow ray per diffuse sample
(voxelLighting.comp:65-80, 260) and the shader's own 15-point sphere table (voxelLighting.comp:23) -- and
must reproduce the shaders' outputs bit for bit:
  * draw: RGBA (gamma-corrected colour and depth) of every pixel of the w/16 x h/16 dispatch and the
    visible flags it sets, for two cameras and two view modes, including transparent and refracting voxels;
  * lighting: the FP32 specular and diffuse light of every lit voxel, before quantisation, for two
    parameter sets with quantised lighting history and per-chunk sample counts (first-sample and
    random-direction paths).
Only the sine is not the GPU's: both sides use the oracle's deterministic sine.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "shader_goldens.npz"))
SCENES = sorted({k.split("_")[0] for k in G.files if k.startswith("s") and k[1].isdigit()})
INV255 = np.float32(0.00392156862)
INV65535 = np.float32(0.0000152590219)
SKY_BOT = [0.71, 0.85, 0.90]
SKY_TOP = [0.00, 0.45, 0.74]
SUN = [0.6, 0.6, 0.6]
AMB = [0.01, 0.01, 0.01]


def oracle_for(pre, vis_on):
    lib = O.load()
    size = tuple(int(x) for x in G[pre + "_size"])
    om = O.OracleMap(size)
    mapb = np.ascontiguousarray(G[pre + "_map"])
    chunks = np.ascontiguousarray(G[pre + "_chunks"])
    mats = np.ascontiguousarray(G[pre + "_materials"])
    state = np.where(mapb[:, 0] != 0, 2, 0).astype(np.uint8)
    vis = (state == 2).astype(np.uint8) if vis_on else np.zeros_like(state)
    lib.dno_import_state(om.ptr, mapb.ctypes.data, chunks.ctypes.data, mats.ctypes.data, state.ctypes.data,
                         vis.ctypes.data, 0)
    hist = G[pre + "_history"]
    diff = (hist[:, 1:4].astype(np.float32) * INV65535).astype(np.float32)
    spec = (hist[:, 4:7].astype(np.float32) * INV255).astype(np.float32)
    om.import_lighting(hist[:, 0], diff, spec)
    om.import_samples(np.ascontiguousarray(G[pre + "_samples"], np.uint32))
    return om, mats, size


@pytest.mark.parametrize("pre", SCENES)
def test_draw_matches_reference_shader(pre):
    lib = O.load()
    W, H = 64, 48
    cams = G[pre + "_cam_mats"]
    k = 0
    for ci in range(len(cams)):
        for vm in (0, 5):
            om, mats, size = oracle_for(pre, vis_on=False)
            p = O.DrawParams()
            for M, dst in zip(cams[ci], (p.invView, p.invCenteredView, p.invProj)):
                for c in range(4):
                    for r in range(4):
                        dst[c][r] = float(M[c * 4 + r])
            p.width, p.height, p.viewMode, p.truncate16 = W, H, vm, 1
            p.sunStrength[:], p.skyBot[:], p.skyTop[:] = SUN, SKY_BOT, SKY_TOP
            p.emissiveStrength = 1.0
            color = np.zeros((H * W, 4), np.float32)
            hit = np.zeros(H * W, np.uint32)
            face = np.zeros(H * W, np.uint8)
            lib.dno_draw(om.ptr, mats.ctypes.data, ctypes.byref(p), color.ctypes.data, hit.ctypes.data, face.ctypes.data, 1)
            want = G[pre + "_draw_rgba"][k].reshape(H * W, 4)
            assert (want[:, 3] > 0).sum() > 100
            same = (color == want) | (np.isnan(color) & np.isnan(want))
            assert same.all(), "%s camera %d mode %d: %d pixel values differ" % (pre, ci, vm, int((~same).sum()))
            st, vis, _, _ = om.export_tiles()
            assert np.array_equal(vis != 0, (G[pre + "_draw_flags"][k] & 4) != 0), (pre, ci, vm)
            om.close()
            k += 1


@pytest.mark.parametrize("pre", SCENES)
def test_lighting_matches_reference_shader(pre):
    lib = O.load()
    sphere = G["sphere15"]
    gidx = G[pre + "_light_gidx"]
    for j, (t, nd) in enumerate(G[pre + "_light_params"]):
        om, mats, size = oracle_for(pre, vis_on=True)
        om.set_requests(G[pre + "_requests"])
        p = O.LightParams()
        p.sunDir[:] = G[pre + "_light_sun"].tolist()
        p.sunStrength[:], p.ambient[:] = SUN, AMB
        p.camPos[:] = G[pre + "_light_cam"].tolist()
        p.skyBot[:], p.skyTop[:] = SKY_BOT, SKY_TOP
        p.shadowSoftness = 10.0
        p.time = float(t)
        p.emissiveStrength = 1.0
        p.numDiffuse, p.maxDiffuse, p.diffuseBounceLimit, p.specBounceLimit = int(nd), 1000, 5, 2
        p.K = 15
        p.flags = O.RNG_SIN | O.PERSIST_TRANSPARENCY | O.REFERENCE_SHADOW
        p.useSpherePoints = 1
        for k in range(15):
            p.spherePts[k][:] = sphere[k].tolist()
        lib.dno_light(om.ptr, mats.ctypes.data, ctypes.byref(p), 1)
        oi, od, os_ = om.export_lighting()
        valid = G[pre + "_light_valid"][j] != 0
        ref = {int(g): (G[pre + "_light_spec"][j][i], G[pre + "_light_diff"][j][i]) for i, g in enumerate(gidx) if valid[i]}
        assert len(ref) == len(oi) and len(ref) > 1000
        bad = 0
        for i in range(len(oi)):
            s, d = ref[int(oi[i])]
            if not (np.array_equal(s, os_[i]) and np.array_equal(d, od[i])):
                bad += 1
        assert bad == 0, "%s params %d: %d of %d voxels differ from the reference shader" % (pre, j, bad, len(oi))
        om.close()
