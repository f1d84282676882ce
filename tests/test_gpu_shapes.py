"""Shape functions (include/DoonEngine/voxelShapes.h) with the per-voxel evaluation on the GPU
(k_shape_count / k_shape_write) against the reference's goldens and the CPU oracle.

Bar: bit-identical maps -- every voxel's normal and albedo words and every tile's chunk flag.
"""
import numpy as np
import pytest

import shape_util as S
import doonengine_gb300 as dn

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", S.SCRIPTS)
def test_shapes_match_reference(gpu_ready, name):
    g = S.goldens()
    ops, _ = S.script(g, name)
    before = dn.load().dn_cuda_launch_count()
    got = S.run_product(tuple(int(x) for x in g["map"]), ops)
    S.same_map(got, (g[name + "_normal"], g[name + "_albedo"], g[name + "_tiles"]), "GPU shapes, script " + name)
    # the evaluation ran on the device: two launches per shape that covers a chunk
    assert dn.load().dn_cuda_launch_count() - before >= len(ops)


def random_script(rng, map_size, n):
    X, Y, Z = (8 * s for s in map_size)
    ops = np.zeros(n, S.OP)
    for k in range(n):
        o = ops[k]
        o["kind"] = rng.integers(0, 8)
        o["c"] = np.round(rng.uniform((-10, -10, -10), (X + 10, Y + 10, Z + 10)) * 4) / 4
        o["v"] = np.round(rng.uniform(3.0, 30.0, 3) * 4) / 4
        o["a"] = np.round(rng.uniform(3.0, 30.0) * 4) / 4
        o["b"] = np.round(rng.uniform(2.0, 20.0) * 4) / 4
        if o["kind"] == 3:
            o["b"] = min(o["b"], o["a"] - 1.0)
        o["euler"] = rng.integers(0, 360, 3)
        removal = rng.random() < 0.3
        o["material"] = 255 if removal else rng.integers(0, 16)
        o["flip"] = int(removal and rng.random() < 0.7)
        o["albedo"] = rng.integers(0, 256, 3)
        o["normal"] = (0.0, 1.0, 0.0)
    return ops


def test_large_random_shapes_match_oracle(gpu_ready):
    """large shapes (up to ~60 voxels across) on a 16x8x16-chunk map, against the CPU oracle"""
    rng = np.random.default_rng(77)
    map_size = (16, 8, 16)
    ops = random_script(rng, map_size, 24)
    mats = np.stack([S.product_matrices(o) for o in ops])
    want = S.run_oracle(map_size, ops, mats)
    got = S.run_product(map_size, ops)
    S.same_map(got, want, "GPU shapes vs oracle")
    assert (got[0] >> 24 != 255).sum() > 10000


def test_shapes_on_a_device_volume_reach_the_gpu_map(gpu_ready):
    """on a device volume the edits are ordinary CPU-map edits: the next DN_sync_gpu uploads them and a
    draw sees the shape"""
    dn.init()
    vol = dn.Volume((4, 4, 4), 64)
    img = dn.Image(64, 48, on_device=True)
    try:
        vol.set_material(1, opacity=1.0)     # materials start zeroed (transparent), as in the reference
        vol.shape("sphere", (1, (0.0, 1.0, 0.0), (200, 50, 50)), (16.25, 16.5, 16.75), a=9.0)
        vol.camera(0.5, 0.5, -0.6, 0.0, 0.0)
        v, p = vol.view_proj(48 / 64)
        for _ in range(2):
            vol.draw(img, v, p)
            vol.sync(dn.DN_READ_WRITE, 1)
        vol.draw(img, v, p)
        assert vol.finish()
        hit = img.numpy()[1]
        assert (hit != 0xFFFFFFFF).sum() > 100
    finally:
        img.close()
        vol.close()
