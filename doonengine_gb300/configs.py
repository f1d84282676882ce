"""Seeded synthetic workloads (the reference publishes no benchmark data; these stand in for its
scenes with the shapes and sizes of the benchmark configurations).

* ``small``  -- 16x16x16 chunks (128^3 voxels), value-noise heightfield with about 35% of the chunks
  non-empty, 16 materials (2 emissive), specular U[0,0.5], one lighting update with 1 diffuse sample and
  K=16 direct / specular rays, then a 640x360 draw.
* ``large``  -- 64x32x64 chunks (512x256x512 voxels), heightfield plus 2000 seeded boxes and spheres of
  3-10 voxels (about 15% of chunks non-empty), 1920x1080 draw from a fixed camera, 1 diffuse sample per voxel per
  frame, K=32 direct / specular rays, accumulated over 64 frames.
"""
from .volume import Volume

CONFIGS = {
    "small": dict(map=(16, 16, 16), seed=1, mean=0.32, amp=0.16, shapes=0, res=(640, 360), K=16,
                  frames=1, cam=(0.1, 0.62, 0.1, 32.0, 42.0)),
    "large": dict(map=(64, 32, 64), seed=2, mean=0.06, amp=0.04, shapes=2000, shape_max=10, res=(1920, 1080), K=32,
                  frames=64, cam=(0.08, 0.42, 0.08, 24.0, 44.0)),
    # parity-test sizes: the same recipe scaled down
    "tiny": dict(map=(6, 5, 7), seed=3, mean=0.3, amp=0.2, shapes=6, res=(96, 64), K=8,
                 frames=3, cam=(0.05, 0.8, 0.1, 35.0, 40.0)),
    "medium": dict(map=(24, 12, 24), seed=4, mean=0.2, amp=0.12, shapes=120, res=(320, 180), K=16,
                   frames=4, cam=(0.1, 0.6, 0.1, 28.0, 43.0)),
}


def build_volume(name, cpu_only=False, **over):
    """Create and fill a volume for configuration ``name``; returns (volume, config dict)."""
    cfg = dict(CONFIGS[name])
    cfg.update(over)
    sx, sy, sz = cfg["map"]
    vol = Volume((sx, sy, sz), min_chunks=cfg.get("min_chunks", max(64, sx * sy * sz // 4)), cpu_only=cpu_only)
    seed = cfg["seed"]
    vol.palette(seed, 16, 2, 0.1, 0.9, 0.5)
    vol.terrain(seed, cfg["mean"], cfg["amp"], 16, 2)
    if cfg["shapes"]:
        vol.shapes(seed, cfg["shapes"], cfg.get("shape_min", 3), cfg.get("shape_max", 24), 14, 0.05, 0.5)
    fx, fy, fz, pitch, yaw = cfg["cam"]
    vol.camera(fx, fy, fz, pitch, yaw, 90.0)
    vol.s.numDirectRays = cfg["K"]
    vol.s.emissiveStrength = 5.0
    vol.s.sunDir.x, vol.s.sunDir.y, vol.s.sunDir.z = 0.4, 1.0, 0.25
    return vol, cfg


RESOLUTIONS = ((320, 180), (640, 360), (1280, 720), (1920, 1080))


def batched_specs(n=64, seed=7, dim_lo=8, dim_hi=64, res=RESOLUTIONS):
    """The batched workload: n independent maps with chunk dimensions uniform in [dim_lo, dim_hi] per axis,
    non-empty chunk fraction uniform in [0.05, 0.5], each with its own seeded camera and a resolution drawn
    from ``res``; K=16 direct / specular rays.  Returns a list of per-map overrides for ``build_volume``."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(x) for x in rng.integers(dim_lo, dim_hi + 1, size=3))
        frac = float(rng.uniform(0.05, 0.5))
        r = res[int(rng.integers(len(res)))]
        cam = (float(rng.uniform(0.05, 0.3)), float(rng.uniform(0.6, 0.9)), float(rng.uniform(0.05, 0.3)),
               float(rng.uniform(20.0, 40.0)), float(rng.uniform(30.0, 60.0)))
        out.append(dict(map=dims, seed=int(seed * 1000 + i), mean=frac, amp=frac * 0.5, shapes=0,
                        res=tuple(r), K=16, cam=cam))
    return out


def serving_specs(n=256, seed=11, lo=(8, 8, 8), hi=(96, 32, 96), res=RESOLUTIONS):
    """The serving workload's maps: chunk dimensions log-uniform per axis between lo and hi (8^3 to
    96x32x96 chunks), non-empty chunk fraction uniform in [0.05, 0.5], own seeded camera, K=16."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(round(float(np.exp(rng.uniform(np.log(a), np.log(b)))))) for a, b in zip(lo, hi))
        frac = float(rng.uniform(0.05, 0.5))
        cam = (float(rng.uniform(0.05, 0.3)), float(rng.uniform(0.6, 0.9)), float(rng.uniform(0.05, 0.3)),
               float(rng.uniform(20.0, 40.0)), float(rng.uniform(30.0, 60.0)))
        out.append(dict(map=dims, seed=int(seed * 1000 + i), mean=frac, amp=frac * 0.5, shapes=0,
                        res=tuple(res[int(rng.integers(len(res)))]), K=16, cam=cam))
    return out
