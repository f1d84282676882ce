"""Side-by-side runner: the CUDA path (through libdoonengine.so's DN_* C API) and the CPU oracle on the same
seeded volume, frame by frame, in the reference's frame order (draw, sync, lighting; main.c:503-505)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import doonengine_gb300 as dn                      # noqa: E402
from doonengine_gb300 import _lib, configs         # noqa: E402
from oracle import oracle as O                     # noqa: E402

REL_TOL = 1e-4      # per-voxel FP32 lighting, relative (absolute below 1e-6)
COLOR_TOL = 2e-6    # draw colour: pow() of CUDA vs the host C library may differ in the last place


def draw_mats(vol, view, proj):
    lib = dn.load()
    iv, icv, ip = _lib.DNmat4(), _lib.DNmat4(), _lib.DNmat4()
    lib.DN_draw_matrices(view, proj, iv, icv, ip)
    return iv, icv, ip


def lighting_close(a, b, rel=REL_TOL, abs_=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) <= np.maximum(abs_, rel * np.maximum(np.abs(a), np.abs(b)))


def compare_lighting(vol, om, where=""):
    gi, gd, gs = vol.export_lighting()
    oi, od, os_ = om.export_lighting()
    assert len(gi) == len(oi), "%s: lighting row count gpu %d oracle %d" % (where, len(gi), len(oi))
    go = np.argsort(gi, kind="stable")
    oo = np.argsort(oi, kind="stable")
    assert np.array_equal(gi[go], oi[oo]), where + ": lit voxel sets differ"
    okd = lighting_close(gd[go], od[oo])
    oks = lighting_close(gs[go], os_[oo])
    bad = np.where(~(okd.all(1) & oks.all(1)))[0]
    assert len(bad) == 0, "%s: %d/%d voxels outside tolerance, first %s gpu %s/%s oracle %s/%s" % (
        where, len(bad), len(gi), gi[go][bad[0]], gd[go][bad[0]], gs[go][bad[0]], od[oo][bad[0]], os_[oo][bad[0]])
    return len(gi), int((gd[go] != od[oo]).any(1).sum() + (gs[go] != os_[oo]).any(1).sum())


def compare_tiles(vol, om, where=""):
    gst, gvis, glu, gns = vol.export_tiles()
    ost, ovis, olu, ons = om.export_tiles()
    assert np.array_equal(gst, ost), "%s: tile states differ at %s" % (where, np.where(gst != ost)[0][:8])
    assert np.array_equal(gvis, ovis), "%s: visible flags differ at %s" % (where, np.where(gvis != ovis)[0][:8])
    assert np.array_equal(glu, olu), "%s: lastUsed differs at %s" % (where, np.where(glu != olu)[0][:8])
    assert np.array_equal(gns, ons), "%s: sample counts differ at %s" % (where, np.where(gns != ons)[0][:8])


def compare_requests(vol, om, where=""):
    g = np.sort(vol.export_requests())
    o = np.sort(om.requests())
    assert np.array_equal(g, o), "%s: request lists differ (gpu %d, oracle %d)" % (where, len(g), len(o))
    return len(g)


def compare_draw(gpu, ora, where=""):
    gc, gh, gf = gpu
    oc, oh, of = ora
    assert np.array_equal(gh, oh), "%s: hit index differs at %d pixels, first %s" % (
        where, int((gh != oh).sum()), np.argwhere(gh != oh)[:3].tolist())
    assert np.array_equal(gf, of), "%s: face differs at %d pixels" % (where, int((gf != of).sum()))
    assert np.array_equal(gc[..., 3], oc[..., 3], equal_nan=True), "%s: depth differs" % where
    # the reference's sky gradient (mix parameter y*0.5+1) goes negative for upward rays and pow() of a
    # negative base is NaN on both sides: NaN positions must agree, the rest within tolerance
    gn, on = np.isnan(gc[..., :3]), np.isnan(oc[..., :3])
    assert np.array_equal(gn, on), "%s: NaN colour at %d differing pixels" % (where, int((gn != on).sum()))
    d = np.where(gn, 0.0, np.abs(gc[..., :3].astype(np.float64) - oc[..., :3]))
    tol = COLOR_TOL * np.maximum(1.0, np.where(on, 0.0, np.abs(oc[..., :3])))
    assert (d <= tol).all(), "%s: colour differs, max %g" % (where, d.max())


class Pair:
    """A product volume and an oracle map stepping in lock step."""

    def __init__(self, name, **over):
        dn.init()
        self.vol, self.cfg = configs.build_volume(name, **over)
        self.om = O.OracleMap(self.vol.map_size)
        self.W, self.H = self.cfg["res"]
        self.img = dn.Image(self.W, self.H, on_device=True)
        self.frame = 0

    def matrices(self):
        v, p = self.vol.view_proj(self.H / self.W)
        return v, p, draw_mats(self.vol, v, p)

    def draw(self, check=True, nthreads=0):
        v, p, (iv, icv, ip) = self.matrices()
        self.vol.draw(self.img, v, p)
        ora = self.om.draw(self.vol.s, iv, icv, ip, self.W, self.H, nthreads=nthreads)
        gpu = self.img.numpy()
        if check:
            compare_draw(gpu, ora, "frame %d draw" % self.frame)
        return gpu, ora

    def sync(self, op=2, split=1, check=True):
        self.om.sync(self.vol.s, op, split)
        self.vol.sync(op, split)
        if check:
            n = compare_requests(self.vol, self.om, "frame %d sync" % self.frame)
            compare_tiles(self.vol, self.om, "frame %d sync" % self.frame)
            return n
        return None

    def light(self, num_diffuse=1, max_diffuse=1000, time=None, check=True, nthreads=0):
        t = 1.25 + 0.5 * self.frame if time is None else time
        self.om.light(self.vol.s, num_diffuse, max_diffuse, t, nthreads=nthreads)
        self.vol.update_lighting(num_diffuse, max_diffuse, t)
        assert self.vol.finish(), dn.load().dn_cuda_last_error().decode()
        r = None
        if check:
            r = compare_lighting(self.vol, self.om, "frame %d lighting" % self.frame)
            compare_tiles(self.vol, self.om, "frame %d after lighting" % self.frame)
        self.frame += 1
        return r

    def step(self, **kw):
        self.draw()
        self.sync()
        return self.light(**kw)

    def close(self):
        self.img.close()
        self.vol.close()
        self.om.close()
