"""Shape functions (include/DoonEngine/voxelShapes.h) on the CPU: the oracle and the product's host half
against goldens made by the reference's own voxelShapes.c (no GPU).

Bar: bit-identical maps (every voxel's normal and albedo words, every tile's chunk flag) and matrices.
"""
import numpy as np
import pytest

import shape_util as S

MAP = (6, 4, 6)


@pytest.mark.parametrize("name", S.SCRIPTS)
def test_product_matrices_match_reference(name):
    """quaternion from Euler angles, rotation matrix, translate * rotation and its inverse (the cone's
    at its apex) -- the product's dn_math against the reference's math header"""
    ops, mats = S.script(S.goldens(), name)
    for k, o in enumerate(ops):
        got = S.product_matrices(o)
        bad = np.where(got.view(np.uint32) != mats[k].view(np.uint32))[0]
        assert len(bad) == 0, "%s op %d (kind %d): matrix entries %s differ: %s vs %s" % (
            name, k, o["kind"], bad[:6], got[bad[:6]], mats[k][bad[:6]])


@pytest.mark.parametrize("name", ["bowl", "kinds"])
def test_oracle_matches_reference(name):
    g = S.goldens()
    ops, mats = S.script(g, name)
    got = S.run_oracle(MAP, ops, mats)
    S.same_map(got, (g[name + "_normal"], g[name + "_albedo"], g[name + "_tiles"]), "oracle, script " + name)


@pytest.mark.parametrize("name", S.SCRIPTS)
def test_product_host_half_matches_reference(name):
    """the oracle's evaluated voxels applied by the product's host half (dn_shape_apply), the transform
    function included"""
    g = S.goldens()
    ops, mats = S.script(g, name)
    got = S.run_product(MAP, ops, host_apply_only=True, mats=mats)
    S.same_map(got, (g[name + "_normal"], g[name + "_albedo"], g[name + "_tiles"]), "host half, script " + name)


def test_goldens_cover_the_cases():
    """every kind, placements and removals with and without flipped normals, a transform function, a
    shape outside the map"""
    g = S.goldens()
    ops = np.concatenate([S.script(g, n)[0] for n in S.SCRIPTS])
    assert set(ops["kind"].tolist()) == set(range(8))
    rem = ops[ops["material"] == 255]
    assert (rem["flip"] == 1).any() and (rem["flip"] == 0).any()
    assert (ops["transform"] == 1).sum() > 10
    assert (ops["c"] < -30).all(axis=1).any()
