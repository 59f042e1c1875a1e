"""Closest-hit / occlusion parity of the GPU traversal against the oracle and
the reference's golden hits.  Bar: triangle ids bit-exact except rays the
oracle classifies as exact-t ties or edge-grazing (reported, not hidden);
hit distance within 1e-6 relative."""
import numpy as np
import pytest

from conftest import C1_HI, C1_LO, golden
from kagayaki_gb300 import Scene, scenes
from oracle import orc

pytestmark = pytest.mark.gpu

T_REL_TOL = 1e-6


def _compare(ids, t, oids, ot, flags):
    ok = flags == 0
    mism = ok & (ids != oids)
    assert mism.sum() == 0, f"{mism.sum()} unclassified id mismatches"
    hit = ok & (oids >= 0)
    rel = np.abs(t[hit] - ot[hit]) / ot[hit]
    assert rel.max() <= T_REL_TOL, rel.max()
    assert (t[ok & (oids < 0)] == np.float32(1e38)).all()
    return int((~ok).sum()), float(rel.max())


@pytest.fixture(scope="module")
def cornell():
    tris, mats, _ = scenes.cornell_box()
    s = Scene(tris, mats)
    s.build_bvh()
    yield s, tris
    s.close()


def test_bvh_is_valid(cornell):
    s, _ = cornell
    s.validate_bvh()
    assert s.bvh["n_wide_nodes"] >= 1


def test_c1_parity_rays_against_reference_golden(cornell):
    s, tris = cornell
    g = golden("c1_trace_ref.npz")
    rays = scenes.parity_rays(1 << 20, C1_LO, C1_HI, seed=1)
    ids, t, st = s.trace_closest(rays, with_stats=True)
    assert st["traversal_overflows"] == 0
    assert st["rays_closest"] == len(rays)
    oids, ot = orc.closest_brute(tris, rays)
    ref_ids = g["ids"].astype(np.int32)
    assert np.array_equal(oids, ref_ids)           # oracle pinned to the reference
    flags = orc.classify(tris, rays, oids, ot)
    n_flag, worst = _compare(ids, t, oids, ot, flags)
    assert n_flag < 100
    head = slice(0, 1 << 16)
    okh = flags[head] == 0
    relh = np.abs(t[head][okh & (ref_ids[head] >= 0)] - g["t_head"][okh & (ref_ids[head] >= 0)])
    assert (relh / g["t_head"][okh & (ref_ids[head] >= 0)]).max() <= T_REL_TOL


def test_icosphere_parity_against_reference_golden():
    g = golden("ico_trace_ref.npz")
    tris, mats, info = scenes.icosphere_field(n_meshes=2, subdiv=3, seed=5, box=6.0)
    rays = scenes.parity_rays(1 << 16, info["lo"], info["hi"], seed=3)
    with Scene(tris, mats) as s:
        s.build_bvh()
        s.validate_bvh()
        ids, t = s.trace_closest(rays)
    oids, ot = orc.closest_bvh(tris, rays)
    flags = orc.classify(tris, rays, oids, ot)
    _compare(ids, t, oids, ot, flags)
    sel = flags == 0
    assert np.array_equal(ids[sel], g["ids"][sel])


def test_trace_any_agrees_with_closest(cornell):
    s, tris = cornell
    rays = scenes.parity_rays(1 << 16, C1_LO, C1_HI, seed=4)
    ids, t = s.trace_closest(rays)
    rng = np.random.default_rng(2)
    tmax = rng.uniform(0.0, 15.0, len(rays)).astype(np.float32)
    occ = s.trace_any(rays, tmax)
    expect = (ids >= 0) & (t < tmax)
    # rays whose closest hit lies within 1e-6 of t_max may go either way
    near = np.abs(t - tmax) <= 1e-6 * np.maximum(t, 1.0)
    assert np.array_equal(occ[~near].astype(bool), expect[~near])
    assert s.trace_any(rays).astype(bool).tolist() == (ids >= 0).tolist()


def test_empty_batch_and_degenerate_rays(cornell):
    s, _ = cornell
    from kagayaki_gb300.structs import RAY
    ids, t = s.trace_closest(np.zeros(0, RAY))
    assert len(ids) == 0
    r = np.zeros(3, RAY)
    r["org"][:, :3] = (0.0, 5.0, 0.0)
    r["dir"][0, :3] = (0.0, 0.0, 0.0)          # zero direction: a miss, no fault
    r["dir"][1, :3] = (1.0, 0.0, 0.0)          # axis-aligned
    r["dir"][2, :3] = (0.0, -1.0, 0.0)
    ids, t = s.trace_closest(r)
    assert ids[0] == -1
    assert ids[1] >= 0 and abs(t[1] - 5.0) < 1e-5
    assert ids[2] >= 0 and abs(t[2] - 5.0) < 1e-5


def test_displaced_icosphere_field_full_size_property():
    """Config-2 geometry (64 x 81,920 displaced icosphere triangles + ground):
    GPU closest hits vs the oracle's conservative CPU BVH on 2^17 rays."""
    tris, mats, info = scenes.icosphere_field()
    assert len(tris) == 64 * 81920 + 2
    rays = scenes.parity_rays(1 << 17, info["lo"], info["hi"], seed=21)
    with Scene(tris, mats) as s:
        b = s.build_bvh()
        s.validate_bvh()
        ids, t, st = s.trace_closest(rays, with_stats=True)
    assert st["traversal_overflows"] == 0
    oids, ot = orc.closest_bvh(tris, rays)
    # exact-t ties and edge grazes are rare on curved meshes: every ray whose
    # answer differs is classified, by brute force over all 5.2M triangles
    # (an exact-t tie, or a reference barycentric within 4 ulp of an edge) or
    # else by exact rational arithmetic on the two candidate triangles (the
    # ray really hits ours first: the reference expression's rounding put it
    # on the other triangle); none may be left unexplained
    bad = np.nonzero(ids != oids)[0]
    assert len(bad) <= 1e-4 * len(rays), (len(bad), b)
    if len(bad):
        flags = orc.classify(tris, rays[bad], oids[bad], ot[bad])
        exact = np.array([orc.exact_winner(tris, rays[i], (int(ids[i]), int(oids[i])))[0] == ids[i]
                          for i in bad])
        print(f"{len(bad)} of {len(rays)} rays differ: {int((flags & 1).sum())} exact-t ties, "
              f"{int((flags & 2).sum())} edge grazes, {int((exact & (flags == 0)).sum())} where exact "
              f"arithmetic confirms ours")
        assert ((flags != 0) | exact).all(), f"{int(((flags == 0) & ~exact).sum())} unexplained id mismatches"
    hit = (oids >= 0) & (ids == oids)
    rel = np.abs(t[hit] - ot[hit]) / ot[hit]
    assert rel.max() <= T_REL_TOL, rel.max()


def test_watertight_closed_mesh():
    """Rays from inside a closed, displaced icosphere aimed exactly at its
    vertices and at the midpoints of its edges (where two or more triangles
    meet) must all hit: the edge functions of neighbouring triangles are
    computed with explicit rounding, so no ray slips through a shared edge."""
    v, f = scenes.icosphere(4)
    rng = np.random.default_rng(8)
    v = (v * (1.0 + 0.03 * rng.uniform(-1, 1, (len(v), 1)))).astype(np.float32)
    uv = np.zeros((len(v), 2), np.float32)
    tris = scenes.canonical(scenes._tris_from_indexed(v, v, uv, f.astype(np.int64), 0, False, 0))
    mats = np.stack([structs_lambert()])
    edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    mids = (v[edges[:, 0]].astype(np.float64) + v[edges[:, 1]].astype(np.float64)) / 2
    targets = np.concatenate([v.astype(np.float64), mids])
    origins = rng.uniform(-0.2, 0.2, (len(targets), 3))
    d = targets - origins
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(len(targets), dtype=scenes.RAY)
    rays["dir"][:, :3] = d.astype(np.float32)
    rays["org"][:, :3] = origins.astype(np.float32)
    with Scene(tris, mats) as s:
        s.build_bvh()
        ids, t = s.trace_closest(rays)
        occ = s.trace_any(rays)
    assert (ids >= 0).all(), f"{int((ids < 0).sum())} of {len(ids)} rays leaked"
    assert occ.all()


def structs_lambert():
    from kagayaki_gb300 import structs
    return structs.make_material(structs.LAMBERT, (0.5, 0.5, 0.5))
