"""Oracle ray casts against convex shapes and shape sets (Compound) vs the reference's known
answers, and the Compound's best-first search vs a per-part loop (CPU only)."""
import numpy as np
import pytest

from tests import _contact_cases as CC


def test_cuboid_ray_doc_test(oracle_lib):
    s, rays, c = CC.cuboid_ray()
    part, toi, nrm = oracle_lib.Compound(s).cast_rays_and_get_normal(rays, c["max_toi"], solid=c["solid"])
    assert part[0] == 0 and toi[0] == c["expect_toi"]
    np.testing.assert_array_equal(nrm[0], np.array(c["expect_normal"], np.float32))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_solid_ray_cast_example(oracle_lib, prec):
    s, c = CC.solid_ray_cast()
    comp = oracle_lib.Compound(s, prec)
    for case in c["cases"]:
        part, toi, _ = comp.cast_rays_and_get_normal(np.array([case["ray"]], np.float32), np.finfo(np.float32).max,
                                                    solid=case["solid"], threads=1)
        if case["expect_toi"] is None:
            assert part[0] == 0xFFFFFFFF
        else:
            assert part[0] == 0 and toi[0] == case["expect_toi"]


def test_compound_equals_per_part_loop(oracle_lib):
    s = CC.mixed_scene(60, seed=2)
    rng = np.random.default_rng(4)
    o = rng.uniform(-12, 12, (3000, 3))
    d = rng.normal(size=(3000, 3))
    rays = np.concatenate([o, d], 1).astype(np.float32)
    comp = oracle_lib.Compound(s)
    part, toi, nrm = comp.cast_rays_and_get_normal(rays, 50.0, threads=1)
    # brute force: every part alone, smallest toi then smallest index
    t, prm, pos, pool = s.arrays()
    best_t = np.full(len(rays), np.inf)
    best_p = np.full(len(rays), 0xFFFFFFFF, np.uint64)
    from parry_gb300.shapes import ShapeSet
    for k in range(len(t)):
        sk = ShapeSet.from_arrays(t[k:k + 1], prm[k:k + 1], pos[k:k + 1], pool)
        pk, tk, _ = oracle_lib.Compound(sk).cast_rays_and_get_normal(rays, 50.0, threads=1)
        hit = pk != 0xFFFFFFFF
        better = hit & (tk < best_t)
        best_t[better] = tk[better]
        best_p[better] = k
    hit = best_p != 0xFFFFFFFF
    assert hit.sum() > 300
    np.testing.assert_array_equal(part[hit], best_p[hit].astype(np.uint32))
    np.testing.assert_array_equal(toi[hit], best_t[hit].astype(np.float32))
    assert np.all(part[~hit] == 0xFFFFFFFF)
