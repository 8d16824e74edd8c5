"""The allocation-free ray cast entry point, through the C ABI.

parrygpu_trimesh_cast_rays_noalloc serves callers that may not allocate device memory while they
run (an engine owning the whole device budget, a frame loop that cannot block on cudaMalloc or on
cudaFree's device-wide wait): its ray-ordering scratch is a fixed array inside the library. This
test checks that two calls in a row give the same hits as parrygpu_trimesh_cast_rays, within the
tolerance of the other ray tests, and that a batch above the fixed maximum is rejected. It uses its
own context so that it passes alone in a fresh process as well as after the other tests; the file
name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REL = 1e-5


def _cast(fn, ctx, mesh, rays, torch):
    n = rays.shape[0]
    feat = torch.empty(n, dtype=torch.int32, device="cuda")
    toi = torch.empty(n, dtype=torch.float32, device="cuda")
    nrm = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    st = fn(ctx.handle, mesh._h, None, C.c_void_p(rays.data_ptr()), n, C.c_float(100.0), 1, C.c_void_p(feat.data_ptr()),
            C.c_void_p(toi.data_ptr()), C.c_void_p(nrm.data_ptr()))
    return st, feat, toi, nrm


@pytest.mark.parametrize("traversal", [1, 2, 3])
def test_noalloc_matches_existing_entry_point_on_two_calls(traversal):
    torch = pytest.importorskip("torch")
    from parry_gb300 import _build
    _build.build()
    import parry_gb300 as pg
    from parry_gb300 import workloads as W

    lib = pg.lib()
    ctx = pg.Context(device=0, ray_traversal=traversal)
    try:
        v, i = W.terrain_mesh(64, 32, seed=31)
        mesh = pg.TriMesh(ctx, v, i)
        for seed in (41, 42):
            rays = torch.from_numpy(W.terrain_rays(200_000, 64, 32, seed=seed)).cuda()
            st0, f0, t0, n0 = _cast(lib.parrygpu_trimesh_cast_rays, ctx, mesh, rays, torch)
            st1, f1, t1, n1 = _cast(lib.parrygpu_trimesh_cast_rays_noalloc, ctx, mesh, rays, torch)
            assert st0 == 0 and st1 == 0, pg.lib().parrygpu_last_error(ctx.handle)
            ctx.sync()
            f0, f1 = f0.cpu().numpy(), f1.cpu().numpy()
            np.testing.assert_array_equal(f1, f0)
            hit = f0.view(np.uint32) != pg.NO_HIT
            assert hit.sum() > 1000
            np.testing.assert_allclose(t1.cpu().numpy()[hit], t0.cpu().numpy()[hit], rtol=REL, atol=0)
            np.testing.assert_allclose(n1.cpu().numpy()[hit], n0.cpu().numpy()[hit], rtol=REL, atol=REL)
        # above the fixed maximum: rejected before any launch
        big = torch.zeros((300_000, 6), dtype=torch.float32, device="cuda")
        st, *_ = _cast(lib.parrygpu_trimesh_cast_rays_noalloc, ctx, mesh, big, torch)
        assert st == 1
        assert b"PARRYGPU_NOALLOC_MAX_RAYS" in lib.parrygpu_last_error(ctx.handle)
        # host rays are refused (they would need staging), and so would another GPU's memory
        host = np.zeros((1000, 6), np.float32)
        out = torch.empty(1000, dtype=torch.int32, device="cuda")
        st = lib.parrygpu_trimesh_cast_rays_noalloc(ctx.handle, mesh._h, None, C.c_void_p(host.ctypes.data), 1000, C.c_float(1.0), 1,
                                                    C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()), None)
        assert st == 1 and b"device memory" in lib.parrygpu_last_error(ctx.handle)
        mesh.close()
    finally:
        ctx.close()
