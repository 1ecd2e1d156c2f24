"""Degenerate and tiny shapes (one pixel, one angle, one-bin detectors, one-row slices): the
tiled kernels' tile and window logic at its boundaries, against the oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SHAPES = [  # nx, ny, px, pa, ss
    (1, 1, 1, 1, 1), (2, 3, 5, 1, 1), (5, 4, 3, 3, 3), (1, 7, 9, 4, 2), (9, 1, 2, 6, 3), (3, 3, 40, 7, 7),
    (100, 2, 100, 10, 5),
]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))


@pytest.mark.parametrize("shape", SHAPES)
def test_tiny_osem_and_operators(gpu_ctx, oracle_lib, shape):
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss = shape
    rng = np.random.default_rng(nx * 100 + ny * 10 + px)
    ang = np.sort(rng.uniform(0, 180, pa)).astype(np.float32)
    img = rng.uniform(0.2, 1.0, (ny, nx)).astype(np.float32)
    meas = (O.projection(img, ang, px) + rng.uniform(0, 0.05, (pa, px))).astype(np.float32)
    x0 = np.ones((ny, nx), np.float32)
    ref = O.osem_run(x0, meas, ang, ss, 2, order=O.ORDER_LITERAL)
    d_s = torch.from_numpy(meas).cuda()[None].contiguous()
    for kern in (xct.KERNELS_TILED, xct.KERNELS_PLAIN):
        plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 2, kernels=kern)
        d_x = torch.from_numpy(x0).cuda()[None].contiguous()
        plan.run_device(d_s, d_x)
        torch.cuda.synchronize()
        got = d_x[0].cpu().numpy()
        assert np.all(np.isfinite(got))
        assert _rel(got, ref) <= 1e-4, (shape, kern)
        plan.close()
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 2)
    # forward projection and exact adjoint
    d_p = torch.empty((1, pa, px), device="cuda")
    plan.fwd(torch.from_numpy(img).cuda()[None].contiguous(), d_p)
    d_a = torch.empty((1, ny, nx), device="cuda")
    plan.adj(d_s, d_a)
    torch.cuda.synchronize()
    assert _rel(d_p[0].cpu().numpy(), O.projection(img, ang, px)) <= 1e-5
    assert _rel(d_a[0].cpu().numpy(), O.adjoint(meas, ang, nx, ny)) <= 1e-5
    # FBP (smallest zero padding), bit-exact backprojection of the oracle's filtered rows
    zp = 64 if px <= 64 else 128
    d_f = torch.empty((1, ny, nx), device="cuda")
    plan.fbp(d_s, d_f, zp=zp)
    fprj = O.fbp_filter(meas, zp)
    d_b = torch.empty((1, ny, nx), device="cuda")
    plan.fbp_backproject(torch.from_numpy(fprj).cuda()[None].contiguous(), d_b)
    torch.cuda.synchronize()
    assert np.array_equal(d_b[0].cpu().numpy(), O.bp_fbp(fprj, ang, nx, ny))
    want = O.bp_fbp(fprj, ang, nx, ny)
    assert np.abs(d_f[0].cpu().numpy() - want).max() <= 1e-5 * max(1.0, np.abs(want).max())
    plan.close()


def test_tiny_reslice_and_cs(gpu_ctx, oracle_lib):
    import xct
    O = oracle_lib
    rng = np.random.default_rng(4)
    for A, H, W in ((1, 1, 1), (3, 1, 5), (2, 9, 1), (7, 3, 2)):
        mt = rng.uniform(0, 1, (A, H, W)).astype(np.float32)
        xs, ys = rng.uniform(-1, 1, A).astype(np.float32), rng.uniform(-1, 1, A).astype(np.float32)
        rp = xct.ReslicePlan(gpu_ctx, W, H, A, xs, ys, 0.5, 1)
        d = torch.empty((H, A, W), device="cuda")
        rp.reslice(torch.from_numpy(mt).cuda(), d)
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), O.reslice(mt, xs, ys, 0.5, 1)), (A, H, W)
        rp.close()
    # compressed sensing on single-slice and two-slice batches of a 5 x 4 image
    ang = np.array([0.0, 60.0, 120.0], np.float32)
    plan = xct.OSEMPlan(gpu_ctx, 5, 4, 6, ang, 3, 2, max_batch=2, kernels=xct.KERNELS_PLAIN)
    for dn in (1, 2):
        meas = rng.uniform(0.1, 1.0, (dn, 3, 6)).astype(np.float32)
        d_x = torch.ones((dn, 4, 5), device="cuda")
        plan.cs_run_device(torch.from_numpy(meas).cuda(), d_x)
        torch.cuda.synchronize()
        want = O.cs_osem_run(np.ones((dn, 4, 5), np.float32), meas, ang, 3, 2, 1e-4, order=O.ORDER_GPU)
        assert np.array_equal(d_x.cpu().numpy(), want), dn
    plan.close()
