"""Known-answer tests of the GPU kernels themselves (tiled and plain), not only through the
oracle: projections at 0 and 90 degrees are column and row sums, a disc projects to its
chord lengths, a uniform image with its own projections as data is a fixed point of OS-EM
(ratio exactly 1 on rays that meet it), and OSEM1 floors NaN and negative measurements at
1e-6 (OSEM.cl:64-66)."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

KERNELS = ["tiled", "plain"]


def _plan(ctx, kern, nx, ny, px, ang, ss=1, it=1, **kw):
    import xct
    k = xct.KERNELS_TILED if kern == "tiled" else xct.KERNELS_PLAIN
    return xct.OSEMPlan(ctx, nx, ny, px, np.asarray(ang, np.float32), ss, it, kernels=k, **kw)


def _fwd(plan, img):
    d_i = torch.from_numpy(np.ascontiguousarray(img, np.float32)).cuda()[None].contiguous()
    d_s = torch.empty((1, plan.pa, plan.px), device="cuda")
    plan.fwd(d_i, d_s)
    torch.cuda.synchronize()
    return d_s[0].cpu().numpy()


@pytest.mark.parametrize("kern", KERNELS)
def test_zero_and_ninety_degrees_are_column_and_row_sums(gpu_ctx, kern):
    rng = np.random.default_rng(0)
    img = rng.uniform(0, 1, (32, 32)).astype(np.float32)
    plan = _plan(gpu_ctx, kern, 32, 32, 32, [0.0, 90.0])
    p = _fwd(plan, img)
    np.testing.assert_allclose(p[0], img.sum(axis=0), rtol=1e-5)
    # at 90 degrees bin X samples row 32 - X (bin 0 looks at row 32, outside the image)
    rows = img.sum(axis=1)
    want = np.array([rows[32 - X] if 32 - X < 32 else 0.0 for X in range(32)], np.float32)
    np.testing.assert_allclose(p[1], want, rtol=1e-4, atol=1e-4)
    plan.close()


@pytest.mark.parametrize("kern", KERNELS)
def test_disc_projects_to_its_chords(gpu_ctx, kern):
    n, r = 128, 40.0
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    img = (((x - n / 2) ** 2 + (y - n / 2) ** 2) <= r * r).astype(np.float32)
    ang = [0.0, 30.0, 77.0, 133.5]
    plan = _plan(gpu_ctx, kern, n, n, n, ang)
    p = _fwd(plan, img)
    X = np.arange(n) - n / 2
    chord = 2 * np.sqrt(np.maximum(r * r - X ** 2, 0))
    inner = np.abs(X) < r - 3
    for k in range(len(ang)):
        assert np.abs(p[k][inner] - chord[inner]).max() < 2.0, ang[k]
        assert abs(p[k].sum() - math.pi * r * r) / (math.pi * r * r) < 0.02, ang[k]
    plan.close()


@pytest.mark.parametrize("kern", KERNELS)
def test_uniform_image_with_its_own_data_is_a_fixed_point(gpu_ctx, kern):
    import xct
    n, px, pa, ss = 32, 48, 20, 4
    ang = np.arange(pa, dtype=np.float32) * (180.0 / pa)
    plan = _plan(gpu_ctx, kern, n, n, px, ang, ss=ss, it=2)
    x = np.full((n, n), 0.7, np.float32)
    meas = _fwd(plan, x)
    d_x = torch.from_numpy(x).cuda()[None].contiguous()
    d_m = torch.from_numpy(meas).cuda()[None].contiguous()
    d_r = torch.zeros((1, pa, px), device="cuda")
    plan.osem1(0, d_x, d_m, d_r)
    torch.cuda.synchronize()
    r = d_r[0].cpu().numpy()
    rows = np.arange(0, pa, ss)
    hit = meas[rows] >= 1e-4
    assert hit.sum() > rows.size * n
    assert np.all(r[rows][hit] == np.float32(1.0))  # the same sums: m / p is exactly 1
    assert np.array_equal(r[rows][~hit], np.maximum(meas[rows][~hit], np.float32(1e-6)))
    plan.run_device(d_m, d_x)
    torch.cuda.synchronize()
    np.testing.assert_allclose(d_x[0].cpu().numpy(), x, rtol=1e-5)
    plan.close()


@pytest.mark.parametrize("kern", KERNELS)
def test_nan_and_negative_measurements_floor_at_1e_6(gpu_ctx, kern):
    n = 16
    plan = _plan(gpu_ctx, kern, n, n, n, [0.0, 45.0])
    d_x = torch.zeros((1, n, n), device="cuda")
    meas = np.array([[np.nan] * n, [-5.0] * n], np.float32)
    d_m = torch.from_numpy(meas).cuda()[None].contiguous()
    d_r = torch.full((1, 2, n), -1.0, device="cuda")
    plan.osem1(0, d_x, d_m, d_r)
    torch.cuda.synchronize()
    assert np.all(d_r[0].cpu().numpy() == np.float32(1e-6))
    plan.close()
