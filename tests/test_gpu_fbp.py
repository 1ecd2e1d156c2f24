"""FBP (FBP.cl, FBP_execution) and the FBP + OS-EM hybrid on the GPU, through the C ABI.

Tolerances:
  * ramp filter: the CUDA filter is a different FFT (shared-memory Stockham, two rows per
    complex transform) from the reference's radix-2 chain; both are float.  The reference
    chain itself sits ~2e-6 rel-L2 from the exact-twiddle double transform, so the CUDA
    filter is held to 1e-5 rel-L2 against the double transform and 2e-5 against the
    reference chain (max abs error 1e-4 of the row maximum).
  * backProjectionFBP: bit-exact given the same filtered sinogram (same expression order,
    same sampler arithmetic, angles summed in order).
  * FBP image and hybrid: what the filter's rounding becomes after the backprojection
    (2e-5 rel-L2) and after base-up + OS-EM (1e-4 rel-L2).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _plan(ctx, f, max_batch=1, **kw):
    import xct
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"][:6]]
    return xct.OSEMPlan(ctx, nx, ny, px, f["angles"], ss, it, max_batch=max_batch, **kw)


@pytest.mark.parametrize("name", ["fbp_64", "fbp_odd"])
def test_fbp_filter_matches_reference_chain(gpu_ctx, name):
    f = _load(name)
    zp = int(f["shape"][6])
    plan = _plan(gpu_ctx, f)
    d_s = torch.from_numpy(f["meas"]).cuda()[None].contiguous()
    d_f = torch.empty_like(d_s)
    plan.fbp_filter(d_s, d_f, zp=zp)
    torch.cuda.synchronize()
    got = d_f[0].cpu().numpy()
    assert _rel(got, f["fprj_f64"]) <= 1e-5
    assert _rel(got, f["fprj"]) <= 2e-5
    assert np.abs(got - f["fprj"]).max() <= 1e-4 * np.abs(f["fprj"]).max()
    plan.close()


@pytest.mark.parametrize("zp", [64, 128, 256, 1024, 4096, 8192, 16384])
def test_fbp_filter_transform_lengths(gpu_ctx, oracle_lib, zp):
    """Every kernel variant (2, 4, 8, 16 values per thread) against the double transform,
    with an odd number of rows (the last CTA filters one row)."""
    import xct
    O = oracle_lib
    px = min(zp, 61 if zp < 128 else (zp // 2 + 3))
    pa = 7
    rng = np.random.default_rng(zp)
    s = rng.normal(1.0, 0.3, (pa, px)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, 32, 32, px, np.arange(pa, dtype=np.float32) * 25.0, 1, 1)
    d_s = torch.from_numpy(s).cuda()[None].contiguous()
    d_f = torch.empty_like(d_s)
    plan.fbp_filter(d_s, d_f, zp=zp)
    torch.cuda.synchronize()
    ref = O.fbp_filter(s.astype(np.float64), zp, dtype=np.float64)
    assert _rel(d_f[0].cpu().numpy(), ref) <= 1e-5
    plan.close()


@pytest.mark.parametrize("name", ["fbp_64", "fbp_odd"])
def test_fbp_backprojection_bit_exact(gpu_ctx, name):
    f = _load(name)
    plan = _plan(gpu_ctx, f)
    ny, nx = f["fbp"].shape
    d_f = torch.from_numpy(f["fprj"]).cuda()[None].contiguous()
    d_i = torch.full((1, ny, nx), 7.0, device="cuda")
    plan.fbp_backproject(d_f, d_i)
    torch.cuda.synchronize()
    got = d_i[0].cpu().numpy()
    assert np.array_equal(got, f["fbp"])
    plan.close()


def test_fbp_backprojection_bit_exact_offcentre(gpu_ctx, oracle_lib):
    """Non-square image, odd bins, irregular angles, rotation centre off px/2, several
    slices per call; partial edge tiles in both directions."""
    import xct
    O = oracle_lib
    nx, ny, px, pa, cx = 150, 70, 171, 83, 87.25
    rng = np.random.default_rng(4)
    ang = np.sort(rng.uniform(0, 180, pa)).astype(np.float32)
    fprj = rng.normal(0, 1, (3, pa, px)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, 1, 1, center_bin=cx, max_batch=3)
    d_f = torch.from_numpy(fprj).cuda().contiguous()
    d_i = torch.zeros((3, ny, nx), device="cuda")
    plan.fbp_backproject(d_f, d_i)
    torch.cuda.synchronize()
    for z in range(3):
        assert np.array_equal(d_i[z].cpu().numpy(), O.bp_fbp(fprj[z], ang, nx, ny, cx=cx)), z
    plan.close()


@pytest.mark.parametrize("name", ["fbp_64", "fbp_odd"])
def test_fbp_image_and_hybrid(gpu_ctx, name):
    f = _load(name)
    nx, ny, px, pa, ss, it, zp, order = [int(v) for v in f["shape"]]
    plan = _plan(gpu_ctx, f)
    d_s = torch.from_numpy(f["meas"]).cuda()[None].contiguous()
    d_i = torch.zeros((1, ny, nx), device="cuda")
    plan.fbp(d_s, d_i, zp=zp)
    torch.cuda.synchronize()
    img = d_i[0].cpu().numpy()
    assert _rel(img, f["fbp"]) <= 2e-5
    d_h = torch.zeros((1, ny, nx), device="cuda")
    plan.hybrid(d_s, d_h, zp=zp, baseup_order=order, sub=f["sub"], it=it)
    torch.cuda.synchronize()
    hyb = d_h[0].cpu().numpy()
    assert _rel(hyb, f["hybrid"]) <= 1e-4
    assert np.abs(hyb - f["hybrid"]).max() <= 1e-3 * np.abs(f["hybrid"]).max()
    # the host-buffer forms give the device forms' results
    out = [np.zeros((ny, nx), np.float32)]
    plan.fbp_run([f["meas"].copy()], out, zp=zp)
    assert np.array_equal(out[0], img)
    out = [np.zeros((ny, nx), np.float32)]
    plan.hybrid_run([f["meas"].copy()], out, zp=zp, baseup_order=order, sub=f["sub"], it=it)
    # the forward projector's per-tile partial sums meet in double atomics in any order
    assert _rel(out[0], hyb) <= 1e-6
    plan.close()


def test_hybrid_base_up_step(gpu_ctx, oracle_lib):
    """Hybrid with zero OS-EM iterations leaves FBP + base-up: checked against the oracle's
    base-up of the GPU's own FBP image (the minimum is exact; exp may differ by 2 ulp)."""
    O = oracle_lib
    f = _load("fbp_64")
    nx, ny, px, pa, ss, it, zp, order = [int(v) for v in f["shape"]]
    plan = _plan(gpu_ctx, f, max_batch=2)
    s2 = np.stack([f["meas"], f["meas"][::-1]]).astype(np.float32)
    d_s = torch.from_numpy(s2).cuda().contiguous()
    d_i = torch.zeros((2, ny, nx), device="cuda")
    plan.fbp(d_s, d_i, zp=zp)
    d_h = torch.zeros((2, ny, nx), device="cuda")
    for order in (0, 1, 4, 9):
        plan.hybrid(d_s, d_h, zp=zp, baseup_order=order, it=0)
        torch.cuda.synchronize()
        for z in range(2):
            want, _ = O.base_up(d_i[z].cpu().numpy(), order)
            got = d_h[z].cpu().numpy()
            assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max() + 1e-12, (order, z)
    plan.close()


def test_fbp_after_osem_keeps_ratio_rows_zero(gpu_ctx, oracle_lib):
    """FBP borrows the plan's ratio buffer; an OS-EM run on the same plan afterwards (pa % ss
    != 0: rows OSEM1 never writes are read as 0) is unchanged."""
    import xct
    O = oracle_lib
    f = _load("fbp_odd")
    ny, nx = f["fbp"].shape
    ang = f["angles"]
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, f["meas"].shape[1], ang, 5, 2)
    d_s = torch.from_numpy(f["meas"]).cuda()[None].contiguous()
    x0 = torch.ones((1, ny, nx), device="cuda")
    a = x0.clone()
    plan.run_device(d_s, a)
    b = torch.zeros((1, ny, nx), device="cuda")
    plan.fbp(d_s, b, zp=256)
    c = x0.clone()
    plan.run_device(d_s, c)
    torch.cuda.synchronize()
    # equal up to the order of the forward projector's double atomics; ratio rows left
    # holding filtered values would move the result by far more
    assert _rel(c.cpu().numpy(), a.cpu().numpy()) <= 1e-6
    plan.close()


def test_fbp_argument_errors(gpu_ctx):
    import xct
    plan = xct.OSEMPlan(gpu_ctx, 32, 32, 40, np.arange(10, dtype=np.float32) * 18, 1, 1)
    d_s = torch.zeros((1, 10, 40), device="cuda")
    d_f = torch.zeros_like(d_s)
    for zp in (32, 48, 100, 32768):
        with pytest.raises(xct.XCTError) as e:
            plan.fbp_filter(d_s, d_f, zp=zp)
        assert "power of two" in str(e.value)
    with pytest.raises(xct.XCTError):
        plan.hybrid(d_s, torch.zeros((1, 32, 32), device="cuda"), baseup_order=-1)
    with pytest.raises(xct.XCTError):
        xct.OSEMPlan(gpu_ctx, 32, 32, 40, np.arange(10, dtype=np.float32), 1, 1, center_bin=float("nan"))
    plan.close()
