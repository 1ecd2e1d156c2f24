"""GPU parity of the two OS-EM kernels on their own (OSEM1, OSEM2) through the C ABI, on
shapes that span several tiles, against the oracle in the GPU evaluation order.

* OSEM2 given the oracle's own ratio image must be BIT-IDENTICAL: the nearest-bin
  backprojection sums the same values in the same angle order with the reference's bin
  arithmetic.
* OSEM1's ratio rows: bit-identical for the plain kernel (sequential ray sums); within
  rel-L2 5e-6 for the tiled kernel (its ray sums add per-tile partials in double).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SHAPES = [
    # nx, ny, px, pa, ss, span (deg), centre offset
    (256, 256, 256, 180, 10, 180.0, 0.0),
    (256, 256, 256, 180, 1, 180.0, 0.0),
    (300, 200, 250, 77, 7, 360.0, 0.0),
    (130, 130, 200, 64, 4, 180.0, 3.5),
]


def _case(shape, seed):
    from xct import phantom as P
    nx, ny, px, pa, ss, span, off = shape
    m = max(nx, ny)
    img = P.rasterize_ellipses(P.ellipse_params(m, 8, seed, axes=(3, m / 4)), m, m)
    img = np.ascontiguousarray(img[(m - ny) // 2:(m - ny) // 2 + ny, (m - nx) // 2:(m - nx) // 2 + nx])
    img = img + np.float32(0.01)
    ang = (np.arange(pa) * (span / pa) - (90.0 if span > 180 else 0.0)).astype(np.float32)
    return img, ang, px * 0.5 + off


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.mark.parametrize("kernels", [0, 1])
@pytest.mark.parametrize("shape", SHAPES)
def test_osem2_bit_identical_given_the_same_ratio(gpu_ctx, oracle_lib, shape, kernels):
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, span, off = shape
    img, ang, cx = _case(shape, 3)
    meas = O.projection(img, ang, px, cx=cx) * np.float32(1.1)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 1, center_bin=cx, kernels=kernels)
    x = np.full((ny, nx), 0.8, np.float32)
    for sub in range(ss):
        ratio = O.osem1(x, meas, ang, ss, sub, cx=cx, order=O.ORDER_GPU)
        want = O.osem2(x, ratio, ang, ss, sub, cx=cx, order=O.ORDER_GPU)
        d_x = _dev(x[None])
        plan.osem2(sub, d_x, _dev(ratio[None]))
        torch.cuda.synchronize()
        got = d_x[0].cpu().numpy()
        bad = np.argwhere(got != want)
        assert bad.size == 0, "subset %d: %d pixels differ, first %s" % (sub, len(bad), bad[:5].tolist())
        x = want
    plan.close()


@pytest.mark.parametrize("kernels", [0, 1])
@pytest.mark.parametrize("shape", SHAPES)
def test_osem1_ratio_matches_oracle(gpu_ctx, oracle_lib, shape, kernels):
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, span, off = shape
    img, ang, cx = _case(shape, 4)
    meas = O.projection(img, ang, px, cx=cx) * np.float32(0.9)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 1, center_bin=cx, kernels=kernels)
    d_img, d_meas = _dev(img[None]), _dev(meas[None])
    for sub in range(ss):
        d_r = torch.full((1, pa, px), -7.0, device="cuda")
        plan.osem1(sub, d_img, d_meas, d_r)
        torch.cuda.synchronize()
        got = d_r[0].cpu().numpy()
        want = O.osem1(img, meas, ang, ss, sub, cx=cx, order=O.ORDER_GPU)
        rows = np.arange(sub, sub + (pa // ss) * ss, ss)
        others = np.setdiff1d(np.arange(pa), rows)
        assert np.all(got[others] == -7.0), "rows outside the subset were written"
        g, w = got[rows].astype(np.float64), want[rows].astype(np.float64)
        if kernels == 1:
            assert np.array_equal(g, w)
        else:
            # per-tile partial sums added in double: a few ulps from the sequential sum
            assert np.linalg.norm(g - w) / np.linalg.norm(w) <= 5e-6
            assert np.max(np.abs(g - w) / np.abs(w)) <= 1e-4
    plan.close()


def test_short_buffers_are_rejected_before_launch(gpu_ctx):
    """The library takes bare pointers; the Python mirror refuses buffers shorter than the
    call touches (no kernel runs), and the plan works afterwards."""
    import xct
    nx, ny, px, pa = 40, 30, 48, 20
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, np.arange(pa, dtype=np.float32) * 9.0, 4, 1, max_batch=2)
    sino = torch.rand((2, pa, px), device="cuda") + 0.1
    img = torch.ones((2, ny, nx), device="cuda")
    short_sino = torch.rand((2, pa - 1, px), device="cuda")
    short_img = torch.ones((2, ny, nx - 1), device="cuda")
    before = xct.launch_count()
    for call in (lambda: plan.run_device(short_sino, img), lambda: plan.run_device(sino, short_img),
                 lambda: plan.fwd(img, short_sino), lambda: plan.adj(short_sino, img),
                 lambda: plan.fbp(sino, short_img), lambda: plan.hybrid(short_sino, img),
                 lambda: plan.cs_run_device(sino, short_img),
                 lambda: plan.rot_center_shift(sino[0], short_sino, -1.0, 1.0),
                 lambda: plan.run([np.zeros(pa * px - 1, np.float32)], [np.zeros(ny * nx, np.float32)])):
        with pytest.raises(xct.XCTError) as e:
            call()
        assert e.value.code == xct.XCT_E_INVALID and "elements" in str(e.value)
    torch.cuda.synchronize()
    assert xct.launch_count() == before
    rp = xct.ReslicePlan(gpu_ctx, px, 6, pa)
    with pytest.raises(xct.XCTError):
        rp.reslice(torch.rand((pa, 6, px - 1), device="cuda"), torch.empty((6, pa, px), device="cuda"))
    with pytest.raises(xct.XCTError):
        rp.reslice(torch.rand((pa, 6, px), device="cuda"), torch.empty((6, pa - 1, px), device="cuda"))
    rp.close()
    with pytest.raises(xct.XCTError):
        xct.denoise_sinogram(sino, torch.empty((2, pa, px - 1), device="cuda"), 0.1)
    plan.run_device(sino, img)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(img).all())
    plan.close()
