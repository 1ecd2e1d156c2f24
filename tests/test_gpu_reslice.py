"""Reslice on the device (Reslice/reslice.cl) through the C ABI: bit-exact against the
oracle (same sampler arithmetic, same correction table), and reslice -> OS-EM straight from
the device sinograms."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.mark.parametrize("correction", [0, 1])
def test_reslice_golden_bit_exact(gpu_ctx, correction):
    import xct
    f = _load("reslice_small")
    baseup = float(f["params"][0])
    A, H, W = f["mt"].shape
    rp = xct.ReslicePlan(gpu_ctx, W, H, A, f["xshift"], f["yshift"], baseup, correction)
    d_mt = torch.from_numpy(f["mt"]).cuda()
    d_s = torch.full((H, A, W), -7.0, device="cuda")
    rp.reslice(d_mt, d_s)
    torch.cuda.synchronize()
    assert np.array_equal(d_s.cpu().numpy(), f["sino_corr" if correction else "sino"])
    rp.close()


def test_reslice_in_angle_chunks(gpu_ctx, oracle_lib):
    """Projections arriving in chunks of angles fill the sinogram rows of their angles."""
    import xct
    O = oracle_lib
    rng = np.random.default_rng(5)
    A, H, W = 45, 33, 130
    mt = rng.uniform(0, 2, (A, H, W)).astype(np.float32)
    xs = rng.uniform(-4, 4, A).astype(np.float32)
    ys = rng.uniform(-3, 3, A).astype(np.float32)
    rp = xct.ReslicePlan(gpu_ctx, W, H, A, xs, ys, -0.5, 1)
    d_mt = torch.from_numpy(mt).cuda()
    d_s = torch.zeros((H, A, W), device="cuda")
    for a0, a1 in [(0, 13), (13, 40), (40, 45)]:
        rp.reslice(d_mt[a0:a1].contiguous(), d_s, first_angle=a0)
    torch.cuda.synchronize()
    assert np.array_equal(d_s.cpu().numpy(), O.reslice(mt, xs, ys, -0.5, 1))
    with pytest.raises(xct.XCTError):
        rp.reslice(d_mt[:10].contiguous(), d_s, first_angle=40)
    rp.close()


def test_denoise_bit_exact(gpu_ctx):
    import xct
    f = _load("reslice_small")
    thr = float(f["params"][1])
    d_src = torch.from_numpy(f["spiky"]).cuda()
    d_dst = torch.empty_like(d_src)
    xct.denoise_sinogram(d_src, d_dst, thr)
    torch.cuda.synchronize()
    assert np.array_equal(d_dst.cpu().numpy(), f["denoised"])
    with pytest.raises(xct.XCTError):
        xct.denoise_sinogram(d_src, d_src, thr)


def test_reslice_then_osem_on_device(gpu_ctx, oracle_lib):
    """CT flow without the file round trip (Reslice_CTreconst_ocl.cpp:26-136): projection
    images of an 8-slice volume -> sinograms in HBM -> OS-EM of all rows in one call."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, H, pa, ss, it = 64, 8, 60, 5, 2
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, H, count=6, seed=4)
    sinos = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, y, n, n), ang, n), 1e5, y)
                      for y in range(H)])                      # [H][A][W]
    mt = np.ascontiguousarray(sinos.transpose(1, 0, 2))        # projections [A][H][W]
    rp = xct.ReslicePlan(gpu_ctx, n, H, pa)
    d_s = torch.empty((H, pa, n), device="cuda")
    rp.reslice(torch.from_numpy(mt).cuda(), d_s)
    plan = xct.OSEMPlan(gpu_ctx, n, n, n, ang, ss, it, max_batch=H)
    d_x = torch.ones((H, n, n), device="cuda")
    plan.run_device(d_s, d_x)
    torch.cuda.synchronize()
    assert np.array_equal(d_s.cpu().numpy(), sinos)  # zero shifts: an exact transpose
    got = d_x.cpu().numpy()
    x0 = np.ones((n, n), np.float32)
    for y in range(H):
        ref = O.osem_run(x0, sinos[y], ang, ss, it, order=O.ORDER_LITERAL)
        assert np.linalg.norm(got[y] - ref) / np.linalg.norm(ref) <= 1e-4, y
    plan.close()
    rp.close()


def test_reslice_staged_windows_bit_exact(gpu_ctx, oracle_lib):
    """The tensor-copy kernel (width a multiple of 4): partial tiles in both directions,
    shifts that move whole windows off the projection, shifts whose rounding moves a sampler
    column or row by one (those columns fall back to global loads), NaN and inf texels, angle
    chunks, and a misaligned projection pointer (the row-walking kernel) -- all equal to the
    oracle."""
    import xct
    O = oracle_lib
    rng = np.random.default_rng(11)
    A, H, W = 37, 45, 388
    mt = rng.uniform(-1, 3, (A, H, W)).astype(np.float32)
    mt[3, 7, 100] = np.nan
    mt[5, 0, 0] = np.inf
    mt[6, 44, 387] = -np.inf
    xs = rng.uniform(-6, 6, A).astype(np.float32)
    ys = rng.uniform(-4, 4, A).astype(np.float32)
    xs[:6] = [-1e-8, 0.49999997, 200.0, -450.0, 63.5, -0.5]
    ys[:6] = [-1e-8, 2.5, -50.0, 7.25, 0.49999997, -44.5]
    for corr, base in ((0, 0.0), (1, 0.75)):
        want = O.reslice(mt, xs, ys, base, corr)
        rp = xct.ReslicePlan(gpu_ctx, W, H, A, xs, ys, base, corr)
        d_mt = torch.from_numpy(mt).cuda()
        d_s = torch.full((H, A, W), -3.0, device="cuda")
        rp.reslice(d_mt, d_s)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_s.cpu().numpy(), want)
        # chunks of angles (aligned views of the same stack)
        d_s.fill_(-3.0)
        for a0, a1 in [(0, 1), (1, 20), (20, 37)]:
            rp.reslice(d_mt[a0:a1], d_s, first_angle=a0)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_s.cpu().numpy(), want)
        # a projection stack one float off 16-byte alignment
        buf = torch.empty(A * H * W + 1, device="cuda")
        buf[1:] = d_mt.reshape(-1)
        d_s.fill_(-3.0)
        rp.reslice(buf[1:].view(A, H, W), d_s)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_s.cpu().numpy(), want)
        rp.close()  # raises if a staged copy missed its wait limit


def test_reslice_staged_wait_limit_fallback(gpu_ctx, oracle_lib):
    """Waits that give up: with a negative limit every CTA of the staged kernel abandons its
    copies at the first tile (nothing stalls; the copies in flight still land before the
    kernel ends), computes every tile from global memory -- still bit-exact -- and the plan
    reports XCT_E_TIMEOUT when destroyed.  The context stays usable afterwards."""
    import xct
    O = oracle_lib
    rng = np.random.default_rng(12)
    A, H, W = 20, 40, 260
    mt = rng.uniform(0, 2, (A, H, W)).astype(np.float32)
    xs = rng.uniform(-3, 3, A).astype(np.float32)
    ys = rng.uniform(-2, 2, A).astype(np.float32)
    want = O.reslice(mt, xs, ys, 0.25, 1)
    d_mt = torch.from_numpy(mt).cuda()
    rp = xct.ReslicePlan(gpu_ctx, W, H, A, xs, ys, 0.25, 1)
    rp.set_wait_limit(-1)
    d_s = torch.full((H, A, W), -3.0, device="cuda")
    rp.reslice(d_mt, d_s)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_s.cpu().numpy(), want)
    with pytest.raises(xct.XCTError) as e:
        rp.close()
    assert e.value.code == xct.XCT_E_TIMEOUT and "wait limit" in str(e.value)
    rp2 = xct.ReslicePlan(gpu_ctx, W, H, A, xs, ys, 0.25, 1)
    d_s.fill_(-3.0)
    rp2.reslice(d_mt, d_s)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_s.cpu().numpy(), want)
    rp2.close()
