"""The slice-interleaved kernels (groups of slices of one geometry; xct_plan_set_multislice):
the forward projector (one 128-byte shared-memory line per texel), the OS-EM and FBP
backprojectors (one bin expression per eight slices) and the exact adjoint (gather form).

It must compute what the per-slice tiled kernel computes -- the same samples and bilinear
weights; only the order in which a ray's samples are added differs (one lane walks the
ray's whole interval in a tile instead of four lanes taking every fourth sample), so the
results agree to float rounding -- and it must meet the OS-EM parity bar against the oracle
(OSEM.cl:38-105 driven as OSEM_execution, GPU.cpp:125-240) on geometries that exercise its
tiles: sizes below and not a multiple of the 42-texel tile, non-square slices, more bins than
pixels, an off-centre axis, unsorted angles over 360 degrees, subsets that do not divide the
angles, angle chunks smaller than a subset, and batches with a remainder that goes to the
per-slice kernel.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

CASES = [  # nx, ny, px, pa, ss, span, centre offset, dN, ms chunk
    (64, 64, 64, 90, 10, 180.0, 0.0, 8, 128),
    (100, 73, 131, 61, 4, 360.0, 2.75, 11, 7),
    (30, 30, 40, 36, 3, 180.0, -1.5, 9, 128),
    (256, 256, 256, 180, 10, 180.0, 0.0, 16, 64),
    (173, 211, 160, 47, 5, 200.0, 0.0, 10, 5),
]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _case(c, seed):
    from xct import phantom as P
    nx, ny, px, pa, ss, span, off, dN, chunk = c
    rng = np.random.default_rng(seed)
    ang = rng.permutation(np.arange(pa) * (span / pa)).astype(np.float32)
    m = max(nx, ny)
    imgs = np.stack([P.rasterize_ellipses(P.ellipse_params(m, 5, seed + z, axes=(2, m / 4)), m, m)[:ny, :nx]
                     for z in range(dN)]).astype(np.float32) + np.float32(0.01)
    return ang, np.ascontiguousarray(imgs), px * 0.5 + off


@pytest.mark.parametrize("case", range(len(CASES)))
def test_multislice_forward_matches_per_slice_kernel_and_oracle(gpu_ctx, oracle_lib, case):
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, span, off, dN, chunk = CASES[case]
    ang, imgs, cx = _case(CASES[case], 40 + case)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 1, center_bin=cx, max_batch=dN)
    d_img = torch.from_numpy(imgs).cuda()
    plan.set_multislice(0)
    ref = torch.empty((dN, pa, px), device="cuda")
    plan.fwd(d_img, ref)
    plan.set_multislice(chunk)
    assert plan.multislice() == chunk
    got = torch.empty((dN, pa, px), device="cuda")
    plan.fwd(d_img, got)
    torch.cuda.synchronize()
    got, ref = got.cpu().numpy(), ref.cpu().numpy()
    assert np.all(np.isfinite(got))
    for z in range(dN):
        assert _rel(got[z], ref[z]) <= 2e-6, z
    for z in (0, 7, dN - 1):
        want = O.projection(imgs[z], ang, px, cx=cx)
        assert _rel(got[z], want) <= 1e-5, z
    plan.close()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_multislice_osem_matches_oracle(gpu_ctx, oracle_lib, case):
    import xct
    from xct import phantom as P
    O = oracle_lib
    nx, ny, px, pa, ss, span, off, dN, chunk = CASES[case]
    ang, imgs, cx = _case(CASES[case], 60 + case)
    meas = np.stack([P.noisy_log_sinogram(O.projection(imgs[z], ang, px, cx=cx), 1e5, z) for z in range(dN)])
    it = 2
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, it, center_bin=cx, max_batch=dN)
    plan.set_multislice(chunk)
    x = torch.ones((dN, ny, nx), device="cuda")
    plan.run_device(torch.from_numpy(meas).cuda(), x)
    torch.cuda.synchronize()
    x = x.cpu().numpy()
    for z in (0, 7, dN - 1):
        want = O.osem_run(np.ones((ny, nx), np.float32), meas[z], ang, ss, it, cx=cx, order=O.ORDER_LITERAL)
        rel = _rel(x[z], want)
        mx = np.abs(x[z] - want).max() / np.abs(want).max()
        assert rel <= 1e-4 and mx <= 1e-3, (z, rel, mx)
    plan.close()


def test_multislice_default_and_switch(gpu_ctx):
    """On by default where a group of eight fills the GPU (2048^2: 2401 tiles of 42), off for
    small slices and for plans of fewer than eight slices; the plain kernels refuse it."""
    import xct
    ang = np.arange(60, dtype=np.float32) * 3.0
    big = xct.OSEMPlan(gpu_ctx, 2048, 2048, 2048, ang, 6, 1, max_batch=8)
    assert big.multislice() == 128
    big.close()
    one = xct.OSEMPlan(gpu_ctx, 2048, 2048, 2048, ang, 6, 1, max_batch=4)
    assert one.multislice() == 0
    one.close()
    small = xct.OSEMPlan(gpu_ctx, 128, 128, 128, ang, 6, 1, max_batch=8)
    assert small.multislice() == 0
    with pytest.raises(RuntimeError):
        small.set_multislice(200)
    small.close()
    plain = xct.OSEMPlan(gpu_ctx, 64, 64, 64, ang, 6, 1, max_batch=8, kernels=xct.KERNELS_PLAIN)
    with pytest.raises(RuntimeError):
        plain.set_multislice(16)
    plain.close()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_multislice_backprojector_bit_identical(gpu_ctx, oracle_lib, case):
    """OSEM2 of dN slices with the eight-slice backprojector (groups of eight, the rest per
    slice) gives every slice the per-slice kernel's image bit for bit, and the oracle's
    (OSEM.cl:71-105 in the GPU order, which is the literal bin expression) bit for bit."""
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, span, off, dN, chunk = CASES[case]
    ang, imgs, cx = _case(CASES[case], 60 + case)
    rng = np.random.default_rng(70 + case)
    ratio = rng.uniform(0.5, 1.5, (dN, pa, px)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 1, center_bin=cx, max_batch=dN)
    d_r = torch.from_numpy(ratio).cuda()
    for sub in (0, ss - 1):
        plan.set_multislice(0)
        ref = torch.from_numpy(imgs).cuda()
        plan.osem2(sub, ref, d_r)
        plan.set_multislice(chunk)
        got = torch.from_numpy(imgs).cuda()
        plan.osem2(sub, got, d_r)
        torch.cuda.synchronize()
        g = got.cpu().numpy()
        r = ref.cpu().numpy()
        assert np.array_equal(g, r), (sub, int(np.count_nonzero(g != r)))
        for z in (0, dN - 1):
            want = O.osem2(imgs[z], ratio[z], ang, ss, sub, cx=cx, order=O.ORDER_GPU)
            assert np.array_equal(g[z], want), (sub, z, int(np.count_nonzero(g[z] != want)))
    plan.close()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_multislice_adjoint_matches_per_slice_kernel_and_oracle(gpu_ctx, oracle_lib, case):
    """The exact adjoint over groups of eight slices (the gather form: each base texel finds
    its own samples, float sums, no atomics) and of four (the scatter form with shared sample
    work) against the per-slice scatter kernel (fixed-point sums) and against the oracle's
    float64 adjoint: the same operator to float rounding."""
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, span, off, dN, chunk = CASES[case]
    ang, _, cx = _case(CASES[case], 80 + case)
    rng = np.random.default_rng(90 + case)
    s_np = rng.uniform(0.5, 1.5, (dN, pa, px)).astype(np.float32)
    sino = torch.from_numpy(s_np).cuda()
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 1, center_bin=cx, max_batch=dN)
    plan.set_multislice(0)
    ref = torch.empty((dN, ny, nx), device="cuda")
    plan.adj(sino, ref)
    plan.set_multislice(chunk)
    got = torch.empty((dN, ny, nx), device="cuda")
    plan.adj(sino, got)
    torch.cuda.synchronize()
    g, r = got.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
    for z in range(dN):
        assert _rel(g[z], r[z]) <= 2e-6, (z, _rel(g[z], r[z]))
    for z in (0, dN - 1):
        want = O.adjoint(s_np[z], ang, nx, ny, cx=cx, dtype=np.float64)
        assert _rel(g[z], want) <= 1e-5, (z, _rel(g[z], want))
    plan.close()


def test_multislice_adjoint_gradient_step(gpu_ctx):
    """XCT_FISTA_ADJOINT (x + coef * A^T r in the adjoint's epilogue) on thirteen slices: eight
    through the gather adjoint, four through the four-slice scatter and one through the
    per-slice kernel give the per-slice result to float rounding."""
    import xct
    from xct import phantom as P
    n, px, pa, ss, it, dN = 96, 96, 60, 6, 2, 13
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, dN, count=6, seed=97)
    imgs = np.stack([P.ellipsoid_slice(prm, z, n, n) for z in range(dN)]).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, max_batch=dN)
    plan.set_lipschitz(plan.power_iteration(trials=10))
    meas = torch.empty((dN, pa, px), device="cuda")
    plan.fwd(torch.from_numpy(imgs).cuda(), meas)
    out = {}
    for ms in (0, 128):
        plan.set_multislice(ms)
        x = torch.zeros((dN, n, n), device="cuda")
        plan.fista_run_device(meas, x, flags=xct.FISTA_ADJOINT | xct.FISTA_UPDATE_X)
        torch.cuda.synchronize()
        out[ms] = x.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(out[128]))
    assert _rel(out[128], out[0]) <= 1e-6
    plan.close()


def test_multislice_dot_product(gpu_ctx):
    """<A x, y> = <x, A^T y> on eight slices of 512^2 with 360 angles through the
    slice-interleaved forward projector and the gather adjoint (to 1e-5 relative)."""
    import xct
    from xct import phantom as P
    n, pa, dN = 512, 360, 8
    plan = xct.OSEMPlan(gpu_ctx, n, n, n, P.uniform_angles(pa), 1, 1, max_batch=dN)
    plan.set_multislice(128)
    g = torch.Generator(device="cuda")
    g.manual_seed(8)
    for _ in range(4):
        x = torch.rand((dN, n, n), device="cuda", generator=g)
        y = torch.rand((dN, pa, n), device="cuda", generator=g)
        ax = torch.empty((dN, pa, n), device="cuda")
        aty = torch.empty((dN, n, n), device="cuda")
        plan.fwd(x, ax)
        plan.adj(y, aty)
        torch.cuda.synchronize()
        for z in range(dN):
            lhs = float((ax[z].double() * y[z].double()).sum())
            rhs = float((x[z].double() * aty[z].double()).sum())
            assert abs(lhs - rhs) <= 1e-5 * abs(lhs), (z, lhs, rhs)
    plan.close()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_multislice_fbp_bit_identical(gpu_ctx, oracle_lib, case):
    """The FBP backprojection of dN slices with the eight-slice kernel (groups of eight, the
    rest per slice) gives every slice the per-slice kernel's image bit for bit, and the
    hybrid's base-up (which uses the per-slice minimum the backprojector reduces) as well;
    slice 0 is also bit-identical to the oracle's backProjectionFBP (FBP.cl:164-188)."""
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, span, off, dN, chunk = CASES[case]
    ang, _, cx = _case(CASES[case], 100 + case)
    rng = np.random.default_rng(110 + case)
    fp = rng.uniform(-0.5, 1.5, (dN, pa, px)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 1, center_bin=cx, max_batch=dN)
    d_fp = torch.from_numpy(fp).cuda()
    out = {}
    for ms in (0, chunk):
        plan.set_multislice(ms)
        x = torch.empty((dN, ny, nx), device="cuda")
        plan.fbp_backproject(d_fp, x)
        h = torch.empty((dN, ny, nx), device="cuda")
        plan.hybrid(d_fp.abs().contiguous(), h, zp=0, it=0)
        torch.cuda.synchronize()
        out[ms] = (x.cpu().numpy(), h.cpu().numpy())
    assert np.array_equal(out[chunk][0], out[0][0]), int(np.count_nonzero(out[chunk][0] != out[0][0]))
    assert np.array_equal(out[chunk][1], out[0][1]), int(np.count_nonzero(out[chunk][1] != out[0][1]))
    want = O.bp_fbp(fp[0], ang, nx, ny, cx=cx)
    assert np.array_equal(out[chunk][0][0], want), int(np.count_nonzero(out[chunk][0][0] != want))
    plan.close()


def test_multislice_compressed_sensing(gpu_ctx, oracle_lib):
    """Compressed-sensing OS-EM (FISTA_OSEM_execution, GPU.cpp:243-405) on a stack of nine
    slices through the slice-interleaved kernels (eight) and the per-slice ones (one) against
    the per-slice kernels alone and against the oracle."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, pa, ss, it, dN, lam = 96, 72, 6, 2, 9, 1.0e-4
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, dN, count=6, seed=123)
    meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, n), 1e5, z)
                     for z in range(dN)]).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, n, n, n, ang, ss, it, max_batch=dN)
    out = {}
    for ms in (0, 128):
        plan.set_multislice(ms)
        x = torch.ones((dN, n, n), device="cuda")
        plan.cs_run_device(torch.from_numpy(meas).cuda(), x, cs_lambda=lam)
        torch.cuda.synchronize()
        out[ms] = x.cpu().numpy().astype(np.float64)
    assert _rel(out[128], out[0]) <= 1e-5
    want = O.cs_osem_run(np.ones((dN, n, n), np.float32), meas, ang, ss, it, lam)
    assert _rel(out[128], want) <= 1e-4
    plan.close()
