"""GPU parity: the CUDA OS-EM path through the C ABI against the oracle and the golden
fixtures (which are bit-identical to the reference's own kernels).

Tolerances (float32 path):
  * against the oracle in the GPU evaluation order: rel-L2 <= 1e-6 (only the order of the
    forward ray sums differs);
  * against the reference fixtures: rel-L2 <= 1e-4 and max-abs <= 1e-3 * image peak (the
    parity bar of this path).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
REL_ORACLE = 1e-6
REL_REF = 1e-4
MAXABS_REF = 1e-3

KERNELS = [0, 1]  # xct.KERNELS_TILED, xct.KERNELS_PLAIN


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _run_device(ctx, meas, x0, ang, ss, it, kernels, **kw):
    import xct
    meas = np.asarray(meas, np.float32)
    x0 = np.asarray(x0, np.float32)
    if meas.ndim == 2:
        meas, x0 = meas[None], x0[None]
    dN, pa, px = meas.shape
    _, ny, nx = x0.shape
    plan = xct.OSEMPlan(ctx, nx, ny, px, ang, ss, it, max_batch=dN, kernels=kernels, **kw)
    d_s, d_x = _dev(meas), _dev(x0)
    plan.run_device(d_s, d_x)
    torch.cuda.synchronize()
    out = d_x.cpu().numpy()
    plan.close()
    return out


@pytest.mark.parametrize("kernels", KERNELS)
@pytest.mark.parametrize("name", ["small_64", "odd_48x40", "cfg1_256"])
def test_osem_matches_reference_fixture(gpu_ctx, oracle_lib, name, kernels):
    O = oracle_lib
    f = _load(name)
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    got = _run_device(gpu_ctx, f["meas"], f["x0"], f["angles"], ss, it, kernels)[0]
    ref = f["osem"]
    assert _rel(got, ref) <= REL_REF
    assert np.abs(got - ref).max() <= MAXABS_REF * np.abs(ref).max()
    gpu_order = O.osem_run(f["x0"], f["meas"], f["angles"], ss, it, sub_order=f["sub"], order=O.ORDER_GPU)
    assert _rel(got, gpu_order) <= REL_ORACLE
    # the error against the FP64 run of the same algorithm is stated, not gated
    assert _rel(got, f["osem_f64"]) < 1e-3


@pytest.mark.parametrize("kernels", KERNELS)
def test_forward_projection_matches_oracle(gpu_ctx, oracle_lib, kernels):
    import xct
    O = oracle_lib
    f = _load("odd_48x40")
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, f["angles"], ss, it, kernels=kernels)
    d_x = _dev(f["phantom"][None])
    d_s = torch.zeros((1, pa, px), device="cuda")
    plan.fwd(d_x, d_s)
    torch.cuda.synchronize()
    want = O.projection(f["phantom"], f["angles"], px, order=O.ORDER_GPU)
    got = d_s[0].cpu().numpy()
    assert _rel(got, want) <= REL_ORACLE
    assert _rel(got, f["clean"]) <= 1e-5
    plan.close()


@pytest.mark.parametrize("kernels", KERNELS)
def test_bp_ref_matches_reference_fixture(gpu_ctx, kernels):
    import xct
    f = _load("small_64")
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, f["angles"], ss, it, kernels=kernels)
    d_s = _dev(f["clean"][None])
    d_x = torch.zeros((1, ny, nx), device="cuda")
    plan.bp_ref(d_s, d_x)
    torch.cuda.synchronize()
    # nearest-bin backprojection summed in angle order: bit-identical
    assert np.array_equal(d_x[0].cpu().numpy(), f["bp_all"])
    plan.close()


@pytest.mark.parametrize("kernels", KERNELS)
def test_batch_equals_single_slices(gpu_ctx, oracle_lib, kernels):
    """dN slices in one call (image2d_array layers, GPU.cpp:139-140) give each slice's
    single-call result."""
    from xct import phantom as P
    O = oracle_lib
    n, pa, ss, it = 40, 30, 5, 2
    ang = P.uniform_angles(pa)
    meas = []
    for s in range(3):
        img = P.rasterize_ellipses(P.ellipse_params(n, 4, 10 + s, axes=(2, 10)), n, n)
        meas.append(P.noisy_log_sinogram(O.projection(img, ang, n), 1e4, s))
    meas = np.stack(meas)
    x0 = np.ones((3, n, n), np.float32)
    batched = _run_device(gpu_ctx, meas, x0, ang, ss, it, kernels)
    for s in range(3):
        single = _run_device(gpu_ctx, meas[s], x0[s], ang, ss, it, kernels)[0]
        assert np.array_equal(batched[s], single)
        want = O.osem_run(x0[s], meas[s], ang, ss, it, order=O.ORDER_GPU)
        assert _rel(batched[s], want) <= REL_ORACLE


def test_host_buffer_run_equals_device_run(gpu_ctx):
    import xct
    f = _load("small_64")
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, f["angles"], ss, it, max_batch=2)
    imgs = [f["x0"].copy(), f["x0"].copy()]
    plan.run([f["meas"], f["meas"]], imgs)
    assert np.array_equal(imgs[0], imgs[1])
    dev = _run_device(gpu_ctx, f["meas"], f["x0"], f["angles"], ss, it, 0)[0]
    assert np.array_equal(imgs[0], dev)
    assert plan.last_ms() > 0
    plan.close()


@pytest.mark.parametrize("kernels", KERNELS)
@pytest.mark.parametrize("cover", [False, True])
def test_non_divisible_subsets(gpu_ctx, oracle_lib, kernels, cover):
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, pa, ss, it = 36, 29, 6, 2
    ang = np.sort(np.random.default_rng(3).uniform(0, 180, pa)).astype(np.float32)
    img = P.rasterize_ellipses(P.ellipse_params(n, 4, 4, axes=(2, 8)), n, n)
    meas = P.noisy_log_sinogram(O.projection(img, ang, n), 1e4, 9)
    x0 = np.ones((n, n), np.float32)
    got = _run_device(gpu_ctx, meas, x0, ang, ss, it, kernels,
                      subset_mode=xct.SUBSETS_COVER if cover else xct.SUBSETS_REF)[0]
    want = O.osem_run(x0, meas, ang, ss, it, order=O.ORDER_GPU, cover=cover)
    assert _rel(got, want) <= REL_ORACLE


@pytest.mark.parametrize("kernels", KERNELS)
def test_measured_fetch_avg_and_bad_values(gpu_ctx, oracle_lib, kernels):
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, pa, ss, it = 32, 24, 4, 2
    ang = P.uniform_angles(pa)
    img = P.rasterize_ellipses(P.ellipse_params(n, 3, 5, axes=(2, 8)), n, n)
    meas = P.noisy_log_sinogram(O.projection(img, ang, n), 1e4, 1)
    meas[2, 3] = np.nan
    meas[5, 7] = -3.0
    meas[9, :] = np.inf
    x0 = np.ones((n, n), np.float32)
    for fetch in (xct.FETCH_EXACT, xct.FETCH_AVG2X2):
        got = _run_device(gpu_ctx, meas, x0, ang, ss, it, kernels, fetch_mode=fetch)[0]
        want = O.osem_run(x0, meas, ang, ss, it, order=O.ORDER_GPU, fetch_mode=fetch)
        fin = np.isfinite(want)
        assert np.array_equal(np.isfinite(got), fin)
        assert _rel(got[fin], want[fin]) <= REL_ORACLE


@pytest.mark.parametrize("mode", [1, 2, 3, 4])
def test_sinogram_correction_modes(gpu_ctx, oracle_lib, mode):
    from xct import phantom as P
    O = oracle_lib
    n, pa, ss, it = 32, 20, 4, 1
    ang = P.uniform_angles(pa)
    img = P.rasterize_ellipses(P.ellipse_params(n, 3, 6, axes=(2, 8)), n, n)
    meas = O.projection(img, ang, n)
    x0 = np.ones((n, n), np.float32)
    got = _run_device(gpu_ctx, meas, x0, ang, ss, it, 0, correction_mode=mode)[0]
    want = O.osem_run(x0, O.sino_correction(meas, ang, mode), ang, ss, it, order=O.ORDER_GPU)
    assert _rel(got, want) <= REL_ORACLE


@pytest.mark.parametrize("kernels", KERNELS)
def test_centre_offset_and_wide_detector(gpu_ctx, oracle_lib, kernels):
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, ss, it = 40, 64, 30, 3, 2
    ang = P.uniform_angles(pa)
    img = P.rasterize_ellipses(P.ellipse_params(n, 4, 8, axes=(2, 10)), n, n)
    cx = px * 0.5 + 3.5
    meas = P.noisy_log_sinogram(O.projection(img, ang, px, cx=cx), 1e4, 2)
    x0 = np.ones((n, n), np.float32)
    got = _run_device(gpu_ctx, meas, x0, ang, ss, it, kernels, center_bin=cx)[0]
    want = O.osem_run(x0, meas, ang, ss, it, order=O.ORDER_GPU, cx=cx)
    assert _rel(got, want) <= REL_ORACLE


def test_zero_iterations_leave_image(gpu_ctx):
    f = _load("small_64")
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    x0 = np.random.default_rng(0).uniform(0.5, 1.5, (ny, nx)).astype(np.float32)
    got = _run_device(gpu_ctx, f["meas"], x0, f["angles"], ss, 0, 0)[0]
    assert np.array_equal(got, x0)


def test_errors_are_reported(gpu_ctx):
    import xct
    f = _load("small_64")
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, f["angles"], ss, it, max_batch=1)
    d_s = torch.zeros((2, pa, px), device="cuda")
    d_x = torch.ones((2, ny, nx), device="cuda")
    with pytest.raises(xct.XCTError) as e:
        plan.run_device(d_s, d_x, dN=2)
    assert e.value.code == xct.XCT_E_INVALID and "max_batch" in str(e.value)
    with pytest.raises(xct.XCTError):
        plan.run_device(d_s, d_x, dN=1, sub=[0] * (ss - 1) + [ss])
    with pytest.raises(xct.XCTError):
        xct.OSEMPlan(gpu_ctx, nx, ny, px, f["angles"], pa + 1, it)
    plan.close()
