"""FISTA with compressed sensing on the GPU (xct_fista_*; FISTA_ocl / FISTA_execution,
CT_reconstruction/GPU.cpp:1755-2299) against the oracle, whose restatement is pinned bit for
bit to the reference's own FISTA.cl / AART.cl / reconstShare.cl kernels (tests/
test_oracle_fista.py, tests/golden/fista_64.npz).

Bars: the Lipschitz estimates to 1e-4 relative (the GPU sums the norm in double, the
reference's work-groups in float, and its forward projector uses the fused order); the
reconstructions rel-L2 <= 1e-4 and max-abs <= 1e-3 of the peak, the OS-EM parity bar.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REL, MAXABS = 1e-4, 1e-3


def _check(got, want, what):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    assert np.all(np.isfinite(got)), what
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    mx = np.abs(got - want).max() / np.abs(want).max()
    assert rel <= REL and mx <= MAXABS, "%s: rel-L2 %.3e, max-abs %.3e of peak" % (what, rel, mx)


def _problem(O, n, px, pa, dN, seed):
    from xct import phantom as P
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, dN, count=6, seed=seed)
    meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, px), 1e4, z)
                     for z in range(dN)]).astype(np.float32)
    return ang, meas


@pytest.mark.parametrize("kernels", ["tiled", "plain"])
@pytest.mark.parametrize("own", [False, True])
def test_power_iteration_matches_oracle(gpu_ctx, oracle_lib, kernels, own):
    import xct
    O = oracle_lib
    n, px, pa, ss = 64, 72, 90, 10
    ang = np.arange(pa, dtype=np.float32) * np.float32(180.0 / pa)
    k = xct.KERNELS_TILED if kernels == "tiled" else xct.KERNELS_PLAIN
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, 1, kernels=k)
    got = plan.power_iteration(trials=30, own_layer=own)
    want = O.power_iteration(ang, n, n, px, ss, trials=30, layer_mode=1 if own else 0)
    assert np.all(got > 0)
    np.testing.assert_allclose(got, want, rtol=1e-4)
    plan.close()


def test_power_iteration_partial_work_group(gpu_ctx, oracle_lib):
    """A reduction width that does not divide the image (the reference's norm then covers the
    first (nx / wg) * wg columns and rows only)."""
    import xct
    O = oracle_lib
    n, px, pa, ss = 80, 80, 60, 6
    ang = np.arange(pa, dtype=np.float32) * np.float32(180.0 / pa)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, 1)
    got = plan.power_iteration(trials=8, work_group=64)
    want = O.power_iteration(ang, n, n, px, ss, trials=8, work_group=64)
    np.testing.assert_allclose(got, want, rtol=1e-4)
    plan.close()


@pytest.mark.parametrize("case", ["tiled", "plain", "correction", "update_x", "nondivisible"])
def test_fista_matches_oracle(gpu_ctx, oracle_lib, case):
    import xct
    O = oracle_lib
    n, px, pa, ss, it, dN = 64, 64, 90, 10, 2, 3
    if case == "nondivisible":
        pa, ss = 84, 10  # 84 = 8*10 + 4: FISTAbackProjection reads rows AART1 never writes
    ang, meas = _problem(O, n, px, pa, dN, 90)
    corr = 2 if case == "correction" else 0
    flags = xct.FISTA_UPDATE_X if case == "update_x" else 0
    kernels = xct.KERNELS_PLAIN if case == "plain" else xct.KERNELS_TILED
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, correction_mode=corr, max_batch=dN, kernels=kernels)
    L = O.power_iteration(ang, n, n, px, ss, trials=30)
    plan.set_lipschitz(L)  # the same L on both sides: this test isolates the reconstruction
    x = torch.zeros((dN, n, n), device="cuda")
    plan.fista_run_device(torch.from_numpy(meas).cuda(), x, alpha=1.0, cs_lambda=1e-4, flags=flags)
    torch.cuda.synchronize()
    want = O.fista_run(np.zeros((dN, n, n)), meas, ang, ss, it, L, 1.0, 1e-4, correction_mode=corr,
                       flags=1 if flags else 0)
    _check(x.cpu().numpy(), want, case)
    plan.close()


def test_fista_golden_fixture(gpu_ctx, oracle_lib):
    import xct
    f = dict(np.load(os.path.join(HERE, "golden", "fista_64.npz")))
    nx, ny, px, pa, ss, it, trials = [int(v) for v in f["shape"]]
    dN = f["meas"].shape[0]
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, f["angles"], ss, it, max_batch=dN)
    L = plan.power_iteration(trials=trials)
    np.testing.assert_allclose(L, f["L"], rtol=1e-4)
    for flags, key in ((0, "fista"), (xct.FISTA_UPDATE_X, "fista_update_x")):
        x = torch.zeros((dN, ny, nx), device="cuda")
        plan.fista_run_device(torch.from_numpy(f["meas"]).cuda(), x, alpha=float(f["alpha"][0]),
                              cs_lambda=float(f["cs_lambda"][0]), sub=f["sub"], flags=flags)
        torch.cuda.synchronize()
        _check(x.cpu().numpy(), f[key], key)
    plan.close()


def test_fista_with_exact_adjoint(gpu_ctx, oracle_lib):
    """XCT_FISTA_ADJOINT: the gradient step through the exact adjoint of the forward
    projector over the subset's angles, checked against the same loop composed of oracle
    operators (residual AART1, adjoint, ISTA3D/FISTA3D) with x_{t+1} stored."""
    import xct
    O = oracle_lib
    n, px, pa, ss, it, dN = 64, 64, 90, 10, 2, 2
    ang, meas = _problem(O, n, px, pa, dN, 95)
    L = O.power_iteration(ang, n, n, px, ss, trials=30)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, max_batch=dN)
    plan.set_lipschitz(L)
    x = torch.zeros((dN, n, n), device="cuda")
    plan.fista_run_device(torch.from_numpy(meas).cuda(), x, flags=xct.FISTA_ADJOINT | xct.FISTA_UPDATE_X)
    torch.cuda.synchronize()
    # the same loop from oracle operators
    sub = O.subset_order(ss)
    lam_d = O.lambda_literal(1e-4)
    dest = np.stack([O.backprojection(meas[z], ang, n, n, ss=ss, sub=int(sub[0]), order=O.ORDER_LITERAL)
                     for z in range(dN)])
    xs, w, beta = dest.copy(), dest.copy(), np.zeros_like(dest)
    res = np.zeros_like(meas)
    X, first = xs, True
    f32 = np.float32
    for _ in range(it):
        for s in sub:
            s = int(s)
            Lf = f32(L[s])
            coef = f32(f32(f32(f32(f32(1.0) * f32(ss)) / f32(pa)) / f32(n)) / Lf) * f32(0.5)
            rows = np.arange(s, pa, ss)
            v = np.empty_like(dest)
            for z in range(dN):
                r = O.aart1(X[z], meas[z], ang, ss, s)
                res[z][rows[:pa // ss]] = r[rows[:pa // ss]]
                masked = np.zeros_like(res[z])
                masked[rows] = res[z][rows]
                v[z] = X[z] + coef * O.adjoint(masked, ang, n, n)
            lam = f32(lam_d / float(Lf) * 0.5)
            if first:
                dest = O.ista3d(v, lam)
                X, first = w, False
            else:
                w_new, x_new, b_new = O.fista3d(xs, v, beta, lam)
                w[...] = w_new
                beta = b_new
                dest = x_new
            xs = dest.copy()
    _check(x.cpu().numpy(), xs, "exact adjoint")
    plan.close()


def test_fista_host_buffers_match_device_call(gpu_ctx, oracle_lib):
    """FISTA_thread's form (host arrays in and out) equals the device call."""
    import xct
    O = oracle_lib
    n, px, pa, ss, it, dN = 48, 48, 60, 6, 2, 2
    ang, meas = _problem(O, n, px, pa, dN, 97)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, max_batch=dN)
    plan.power_iteration()
    d_x = torch.zeros((dN, n, n), device="cuda")
    plan.fista_run_device(torch.from_numpy(meas).cuda(), d_x)
    torch.cuda.synchronize()
    outs = [np.full((n, n), np.nan, np.float32) for _ in range(dN)]  # not read
    plan.fista_run([m.copy() for m in meas], outs)
    for z in range(dN):
        assert np.array_equal(outs[z], d_x[z].cpu().numpy())
    plan.close()


def test_fista_256_matches_oracle(gpu_ctx, oracle_lib):
    """The single-slice workload's size (256^2, 180 angles, 256 bins), 10 subsets x 2, two
    slices, L from the GPU power iteration on both sides."""
    import xct
    O = oracle_lib
    n, px, pa, ss, it, dN = 256, 256, 180, 10, 2, 2
    ang, meas = _problem(O, n, px, pa, dN, 99)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, max_batch=dN)
    L = plan.power_iteration()
    np.testing.assert_allclose(L, O.power_iteration(ang, n, n, px, ss, trials=30), rtol=1e-4)
    x = torch.zeros((dN, n, n), device="cuda")
    plan.fista_run_device(torch.from_numpy(meas).cuda(), x)
    torch.cuda.synchronize()
    _check(x.cpu().numpy(), O.fista_run(np.zeros((dN, n, n)), meas, ang, ss, it, L), "256^2")
    plan.close()
