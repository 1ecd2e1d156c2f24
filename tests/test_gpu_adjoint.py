"""The differentiable projector pair: xct_fwd and its exact adjoint xct_adj.

* dot-product test <A x, y> = <x, A^T y> on 32 seeded (x, y) pairs, 1024^2 image, 720
  angles, 1024 bins, to 1e-5 relative (inner products accumulated in float64);
* A^T against the oracle's scatter adjoint (rel-L2 1e-5: the GPU sums fixed-point
  contributions per window of angles, each rounded at 2^-22 of the window's largest value),
  also for a sinogram of 1e-6-scale values whose centre ray is 1.0 at every angle (rays far
  below their window's largest value keep float precision: checked by linearity on the GPU);
  two runs give identical bits when every ray of a window is within 2^6 of its largest
  (integer sums do not depend on the atomics' order);
* gradient of the Poisson log-likelihood against central finite differences of an FP64
  model (64^2, 90 angles);
* a 50-step unrolled reconstruction: gradients with per-iteration checkpointing equal the
  stored-graph gradients, and the per-step gradient direction A^T(y - Ax) is compared with
  the reference FISTA.cl gradient step (AART1 residual + FISTAbackProjection), which uses a
  nearest-bin floor backprojector instead of the adjoint (the agreement is reported).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _plan(ctx, n, px, pa, ss=1, max_batch=1):
    import xct
    from xct import phantom as P
    return xct.OSEMPlan(ctx, n, n, px, P.uniform_angles(pa), ss, 1, max_batch=max_batch)


def test_dot_product_identity_1024(gpu_ctx):
    n, px, pa = 1024, 1024, 720
    plan = _plan(gpu_ctx, n, px, pa, max_batch=1)
    g = torch.Generator(device="cuda")
    g.manual_seed(4)
    yy, xx = torch.meshgrid(torch.arange(n, device="cuda"), torch.arange(n, device="cuda"), indexing="ij")
    disc = (((xx - n / 2) ** 2 + (yy - n / 2) ** 2) <= (0.45 * n) ** 2).float()
    worst = 0.0
    for k in range(32):
        x = (torch.rand((1, n, n), device="cuda", generator=g) * disc).contiguous()
        y = torch.rand((1, pa, px), device="cuda", generator=g).contiguous()
        ax = torch.empty((1, pa, px), device="cuda")
        aty = torch.empty((1, n, n), device="cuda")
        plan.fwd(x, ax)
        plan.adj(y, aty)
        lhs = float((ax.double() * y.double()).sum())
        rhs = float((x.double() * aty.double()).sum())
        worst = max(worst, abs(lhs - rhs) / abs(lhs))
    assert worst <= 1e-5, worst
    plan.close()


@pytest.mark.parametrize("shape", [(64, 64, 90), (130, 150, 77), (256, 256, 180)])
def test_adjoint_matches_oracle(gpu_ctx, oracle_lib, shape):
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, px, pa = shape
    ang = P.uniform_angles(pa)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, 1, 1)
    y = np.random.default_rng(pa).uniform(0, 1, (pa, px)).astype(np.float32)
    out = torch.empty((1, n, n), device="cuda")
    plan.adj(torch.from_numpy(y).cuda().reshape(1, pa, px).contiguous(), out)
    torch.cuda.synchronize()
    got = out[0].cpu().numpy().astype(np.float64)
    want = O.adjoint(y, ang, n, n, dtype=np.float64)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-5
    plan.close()


def test_poisson_likelihood_gradient_matches_finite_differences(gpu_ctx, oracle_lib):
    import xct.autograd as xa
    from xct import phantom as P
    O = oracle_lib
    n, px, pa = 64, 64, 90
    ang = P.uniform_angles(pa)
    plan = _plan(gpu_ctx, n, px, pa)
    rng = np.random.default_rng(9)
    x = (0.05 + 0.1 * rng.uniform(size=(n, n))).astype(np.float64)
    y = O.projection(x * 1.2, ang, px, dtype=np.float64)

    def nll64(v):
        p = O.projection(v, ang, px, dtype=np.float64)
        m = p > 0
        return float(np.sum(p[m] - y[m] * np.log(p[m])))

    xt = torch.from_numpy(x.astype(np.float32)).cuda().reshape(1, n, n).requires_grad_(True)
    yt = torch.from_numpy(y.astype(np.float32)).cuda().reshape(1, pa, px)
    loss = xa.poisson_nll(xt, yt, plan)
    loss.backward()
    grad = xt.grad[0].cpu().numpy().astype(np.float64)
    h = 1e-4
    errs = []
    for (i, j) in rng.integers(8, n - 8, size=(16, 2)):
        e = np.zeros_like(x)
        e[i, j] = h
        fd = (nll64(x + e) - nll64(x - e)) / (2 * h)
        errs.append(abs(fd - grad[i, j]) / max(abs(fd), 1e-3))
    assert max(errs) <= 1e-3, errs
    plan.close()


def test_unrolled_reconstruction_checkpointing_and_reference_gradient(gpu_ctx, oracle_lib):
    import xct.autograd as xa
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, iters = 64, 64, 90, 50
    ang = P.uniform_angles(pa)
    plan = _plan(gpu_ctx, n, px, pa)
    truth = P.rasterize_ellipses(P.ellipse_params(n, 5, 7, axes=(3, 15)), n, n)
    y_np = O.projection(truth, ang, px)
    y = torch.from_numpy(y_np).cuda().reshape(1, pa, px)
    step = 1.0 / (pa * n * 1.5)  # below 1/||A||^2 for this geometry
    grads = []
    for ckpt in (True, False):
        st = torch.tensor(step, device="cuda", requires_grad=True)
        yy = y.clone().requires_grad_(True)
        x = xa.unrolled_gradient_descent(torch.zeros((1, n, n), device="cuda"), yy, plan, st, iters,
                                         checkpoint_each=ckpt)
        loss = ((x - torch.from_numpy(truth).cuda()) ** 2).sum()
        loss.backward()
        grads.append((float(st.grad), yy.grad.clone()))
    (g1, gy1), (g2, gy2) = grads
    # recomputation repeats the forward pass; the adjoint's float atomics (rays far below their
    # window's largest value) sum in a run-dependent order, so the two graphs agree to rounding
    assert abs(g1 - g2) <= 1e-3 * abs(g2)
    assert float((gy1 - gy2).norm() / gy2.norm()) <= 1e-3

    # the gradient direction of one step vs the reference FISTA.cl gradient step
    x0 = np.full((n, n), 0.05, np.float32)
    res = O.aart1(x0, y_np, ang, 1, 0)
    ref_step = O.fista_bp(x0, res, ang, 1, 0, 1.0, 1.0) - x0   # x + c * B_floor(y - A x)
    xt = torch.from_numpy(x0).cuda().reshape(1, n, n)
    r = torch.from_numpy(y_np).cuda().reshape(1, pa, px) - xa.project(xt, plan)
    ours = xa.backproject(r, plan)[0].cpu().numpy()
    cos = float(np.sum(ours * ref_step) / (np.linalg.norm(ours) * np.linalg.norm(ref_step)))
    assert cos > 0.95, cos
    plan.close()


def test_adjoint_high_dynamic_range(gpu_ctx, oracle_lib):
    """One bright ray (1.0) per angle, through the image centre, among rays of ~1e-6: the
    tiles round the centre see a bright ray in every window of angles.  Rounding the small
    rays to the bright window's fixed-point unit (2^-21) puts texels off the bright lines ~20%
    off; the small rays keep float precision instead.

    Geometry-free check: adj(y) = adj(bright rays) + adj(small rays) texel by texel, all three
    on the GPU, to float summation noise (the bright taps round identically in the first two,
    so only mixing magnitudes in one window could break it).  Against the float64 oracle the
    texels off the blob agree to 2e-3: the float32 sample coordinates alone move them by up to
    ~6e-4 (a plain float scatter measures the same on this input)."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, px, pa = 128, 128, 720
    ang = P.uniform_angles(pa)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, 1, 1)
    rng = np.random.default_rng(21)
    y = (rng.uniform(1.0, 2.0, (pa, px)) * 1e-6).astype(np.float32)
    bright = np.zeros_like(y)
    bright[:, px // 2] = 1.0
    small = y.copy()
    small[:, px // 2] = 0.0
    y[:, px // 2] = 1.0

    def adj(v):
        out = torch.empty((1, n, n), device="cuda")
        plan.adj(torch.from_numpy(v).cuda().reshape(1, pa, px).contiguous(), out)
        torch.cuda.synchronize()
        return out[0].cpu().numpy().astype(np.float64)

    got, got_b, got_s = adj(y), adj(bright), adj(small)
    yy, xx = np.mgrid[0:n, 0:n]
    far = np.hypot(xx + 0.5 - n / 2, yy + 0.5 - n / 2) > 6  # off the bright blob
    # the small rays of adj(y) go through float atomics into the running total: ~3600 rounded
    # adds per texel at 2^-24 each bound the difference by ~2e-4 (measured 4e-5 at most)
    lin = np.abs(got - (got_b + got_s))[far] / np.abs(got)[far]
    assert lin.max() <= 2e-4, lin.max()
    want = O.adjoint(y, ang, n, n, dtype=np.float64)
    rel = np.abs(got - want)[far] / np.abs(want)[far]
    assert rel.max() <= 2e-3, rel.max()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 2e-5
    plan.close()


def test_adjoint_is_deterministic(gpu_ctx):
    """Integer accumulation per window: with every ray within 2^6 of its window's largest
    value, the same input gives the same bits every run, on an odd shape with an off-centre
    axis."""
    import xct
    nx, ny, px, pa = 150, 97, 170, 61
    ang = np.sort(np.random.default_rng(8).uniform(0, 180, pa)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, 1, 1, center_bin=px * 0.5 + 2.25, max_batch=2)
    g = torch.Generator(device="cuda")
    g.manual_seed(4)
    y = torch.rand((2, pa, px), device="cuda", generator=g) + 1.0  # in [1, 2)
    a = torch.empty((2, ny, nx), device="cuda")
    b = torch.empty_like(a)
    plan.adj(y, a)
    plan.adj(y, b)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    plan.close()


def test_unrolled_reconstruction_at_operator_size(gpu_ctx, oracle_lib):
    """The differentiable pair at the operator workload's size (1024^2, 720 angles, 1024
    bins): a 50-step unrolled gradient reconstruction, checkpointed every iteration and not,
    gives the same gradients (to the rounding of the adjoint's float-atomic rays) while the
    checkpointed graph keeps less device memory; and the reference's own gradient step at that
    size -- one FISTA_execution iteration of one subset (AART1 residual, FISTAbackProjection,
    ISTA3D; GPU.cpp:1755-1924) -- matches the oracle's restatement of FISTA.cl/AART.cl."""
    import xct
    import xct.autograd as xa
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, iters = 1024, 1024, 720, 50
    ang = P.uniform_angles(pa)
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, 1, 1, max_batch=1)
    truth_np = P.rasterize_ellipses(P.ellipse_params(n, 8, 11, axes=(20, 240), mu=(0.001, 0.01)), n, n)
    truth = torch.from_numpy(truth_np).cuda().reshape(1, n, n)
    y = torch.empty((1, pa, px), device="cuda")
    plan.fwd(truth, y)
    step = 1.0 / (pa * n * 1.5)
    grads, peaks = [], []
    for ckpt in (True, False):
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        st = torch.tensor(step, device="cuda", requires_grad=True)
        yy = y.clone().requires_grad_(True)
        x = xa.unrolled_gradient_descent(torch.zeros((1, n, n), device="cuda"), yy, plan, st, iters,
                                         checkpoint_each=ckpt)
        loss = ((x - truth) ** 2).sum()
        loss.backward()
        torch.cuda.synchronize()
        peaks.append(torch.cuda.max_memory_allocated() - base)
        grads.append((float(st.grad), yy.grad.clone()))
        del x, loss, yy, st
    (g1, gy1), (g2, gy2) = grads
    assert np.isfinite(g1) and abs(g1 - g2) <= 1e-3 * abs(g2)
    assert float((gy1 - gy2).norm() / gy2.norm()) <= 1e-3
    # checkpointed: one iterate per step (4 MB) instead of the iterate, its residual
    # projection and the clamp's mask (measured 238 MB against 443 MB)
    assert peaks[0] < 0.65 * peaks[1], peaks
    # the reference gradient step (FISTAbackProjection, floor rule) against the oracle
    L = plan.power_iteration(trials=10)
    meas = y.cpu().numpy()
    x = torch.zeros((1, n, n), device="cuda")
    plan.fista_run_device(y, x, it=1)
    torch.cuda.synchronize()
    want = O.fista_run(np.zeros((1, n, n), np.float32), meas, ang, 1, 1, L)
    got = x.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel <= 1e-4, rel
    plan.close()
