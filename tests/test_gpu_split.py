"""An OS-EM call on two or more slices runs them as two halves on two streams (the second
half on the plan's own stream, with offset views of the plan's ratio, accumulator and
corrected-sinogram buffers).  A batch of 3 (halves of 2 and 1) equals the three slices run
one per call, for both kernel families, with and without a sinogram correction, through the
device and the host-buffer forms (the latter with each half's copies on its own stream); and
the caller's stream sees the finished result."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("kern", ["tiled", "plain"])
@pytest.mark.parametrize("correction", [0, 2])
def test_batch_of_three_equals_single_slices(gpu_ctx, kern, correction):
    import xct
    from xct import phantom as P
    nx, ny, px, pa, ss, it = 96, 80, 110, 48, 4, 2
    ang = np.sort(np.random.default_rng(3).uniform(0, 180, pa)).astype(np.float32)
    k = xct.KERNELS_TILED if kern == "tiled" else xct.KERNELS_PLAIN
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, it, max_batch=3, kernels=k, correction_mode=correction)
    one = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, it, max_batch=1, kernels=k, correction_mode=correction)
    m = max(nx, ny)
    imgs = np.stack([P.rasterize_ellipses(P.ellipse_params(m, 5, z, axes=(3, 20)), m, m)[:ny, :nx] + 0.01
                     for z in range(3)]).astype(np.float32)
    d_i = torch.from_numpy(imgs).cuda()
    sino = torch.empty((3, pa, px), device="cuda")
    plan.fwd(d_i, sino)
    sino = (sino * 1.01 + 0.02).contiguous()  # not the images' own projections
    x = torch.ones((3, ny, nx), device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    plan.run_device(sino, x, stream=s)
    # the default stream waits only for the caller's stream: the library must have joined
    # its second stream back into it
    ev = torch.cuda.Event()
    ev.record(s)
    torch.cuda.current_stream().wait_event(ev)
    got = x.cpu().numpy()
    want = []
    for z in range(3):
        xz = torch.ones((1, ny, nx), device="cuda")
        one.run_device(sino[z:z + 1].contiguous(), xz)
        torch.cuda.synchronize()
        want.append(xz[0].cpu().numpy())
    want = np.stack(want)
    tol = 1e-6 if kern == "tiled" else 0.0  # double atomics add in any order; plain: none
    for z in range(3):
        assert _rel(got[z], want[z]) <= tol, (kern, correction, z)
    # host-buffer form
    out = [np.ones((ny, nx), np.float32) for _ in range(3)]
    plan.run([sino[z].cpu().numpy().copy() for z in range(3)], out)
    for z in range(3):
        assert _rel(out[z], want[z]) <= tol, (kern, correction, z)
    plan.close()
    one.close()


def test_device_call_captures_into_a_cuda_graph(gpu_ctx):
    """A caller can capture xct_osem_run_device -- both halves of the batch and the fork and
    join between its streams -- into a CUDA graph and replay it (small slices gain 10-25 % from
    replay); each replay gives the direct call's result."""
    import xct
    from xct import phantom as P
    n, pa, ss, it = 64, 45, 5, 2
    ang = P.uniform_angles(pa)
    plan = xct.OSEMPlan(gpu_ctx, n, n, n, ang, ss, it, max_batch=3)
    imgs = np.stack([P.rasterize_ellipses(P.ellipse_params(n, 4, z, axes=(3, 14)), n, n) + 0.01
                     for z in range(3)]).astype(np.float32)
    sino = torch.empty((3, pa, n), device="cuda")
    plan.fwd(torch.from_numpy(imgs).cuda(), sino)
    x = torch.ones((3, n, n), device="cuda")
    plan.run_device(sino, x)
    torch.cuda.synchronize()
    want = x.cpu().numpy()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.run_device(sino, x, stream=s)
    for _ in range(2):
        x.fill_(1.0)
        g.replay()
        torch.cuda.synchronize()
        assert _rel(x.cpu().numpy(), want) <= 1e-6
    del g
    plan.close()


@pytest.mark.parametrize("correction", [0, 2])
def test_fbp_host_batch_equals_device(gpu_ctx, correction):
    """xct_fbp_run on a batch of 3 (halves of 2 and 1, each with its own copies on its own
    stream, using the plan's filtered-sinogram and corrected-sinogram buffers from its first
    slice on) equals xct_fbp_run_device on the same slices, bit for bit."""
    import xct
    nx, ny, px, pa = 96, 80, 110, 48
    ang = np.sort(np.random.default_rng(5).uniform(0, 180, pa)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, 4, 1, max_batch=3, correction_mode=correction)
    rng = np.random.default_rng(6)
    sinos = [rng.uniform(0.0, 1.0, (pa, px)).astype(np.float32) for _ in range(3)]
    d_s = torch.from_numpy(np.stack(sinos)).cuda()
    d_x = torch.empty((3, ny, nx), device="cuda")
    plan.fbp(d_s, d_x, zp=256)
    torch.cuda.synchronize()
    want = d_x.cpu().numpy()
    out = [np.full((ny, nx), np.nan, np.float32) for _ in range(3)]
    plan.fbp_run(sinos, out, zp=256)
    for z in range(3):
        assert np.array_equal(out[z], want[z]), z
    plan.close()


@pytest.mark.parametrize("correction", [0, 2])
def test_hybrid_host_batch_equals_device(gpu_ctx, correction):
    """xct_hybrid_run on a batch of 3 (halves with their own copies, each running FBP, base-up
    and OS-EM on the plan's buffers from its first slice on) equals xct_hybrid_run_device on
    the same slices, bit for bit with the plain kernels."""
    import xct
    nx, ny, px, pa, ss = 96, 80, 110, 48, 4
    ang = np.sort(np.random.default_rng(7).uniform(0, 180, pa)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 2, max_batch=3, correction_mode=correction,
                        kernels=xct.KERNELS_PLAIN)
    rng = np.random.default_rng(8)
    sinos = [rng.uniform(0.05, 1.0, (pa, px)).astype(np.float32) for _ in range(3)]
    d_s = torch.from_numpy(np.stack(sinos)).cuda()
    d_x = torch.empty((3, ny, nx), device="cuda")
    plan.hybrid(d_s, d_x, zp=256, it=2)
    torch.cuda.synchronize()
    want = d_x.cpu().numpy()
    out = [np.full((ny, nx), np.nan, np.float32) for _ in range(3)]
    plan.hybrid_run(sinos, out, zp=256, it=2)
    for z in range(3):
        assert np.array_equal(out[z], want[z]), z
    plan.close()
