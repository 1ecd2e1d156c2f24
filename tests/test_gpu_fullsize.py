"""Parity at the full per-slice workload size (2048x2048 image, 1500 angles over 180 deg, 2048
bins, 15 subsets x 4 iterations), where the CPU oracle takes minutes per slice.  Checked
through properties that do not depend on size:

  * the tiled kernels against the plain kernels, which evaluate the reference's launch shape
    and are bit-identical to the oracle's GPU order (tested at every small size): the OS-EM
    parity bar, rel-L2 <= 1e-4 and max-abs <= 1e-3 of the peak;
  * the forward projector is linear: A(x + 2y) = A x + 2 A y to float rounding;
  * the exact adjoint: <A x, y> = <x, A^T y> to 1e-5 relative;
  * OS-EM is equivariant under a common power-of-two scale of data and initial image (the
    update is multiplicative; only the 1e-6 floor and the 1e-4 pass-through threshold do not
    scale, which moves background values only);
  * reslicing with no shifts is an exact transpose.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

N, PA, SS, IT = 2048, 1500, 15, 4


def _rel(a, b):
    a = a.double()
    b = b.double()
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


@pytest.fixture(scope="module")
def fullsize(gpu_ctx):
    import xct
    from xct import phantom as P
    ang = P.uniform_angles(PA)
    plan = xct.OSEMPlan(gpu_ctx, N, N, N, ang, SS, IT, max_batch=1)
    pars = P.ellipsoid_params(N, 100, 30, 2, mu=(0.005, 0.1))
    img = P.ellipsoid_slice(pars, 50, N, N, torch_device="cuda").reshape(1, N, N).contiguous()
    clean = torch.empty((1, PA, N), device="cuda")
    plan.fwd(img, clean)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    meas = P.noisy_log_sinogram_torch(clean[0], 5e4, generator=gen).reshape(1, PA, N).contiguous()
    yield {"plan": plan, "ang": ang, "img": img, "clean": clean, "meas": meas}
    plan.close()


def test_fullsize_tiled_matches_plain_kernels(gpu_ctx, fullsize):
    import xct
    ang, meas = fullsize["ang"], fullsize["meas"]
    plain = xct.OSEMPlan(gpu_ctx, N, N, N, ang, SS, IT, max_batch=1, kernels=xct.KERNELS_PLAIN)
    xp = torch.ones((1, N, N), device="cuda")
    plain.run_device(meas, xp)
    xt = torch.ones((1, N, N), device="cuda")
    fullsize["plan"].run_device(meas, xt)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(xt).all())
    assert _rel(xt, xp) <= 1e-4
    assert float((xt - xp).abs().max()) <= 1e-3 * float(xp.abs().max())
    plain.close()


def test_fullsize_forward_is_linear(fullsize):
    plan, img = fullsize["plan"], fullsize["img"]
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    y = torch.rand((1, N, N), device="cuda", generator=g)
    a = torch.empty((1, PA, N), device="cuda")
    b = torch.empty_like(a)
    c = torch.empty_like(a)
    plan.fwd(img, a)
    plan.fwd(y, b)
    plan.fwd((img + 2.0 * y).contiguous(), c)
    torch.cuda.synchronize()
    assert _rel(c, a + 2.0 * b) <= 1e-6


def test_fullsize_adjoint_dot_product(fullsize):
    plan = fullsize["plan"]
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    x = torch.rand((1, N, N), device="cuda", generator=g)
    y = torch.rand((1, PA, N), device="cuda", generator=g)
    ax = torch.empty((1, PA, N), device="cuda")
    aty = torch.empty((1, N, N), device="cuda")
    plan.fwd(x, ax)
    plan.adj(y, aty)
    torch.cuda.synchronize()
    lhs = float((ax.double() * y.double()).sum())
    rhs = float((x.double() * aty.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_fullsize_osem_scale_equivariance(fullsize):
    plan, meas = fullsize["plan"], fullsize["meas"]
    x1 = torch.ones((1, N, N), device="cuda")
    plan.run_device(meas, x1, it=1)
    x2 = torch.full((1, N, N), 4.0, device="cuda")
    plan.run_device((meas * 4.0).contiguous(), x2, it=1)
    torch.cuda.synchronize()
    assert _rel(x2, 4.0 * x1) <= 1e-4
    assert bool((x1 >= 0).all()) and bool((x2 >= 0).all())


def test_fullsize_reslice_is_a_transpose(gpu_ctx):
    import xct
    rows = 8
    g = torch.Generator(device="cuda")
    g.manual_seed(9)
    mt = torch.rand((PA, rows, N), device="cuda", generator=g)
    rp = xct.ReslicePlan(gpu_ctx, N, rows, PA)
    out = torch.empty((rows, PA, N), device="cuda")
    rp.reslice(mt, out)
    torch.cuda.synchronize()
    assert torch.equal(out, mt.transpose(0, 1))
    rp.close()
