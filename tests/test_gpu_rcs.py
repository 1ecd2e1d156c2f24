"""Rotation-centre search (RotationCenterSearch/) on the GPU through the C ABI.

Tolerances: rotCenterShift is bit-exact (same sampler arithmetic).  The focus index's
per-pixel terms are the reference's operation for operation; its image-wide sums are taken
in double, so it is held to 1e-6 of the oracle's double sums and 1e-5 of the reference's
float work-group order.  The one-iteration OS-EM images carry the OS-EM parity bar
(1e-4 rel-L2), which moves the indices by ~1e-5."""
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


def _plan(ctx, f, max_batch):
    import xct
    n_img, px, pa, ss, n, L = [int(v) for v in f["shape"]]
    return xct.OSEMPlan(ctx, n_img, n_img, px, f["angles"], ss, 1, max_batch=max_batch)


def test_rot_center_shift_bit_exact(gpu_ctx):
    f = _load("rcs_64")
    n = int(f["shape"][4])
    start, step, _ = [float(v) for v in f["shift"]]
    plan = _plan(gpu_ctx, f, 1)
    d_s = torch.from_numpy(f["sino"]).cuda().contiguous()
    d_o = torch.zeros((n,) + f["sino"].shape, device="cuda")
    plan.rot_center_shift(d_s, d_o, start, step)
    torch.cuda.synchronize()
    assert np.array_equal(d_o.cpu().numpy(), f["shifted"])
    plan.close()


def test_focus_index_matches_oracle(gpu_ctx):
    f = _load("rcs_64")
    n = int(f["shape"][4])
    start, step, _ = [float(v) for v in f["shift"]]
    ang = f["angles"]
    plan = _plan(gpu_ctx, f, 4)  # n > max_batch: chunked
    d_i = torch.from_numpy(f["imgs"]).cuda().contiguous()
    d_f = torch.zeros(n, device="cuda")
    plan.focus_index(d_i, d_f, start, step, float(ang[0]), float(ang[-1]))
    torch.cuda.synchronize()
    got = d_f.cpu().numpy().astype(np.float64)
    assert np.abs(got / f["findex_f64"] - 1).max() <= 1e-6
    assert np.abs(got / f["findex"] - 1).max() <= 1e-5
    # a sub-range with its shift offset gives the same indices
    d_f2 = torch.zeros(n - 3, device="cuda")
    plan.focus_index(d_i[3:].contiguous(), d_f2, start, step, float(ang[0]), float(ang[-1]), offset=3)
    torch.cuda.synchronize()
    assert np.array_equal(d_f2.cpu().numpy(), d_f.cpu().numpy()[3:])
    plan.close()


@pytest.mark.parametrize("max_batch", [9, 4])
def test_search_matches_oracle(gpu_ctx, max_batch):
    f = _load("rcs_64")
    n_img, px, pa, ss, n, L = [int(v) for v in f["shape"]]
    start, step, _ = [float(v) for v in f["shift"]]
    plan = _plan(gpu_ctx, f, max_batch)
    d_s = torch.from_numpy(f["sino"]).cuda().contiguous()
    d_i = torch.zeros((n, n_img, n_img), device="cuda")
    fi, best = plan.rot_center_search(d_s, d_i, start, step)
    imgs = d_i.cpu().numpy()
    for i in range(n):
        assert _rel(imgs[i], f["imgs"][i]) <= 1e-4, i
    assert np.abs(fi / f["findex_f64"] - 1).max() <= 1e-4
    assert best == int(np.argmin(f["findex"]))
    plan.close()


def test_search_finds_known_centre_offset(gpu_ctx, oracle_lib):
    """A 128x128 slice projected about px/2 + 2 (180 angles, I0 = 1e6): shifts -5..5 in
    steps of 1 pick +2, as the oracle does."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, pa, off = 128, 180, 2.0
    img = P.rasterize_ellipses(P.ellipse_params(n, 8, 2, axes=(4, n / 5)), n, n)
    ang = P.uniform_angles(pa)
    sino = P.noisy_log_sinogram(O.projection(img, ang, n, cx=n / 2 + off), 1e6, 3)
    plan = xct.OSEMPlan(gpu_ctx, n, n, n, ang, 10, 1, max_batch=11)
    d_s = torch.from_numpy(sino).cuda().contiguous()
    d_i = torch.zeros((11, n, n), device="cuda")
    fi, best = plan.rot_center_search(d_s, d_i, -5.0, 1.0)
    shifts = O.shift_values(-5.0, 1.0, 11)
    assert shifts[best] == off, (fi, best)
    plan.close()


def test_search_argument_errors(gpu_ctx):
    import xct
    plan = xct.OSEMPlan(gpu_ctx, 32, 32, 32, np.arange(20, dtype=np.float32) * 9, 4, 1)
    d_s = torch.zeros((20, 32), device="cuda")
    with pytest.raises(xct.XCTError):
        plan.rot_center_search(d_s, torch.zeros((0, 32, 32), device="cuda"), 0.0, 1.0, n=0)
    with pytest.raises(xct.XCTError):
        plan.rot_center_search(d_s, torch.zeros((2, 32, 32), device="cuda"), float("nan"), 1.0)
    plan.close()
