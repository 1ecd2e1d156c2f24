"""Seeded random geometries through both OS-EM kernels, against the oracle in the GPU
evaluation order (OSEM.cl:38-105).  Each case draws: sizes 17..333 (odd, non-square), 16..300
bins, 5..150 angles over 180, 200 or 360 degrees in arbitrary or sorted order with one angle
repeated, 1..12 subsets (mostly not dividing the angle count), a rotation centre up to 6 bins
off the middle, and a forward tile size and angle chunk (1..128) for the tiled kernels.  The
phantom leaves empty rays, so OSEM1's small-projection branch (ratio = measured value) runs too.

* OSEM2 given the oracle's ratio image is bit-identical (same bins, same angle order);
* OSEM1's ratio rows are bit-identical for the plain kernels and within 5e-6 rel-L2 (1e-4 per
  bin) for the tiled ones, whose per-tile partial ray sums meet in double; rows outside the
  subset stay untouched;
* the FBP backprojector on the same geometries is bit-identical to backProjectionFBP;
* the exact adjoint passes the dot-product test against the forward projector and matches
  the oracle's scatter adjoint.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

CASES = 16


def _geometry(seed):
    rng = np.random.default_rng(1000 + seed)
    nx, ny = int(rng.integers(17, 334)), int(rng.integers(17, 334))
    px, pa = int(rng.integers(16, 301)), int(rng.integers(5, 151))
    ss = int(rng.integers(1, min(12, pa) + 1))
    span = float(rng.choice([180.0, 200.0, 360.0]))
    ang = rng.uniform(0.0, span, pa).astype(np.float32)
    if rng.uniform() < 0.5:
        ang = np.sort(ang)
    ang[1] = ang[0]  # a repeated angle
    cx = px * 0.5 + float(rng.uniform(-6.0, 6.0))
    tile = int(rng.choice([44, 60, 76, 92]))
    chunk = int(rng.choice([1, 7, 16, 33, 64, 128]))
    subs = sorted(set(int(s) for s in rng.integers(0, ss, 3)))
    return nx, ny, px, pa, ss, ang, cx, tile, chunk, subs, rng


def _image(nx, ny, rng):
    from xct import phantom as P
    m = max(nx, ny)
    img = P.rasterize_ellipses(P.ellipse_params(m, 6, int(rng.integers(0, 1 << 30)), axes=(2, m / 5)), m, m)
    y0, x0 = (m - ny) // 2, (m - nx) // 2  # the centre, where the ellipses are
    return np.ascontiguousarray(img[y0:y0 + ny, x0:x0 + nx], np.float32)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.mark.parametrize("kernels", [0, 1])
@pytest.mark.parametrize("seed", range(CASES))
def test_random_geometry_parity(gpu_ctx, oracle_lib, seed, kernels):
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, ang, cx, tile, chunk, subs, rng = _geometry(seed)
    img = _image(nx, ny, rng)
    meas = O.projection(img, ang, px, cx=cx) * np.float32(1.05) + np.float32(0.003)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, ss, 1, center_bin=cx, kernels=kernels)
    if kernels == xct.KERNELS_TILED:
        plan.set_tuning(tile, chunk)
    where = "case %d (nx %d ny %d px %d pa %d ss %d cx %.3f tile %d chunk %d)" % (
        seed, nx, ny, px, pa, ss, cx, tile, chunk)
    x = (img * np.float32(0.7) + np.float32(0.2)).astype(np.float32)
    d_img, d_meas = _dev(img[None]), _dev(meas[None])
    for sub in subs:
        # OSEM1
        d_r = torch.full((1, pa, px), -7.0, device="cuda")
        plan.osem1(sub, d_img, d_meas, d_r)
        torch.cuda.synchronize()
        got = d_r[0].cpu().numpy()
        want = O.osem1(img, meas, ang, ss, sub, cx=cx, order=O.ORDER_GPU)
        rows = np.arange(sub, sub + (pa // ss) * ss, ss)
        others = np.setdiff1d(np.arange(pa), rows)
        assert np.all(got[others] == -7.0), where + ": rows outside the subset were written"
        g, w = got[rows].astype(np.float64), want[rows].astype(np.float64)
        if kernels == xct.KERNELS_PLAIN:
            assert np.array_equal(g, w), where
        else:
            assert np.linalg.norm(g - w) / np.linalg.norm(w) <= 5e-6, where
            assert np.max(np.abs(g - w) / np.maximum(np.abs(w), 1e-30)) <= 1e-4, where
        # OSEM2 on the oracle's ratio
        ratio = O.osem1(x, meas, ang, ss, sub, cx=cx, order=O.ORDER_GPU)
        want2 = O.osem2(x, ratio, ang, ss, sub, cx=cx, order=O.ORDER_GPU)
        d_x = _dev(x[None])
        plan.osem2(sub, d_x, _dev(ratio[None]))
        torch.cuda.synchronize()
        got2 = d_x[0].cpu().numpy()
        bad = np.argwhere(got2 != want2)
        assert bad.size == 0, "%s, subset %d: %d pixels differ, first %s" % (where, sub, len(bad), bad[:5].tolist())
        x = want2
    plan.close()


@pytest.mark.parametrize("seed", range(CASES))
def test_random_geometry_fbp_backprojection(gpu_ctx, oracle_lib, seed):
    """backProjectionFBP (FBP.cl:164-188) on the same random geometries, two slices per call
    of normal-distributed filtered sinograms: bit-identical to the oracle (partial edge tiles,
    windows bounded by the tile corners at every angle, bins off the detector)."""
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, ang, cx, tile, chunk, subs, rng = _geometry(seed)
    fprj = rng.normal(0.0, 1.0, (2, pa, px)).astype(np.float32)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, 1, 1, center_bin=cx, max_batch=2)
    d_i = torch.zeros((2, ny, nx), device="cuda")
    plan.fbp_backproject(_dev(fprj), d_i)
    torch.cuda.synchronize()
    for z in range(2):
        got = d_i[z].cpu().numpy()
        want = O.bp_fbp(fprj[z], ang, nx, ny, cx=cx)
        bad = np.argwhere(got != want)
        assert bad.size == 0, "case %d slice %d: %d pixels differ, first %s" % (seed, z, len(bad), bad[:5].tolist())
    plan.close()


@pytest.mark.parametrize("seed", range(CASES))
def test_random_geometry_adjoint(gpu_ctx, oracle_lib, seed):
    """The exact adjoint on the same random geometries: <A x, y> = <x, A^T y> to 1e-5 (inner
    products in float64) with the forward projector, and A^T y against the oracle's scatter
    adjoint to 1e-5 rel-L2."""
    import xct
    O = oracle_lib
    nx, ny, px, pa, ss, ang, cx, tile, chunk, subs, rng = _geometry(seed)
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, 1, 1, center_bin=cx)
    x = rng.uniform(0.0, 1.0, (1, ny, nx)).astype(np.float32)
    y = rng.uniform(0.0, 1.0, (1, pa, px)).astype(np.float32)
    ax = torch.empty((1, pa, px), device="cuda")
    aty = torch.empty((1, ny, nx), device="cuda")
    plan.fwd(_dev(x), ax)
    plan.adj(_dev(y), aty)
    torch.cuda.synchronize()
    ax, aty = ax.cpu().numpy().astype(np.float64), aty.cpu().numpy().astype(np.float64)
    lhs = float(np.sum(ax * y))
    rhs = float(np.sum(x * aty))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs), (seed, lhs, rhs)
    want = O.adjoint(y[0], ang, nx, ny, cx=cx, dtype=np.float64)
    assert np.linalg.norm(aty[0] - want) / np.linalg.norm(want) <= 1e-5, seed
    plan.close()
