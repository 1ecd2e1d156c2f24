"""CPU tests of the oracle: pinned against the reference's own kernels (when the reference
checkout is present), against the committed golden fixtures, and against known answers."""
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _ref_subset_order(ss):
    """Direct transcription of the loop at CT_reconstruction/GPU.cpp:564-582."""
    sub = [0] * ss
    k = sum((ss >> i) & 1 for i in range(32))
    if k == 1:
        m1 = 0
        sub[m1] = 0
        m1 += 1
        i, m2 = ss, 1
        while i > 1:
            for j in range(m2):
                sub[m1] = sub[j] + i // 2
                m1 += 1
            i //= 2
            m2 *= 2
    else:
        sub = list(range(ss))
    return sub


@pytest.mark.parametrize("ss", [1, 2, 3, 4, 8, 10, 15, 16, 20, 32, 64, 100])
def test_subset_order_matches_reference_loop(oracle_lib, ss):
    assert list(oracle_lib.subset_order(ss)) == _ref_subset_order(ss)


@pytest.mark.parametrize("name", ["small_64", "odd_48x40", "cfg1_256"])
def test_oracle_reproduces_golden(oracle_lib, name):
    O = oracle_lib
    f = _load(name)
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    out = O.osem_run(f["x0"], f["meas"], f["angles"], ss, it, sub_order=f["sub"], order=O.ORDER_LITERAL)
    assert np.array_equal(out, f["osem"])
    clean = O.projection(f["phantom"], f["angles"], px, order=O.ORDER_LITERAL)
    assert np.array_equal(clean, f["clean"])
    r0 = O.osem1(f["x0"], f["meas"], f["angles"], ss, int(f["sub"][0]), order=O.ORDER_LITERAL)
    assert np.array_equal(r0, f["ratio0"])
    u0 = O.osem2(f["x0"], r0, f["angles"], ss, int(f["sub"][0]), order=O.ORDER_LITERAL)
    assert np.array_equal(u0, f["upd0"])
    bp = O.backprojection(f["clean"], f["angles"], nx, ny, 1, 0, order=O.ORDER_LITERAL)
    assert np.array_equal(bp, f["bp_all"])


@pytest.mark.parametrize("name", ["small_64", "odd_48x40", "cfg1_256"])
def test_gpu_order_close_to_literal(oracle_lib, name):
    """The CUDA kernels' evaluation order (canonical forward, literal backprojector bins)
    stays within 1e-5 rel-L2 of the reference order after the full run."""
    O = oracle_lib
    f = _load(name)
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    out = O.osem_run(f["x0"], f["meas"], f["angles"], ss, it, sub_order=f["sub"], order=O.ORDER_GPU)
    assert _rel(out, f["osem"]) < 1e-5
    assert np.abs(out - f["osem"]).max() <= 1e-4 * np.abs(f["osem"]).max()


def test_fp64_companion_stated(oracle_lib):
    f = _load("cfg1_256")
    # FP32 vs FP64 of the same algorithm (a reported figure, not a gate)
    e = _rel(f["osem"], f["osem_f64"])
    assert 0 < e < 1e-3


_REF_SHAPES = [(64, 64, 64, 90, 10), (48, 40, 56, 36, 4)]


@pytest.mark.parametrize("shape", _REF_SHAPES)
def test_oracle_bit_identical_to_reference_kernels(oracle_lib, shape):
    """oracle/_ref: the reference's OSEM.cl and reconstShare.cl compiled through the
    OpenCL-C shim.  Only where the reference checkout exists."""
    O = oracle_lib
    if not O.ref_available():
        pytest.skip("reference checkout not present")
    from xct import phantom as P
    nx, ny, px, pa, ss = shape
    m = max(nx, ny)
    img = P.rasterize_ellipses(P.ellipse_params(m, 8, 3, axes=(2, 15)), nx, ny)
    ang = (np.sort(np.random.default_rng(5).uniform(0, 180, pa))).astype(np.float32)
    ref = O.RefKernels(*shape)
    meas = P.noisy_log_sinogram(O.projection(img, ang, px, order=O.ORDER_LITERAL), 1e4, 3)
    meas[3, 5] = np.nan
    meas[7, 9] = -1.0
    sub = O.subset_order(ss)
    x0 = np.full((ny, nx), 0.5, np.float32)
    for fetch in (0, 1):
        r = ref.osem_execution(x0[None], meas[None], ang, sub, 2, fetch_mode=fetch)[0]
        o = O.osem_run(x0, meas, ang, ss, 2, sub_order=sub, order=O.ORDER_LITERAL, fetch_mode=fetch)
        assert np.array_equal(r, o), "fetch mode %d" % fetch
    for sub0 in range(ss):
        rp = ref.projection(img, ang, sub0)
        op = O.projection(img, ang, px, ss=ss, sub=sub0, order=O.ORDER_LITERAL)
        rows = np.arange(sub0, sub0 + (pa // ss) * ss, ss)
        assert np.array_equal(rp[rows], op[rows])
        rb = ref.backprojection(meas, ang, sub0)
        ob = O.backprojection(meas, ang, nx, ny, ss, sub0, order=O.ORDER_LITERAL)
        assert np.array_equal(rb, ob)


def test_kat_zero_degree_projection_is_column_sums(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(0)
    img = rng.uniform(0, 1, (32, 32)).astype(np.float32)
    p = O.projection(img, np.array([0.0], np.float32), 32)
    np.testing.assert_allclose(p[0], img.sum(axis=0), rtol=1e-5)


def test_kat_ninety_degree_projection_is_row_sums(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(1)
    img = rng.uniform(0, 1, (32, 32)).astype(np.float32)
    p = O.projection(img, np.array([90.0], np.float32), 32)
    # x = Yc*sin + nx/2 runs along the image rows and y = -Xc + ny/2, so bin X sums row
    # 32 - X (bin 0 looks at row 32, outside the image)
    rows = img.sum(axis=1)
    want = np.array([rows[32 - X] if 32 - X < 32 else 0.0 for X in range(32)], np.float32)
    np.testing.assert_allclose(p[0], want, rtol=1e-4, atol=1e-4)


def test_kat_disc_chord_lengths(oracle_lib):
    O = oracle_lib
    n, r = 128, 40.0
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    img = (((x - n / 2) ** 2 + (y - n / 2) ** 2) <= r * r).astype(np.float32)
    ang = np.array([0.0, 30.0, 77.0], np.float32)
    p = O.projection(img, ang, n)
    X = np.arange(n) - n / 2
    chord = 2 * np.sqrt(np.maximum(r * r - X ** 2, 0))
    inner = np.abs(X) < r - 3
    for k in range(3):
        assert np.abs(p[k][inner] - chord[inner]).max() < 2.0
        assert abs(p[k].sum() - math.pi * r * r) / (math.pi * r * r) < 0.02


def test_kat_consistent_uniform_data_is_a_fixed_point(oracle_lib):
    """A uniform image with its own projections as data keeps a ratio of 1 and is not
    changed by an OS-EM step where every pixel's bins land on the detector."""
    O = oracle_lib
    n, px, pa, ss = 32, 48, 20, 4
    x = np.full((n, n), 0.7, np.float32)
    ang = np.arange(pa, dtype=np.float32) * (180.0 / pa)
    meas = O.projection(x, ang, px)
    r = O.osem1(x, meas, ang, ss, 0)
    rows = np.arange(0, pa, ss)
    hit = meas[rows] >= 1e-4  # rays that miss the image keep the 1e-6 floor
    assert hit.sum() > rows.size * n
    np.testing.assert_allclose(r[rows][hit], 1.0, rtol=1e-6)
    # below 1e-4 the measured value passes through, floored at 1e-6 (OSEM.cl:64-66)
    want = np.maximum(meas[rows][~hit], np.float32(1e-6))
    assert np.array_equal(r[rows][~hit], want)
    out = O.osem_run(x, meas, ang, ss, 2)
    np.testing.assert_allclose(out, x, rtol=1e-5)


def test_nonfinite_and_negative_measurements(oracle_lib):
    """OSEM1 floors measured values at 1e-6 (NaN too, OSEM.cl:64-65) and passes them
    through where the estimate is below 1e-4."""
    O = oracle_lib
    n = 16
    x = np.zeros((n, n), np.float32)
    ang = np.array([0.0, 45.0], np.float32)
    meas = np.array([[np.nan] * n, [-5.0] * n], np.float32)
    r = O.osem1(x, meas, ang, 1, 0, nrows=2)
    assert np.all(r == np.float32(1e-6))


def test_noncovered_rows_ref_vs_cover(oracle_lib):
    """pa % ss != 0: OSEM2 reads rows OSEM1 never writes (GPU.cpp:169 vs OSEM.cl:93).
    ref mode reads them as 0; cover mode projects them.  Both stay finite."""
    O = oracle_lib
    n, pa, ss = 24, 23, 5
    from xct import phantom as P
    img = P.rasterize_ellipses(P.ellipse_params(n, 3, 2, axes=(2, 6)), n, n)
    ang = np.linspace(0, 180, pa, endpoint=False).astype(np.float32)
    meas = O.projection(img, ang, n)
    x0 = np.ones((n, n), np.float32)
    a = O.osem_run(x0, meas, ang, ss, 2, cover=False)
    b = O.osem_run(x0, meas, ang, ss, 2, cover=True)
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    assert not np.array_equal(a, b)


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_sino_correction_bit_identical_to_reference_kernel(oracle_lib, mode):
    O = oracle_lib
    if not O.ref_available():
        pytest.skip("reference checkout not present")
    pa, px = 36, 56
    ang = np.linspace(-30, 200, pa).astype(np.float32)
    meas = np.random.default_rng(mode).uniform(0, 3, (pa, px)).astype(np.float32)
    ref = O.RefKernels(48, 40, px, pa, 4)
    assert np.array_equal(ref.sino_correction(meas, ang, mode), O.sino_correction(meas, ang, mode))


def test_oracle_adjoint_dot_product_identity_f64(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(12)
    n, px, pa = 40, 52, 33
    ang = np.sort(rng.uniform(0, 180, pa)).astype(np.float32)
    x = rng.uniform(0, 1, (n, n))
    y = rng.uniform(0, 1, (pa, px))
    ax = O.projection(x, ang, px, dtype=np.float64)
    aty = O.adjoint(y, ang, n, n, dtype=np.float64)
    lhs, rhs = float(np.sum(ax * y)), float(np.sum(x * aty))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


# ---------------------------------------------------------------- FBP and the hybrid
@pytest.mark.parametrize("name", ["fbp_64", "fbp_odd"])
def test_fbp_oracle_reproduces_golden(oracle_lib, name):
    """Filter (FBP.cl:34-160), backProjectionFBP (FBP.cl:164-188), base-up
    (reconstShare.cl:87-177) and the hybrid's OS-EM, literal order: bit-exact against the
    fixtures (which the reference kernels reproduced when they were written)."""
    O = oracle_lib
    f = _load(name)
    nx, ny, px, pa, ss, it, zp, order = [int(v) for v in f["shape"]]
    fprj = O.fbp_filter(f["meas"], zp)
    assert np.array_equal(fprj, f["fprj"])
    img = O.bp_fbp(fprj, f["angles"], nx, ny)
    assert np.array_equal(img, f["fbp"])
    based, amin = O.base_up(img, order)
    assert np.array_equal(based, f["base_up"]) and amin == f["minimum"][0]
    hyb = O.osem_run(based, f["meas"], f["angles"], ss, it, sub_order=f["sub"], order=O.ORDER_LITERAL)
    assert np.array_equal(hyb, f["hybrid"])


def test_fbp_filter_float_chain_accuracy(oracle_lib):
    """The reference's float radix-2 chain against the same transform in double with exact
    twiddles: ~2e-6 rel-L2 (the yardstick for the CUDA filter's tolerance)."""
    f = _load("fbp_64")
    e = _rel(f["fprj"], f["fprj_f64"])
    assert 0 < e < 1e-5


def test_fbp_filter_is_a_ramp(oracle_lib):
    """Known answer: a constant row has only a DC component, which the ramp removes, so the
    circularly filtered row of a full-width constant is ~0 where the padded signal is
    periodic; and the filter is linear."""
    O = oracle_lib
    rng = np.random.default_rng(3)
    a = rng.normal(size=(3, 40)).astype(np.float64)
    b = rng.normal(size=(3, 40)).astype(np.float64)
    fa = O.fbp_filter(a, 64, dtype=np.float64)
    fb = O.fbp_filter(b, 64, dtype=np.float64)
    fab = O.fbp_filter(2.0 * a - b, 64, dtype=np.float64)
    assert np.abs(fab - (2.0 * fa - fb)).max() < 1e-12
    const = np.ones((1, 64))
    assert np.abs(O.fbp_filter(const, 64, dtype=np.float64)).max() < 1e-12
    # the ramp's response to a centred delta: h[0] = sum_k |k| pi/zp / zp > 0, h[n] < 0 nearby
    d = np.zeros((1, 64))
    d[0, 32] = 1.0
    r = O.fbp_filter(d, 256, dtype=np.float64)[0]
    assert r[32] > 0 and r[31] < 0 and r[33] < 0 and abs(r[31] - r[33]) < 1e-12


@pytest.mark.parametrize("shape", [(64, 64, 64, 90, 128), (50, 44, 61, 45, 256)])
def test_fbp_oracle_bit_identical_to_reference_kernels(oracle_lib, shape):
    """oracle/_ref's FBP.cl build against the oracle on a fresh shape with irregular angles
    and a non-default zero padding.  Only where the reference checkout exists."""
    O = oracle_lib
    if not O.ref_available():
        pytest.skip("reference checkout not present")
    from xct import phantom as P
    nx, ny, px, pa, zp = shape
    m = max(nx, ny)
    img = P.rasterize_ellipses(P.ellipse_params(m, 5, 9, axes=(2, 12)), nx, ny)
    ang = (np.sort(np.random.default_rng(8).uniform(0, 180, pa))).astype(np.float32)
    meas = P.noisy_log_sinogram(O.projection(img, ang, px), 1e4, 6)
    ref = O.RefKernels(nx, ny, px, pa, 1, zp)
    r_fprj, r_img = ref.fbp(np.stack([meas, meas[::-1].copy()]), ang)
    for z, s in enumerate([meas, meas[::-1].copy()]):
        fprj = O.fbp_filter(s, zp)
        assert np.array_equal(r_fprj[z], fprj)
        assert np.array_equal(r_img[z], O.bp_fbp(fprj, ang, nx, ny))
    for order in (0, 1, 4, 7):
        rb, rm = ref.base_up(r_img, order)
        for z in range(2):
            ob, om = O.base_up(r_img[z], order)
            assert np.array_equal(rb[z], ob) and rm[z] == om


# ------------------------------------------------------------- rotation-centre search
def test_rcs_oracle_reproduces_golden(oracle_lib):
    """rotCenterShift, setMask, imgFocusIndex (literal work-group order and double sums) and
    the one-iteration OS-EM of the search, bit-exact against the pinned fixture."""
    O = oracle_lib
    f = _load("rcs_64")
    n_img, px, pa, ss, n, L = [int(v) for v in f["shape"]]
    start, step, _ = [float(v) for v in f["shift"]]
    shifts = O.shift_values(start, step, n)
    x0 = np.ones((n_img, n_img), np.float32)
    for i, s in enumerate(shifts):
        sh = O.rot_center_shift(f["sino"], s)
        assert np.array_equal(sh, f["shifted"][i])
        img = O.osem_run(x0, sh, f["angles"], ss, 1, sub_order=f["sub"], order=O.ORDER_LITERAL)
        assert np.array_equal(img, f["imgs"][i])
        m = O.set_mask(n_img, n_img, s, float(f["angles"][0]), float(f["angles"][-1]))
        assert np.array_equal(m, f["masks"][i])
        assert np.float32(O.focus_index(img, m, L)) == f["findex"][i]
        assert O.focus_index(img, m, 0) == f["findex_f64"][i]
    # the float work-group order and the double sums agree to ~1e-7
    assert np.abs(f["findex"] / f["findex_f64"] - 1).max() < 1e-5


def test_rcs_mask_known_answers(oracle_lib):
    """setMask with shift 0 over 0..180 deg keeps the disc of radius W/2 (minus the
    half-plane test's boundary); a positive shift shrinks the right edge (rp = W/2) and
    not the left (rm = -W/2 + s)."""
    O = oracle_lib
    W = 64
    m0 = O.set_mask(W, W, 0.0, 0.0, 179.0)
    yy, xx = np.mgrid[0:W, 0:W].astype(np.float64) - W // 2
    disc = (xx * xx + yy * yy) <= (W // 2) ** 2
    assert m0.sum() > 0.9 * disc.sum() and not np.any(m0[~disc])
    m4 = O.set_mask(W, W, 4.0, 0.0, 179.0)
    assert m4.sum() < m0.sum() and not np.any(m4[~disc])


@pytest.mark.parametrize("shape", [(64, 72, 60, 32, 2), (48, 48, 40, 16, 0)])
def test_rcs_oracle_bit_identical_to_reference_kernels(oracle_lib, shape):
    """oracle/_ref's rotCenterSearch.cl build against the oracle: other sizes, work-group
    sizes and a shift offset (offsetN).  Only where the reference checkout exists."""
    O = oracle_lib
    if not (O.ref_available() and O.rcs_available()):
        pytest.skip("reference checkout not present")
    from xct import phantom as P
    n_img, px, pa, L, off = shape
    img = P.rasterize_ellipses(P.ellipse_params(n_img, 5, 4, axes=(2, n_img / 4)), n_img, n_img)
    ang = P.uniform_angles(pa)
    sino = P.noisy_log_sinogram(O.projection(img, ang, px, cx=px / 2 - 1.5), 1e5, 2)
    n, start, step = 5, -1.25, 0.75
    R = O.RefRotCenter(n_img, n_img)
    shifted = R.rot_center_shift(sino, n + off, start, step)
    sv = O.shift_values(start, step, n + off)
    for i in range(n + off):
        assert np.array_equal(shifted[i], O.rot_center_shift(sino, sv[i]))
    x0 = np.ones((n_img, n_img), np.float32)
    imgs = np.stack([O.osem_run(x0, shifted[off + i], ang, 4, 1) for i in range(n)])
    masks, fi = R.focus_index(imgs, L, start, step, float(ang[0]), float(ang[-1]), offsetN=off)
    for i in range(n):
        m = O.set_mask(n_img, n_img, sv[off + i], float(ang[0]), float(ang[-1]))
        assert np.array_equal(masks[i], m)
        assert np.float32(O.focus_index(imgs[i], m, L)) == fi[i]


# ------------------------------------------------------------------------- reslice
def test_reslice_oracle_reproduces_golden(oracle_lib):
    O = oracle_lib
    f = _load("reslice_small")
    baseup, thr = [float(v) for v in f["params"]]
    assert np.array_equal(O.reslice(f["mt"], f["xshift"], f["yshift"], baseup, 0), f["sino"])
    assert np.array_equal(O.reslice(f["mt"], f["xshift"], f["yshift"], baseup, 1), f["sino_corr"])
    assert np.array_equal(O.denoise_sinogram(f["spiky"], thr), f["denoised"])


def test_reslice_known_answers(oracle_lib):
    """Zero shifts and baseup: reslicing is an exact transpose of the angle and row axes;
    an integer shift moves the data by whole pixels with zeros shifted in."""
    O = oracle_lib
    rng = np.random.default_rng(2)
    mt = rng.normal(size=(7, 5, 9)).astype(np.float32)
    assert np.array_equal(O.reslice(mt), mt.transpose(1, 0, 2))
    xs = np.full(7, 2.0, np.float32)
    out = O.reslice(mt, xs)
    assert np.array_equal(out[:, :, :-2], mt.transpose(1, 0, 2)[:, :, 2:])
    assert not np.any(out[:, :, -2:])
    s = np.zeros((1, 6, 3), np.float32)
    s[0, 2, 1] = 5.0  # a one-angle spike
    d = O.denoise_sinogram(s, 1.0)
    assert d[0, 2, 1] == 0.0 and d.sum() == 0.0


@pytest.mark.parametrize("shape", [(64, 48, 30), (37, 21, 11)])
def test_reslice_oracle_bit_identical_to_reference_kernels(oracle_lib, shape):
    O = oracle_lib
    if not O.reslice_available():
        pytest.skip("reference checkout not present")
    W, H, A = shape
    rng = np.random.default_rng(W)
    mt = rng.normal(1, 0.5, (A, H, W)).astype(np.float32)
    xs = rng.uniform(-3, 3, A).astype(np.float32)
    ys = rng.uniform(-2, 2, A).astype(np.float32)
    R = O.RefReslice(W, H, A)
    for x, y, bu, c in [(None, None, 0.0, 0), (xs, ys, 0.25, 0), (xs, ys, -0.1, 1)]:
        assert np.array_equal(R.reslice(mt, x, y, bu, c), O.reslice(mt, x, y, bu, c))
    s = O.reslice(mt)
    s[:, 5, :] += 3.0
    for thr in (0.5, 2.0):
        assert np.array_equal(R.denoise(s, thr), O.denoise_sinogram(s, thr))


# --------------------------------------------------------------- compressed sensing
def test_cs_oracle_reproduces_golden(oracle_lib):
    O = oracle_lib
    f = _load("cs_64")
    n, px, pa, ss, it, dN = [int(v) for v in f["shape"]]
    lam = float(f["cs_lambda"][0])
    out = O.cs_osem_run(f["x0"], f["meas"], f["angles"], ss, it, lam, f["sub"], order=O.ORDER_LITERAL)
    assert np.array_equal(out, f["cs"])


def test_cs_proximal_known_answers(oracle_lib):
    """Interior voxels of a constant volume are fixed points of ISTA3D/FISTA3D's selection;
    a lone bright voxel moves toward its neighbours by 6 lambda (the l1 pull of six
    neighbours); lambda follows the reference's six-digit text of CSlambda."""
    O = oracle_lib
    lam = O.cs_lambda(1e-4)
    assert lam == np.float32(1e-4)
    assert O.cs_lambda(np.float32(1.2345678e-3)) == np.float32(1.23457e-3)
    v = np.full((3, 8, 8), 0.5, np.float32)
    x = O.ista3d(v, lam)
    assert np.all(x[1:, 1:-1, 1:-1] == np.float32(0.5))
    v2 = v.copy()
    v2[1, 4, 4] = 0.9
    x2 = O.ista3d(v2, lam)
    assert x2[1, 4, 4] == np.float32(np.float32(0.9) - np.float32(6.0) * np.float32(lam))
    w, xf, b = O.fista3d(v, v, np.zeros_like(v), lam)
    assert np.all(b == 1.0) and np.all(xf[1:, 1:-1, 1:-1] == np.float32(0.5))


@pytest.mark.parametrize("shape", [(48, 56, 36, 4, 4, 2), (40, 40, 30, 3, 2, 3)])
def test_cs_oracle_bit_identical_to_reference_kernels(oracle_lib, shape):
    O = oracle_lib
    if not O.ref_available():
        pytest.skip("reference checkout not present")
    from xct import phantom as P
    n, px, pa, ss, dN, it = shape
    ang = (np.sort(np.random.default_rng(n).uniform(0, 180, pa))).astype(np.float32)
    prm = P.ellipsoid_params(n, dN, count=5, seed=7)
    meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, px), 1e4, z)
                     for z in range(dN)])
    x0 = np.full((dN, n, n), 0.7, np.float32)
    so = O.subset_order(ss)
    ref = O.RefKernels(n, n, px, pa, ss)
    assert np.array_equal(ref.fista_osem_execution(x0, meas, ang, so, it),
                          O.cs_osem_run(x0, meas, ang, ss, it, 1e-4, so, order=O.ORDER_LITERAL))
