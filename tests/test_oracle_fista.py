"""CPU tests of the FISTA oracle (power iteration for the Lipschitz estimates and
FISTA_execution) pinned bit for bit against the reference's own kernels -- powerIter1/2/3,
AART1, FISTAbackProjection, ISTA3D/FISTA3D, backProjection and sinogramCorrection of
CT_reconstruction/FISTA.cl, AART.cl and reconstShare.cl -- compiled through the OpenCL-C shim
(oracle/build_ref.py) and driven as GPU.cpp:1755-1924 and 2079-2188 drive them, and against
the committed golden fixture where that build is absent."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _ref(oracle_lib, *shape, cs_lambda="0.0001"):
    if not oracle_lib.ref_available():
        pytest.skip("reference checkout not present (the golden fixture test covers this machine)")
    return oracle_lib.RefKernels(*shape, cs_lambda=cs_lambda)


def _problem(O, n, px, pa, seed):
    from xct import phantom as P
    ang = P.uniform_angles(pa)
    imgs = [P.rasterize_ellipses(P.ellipse_params(n, 5, seed + z, axes=(3, n / 4)), n, n) for z in range(3)]
    meas = np.stack([P.noisy_log_sinogram(O.projection(im, ang, px), 1e5, seed + z) for z, im in enumerate(imgs)])
    return ang, meas


@pytest.mark.parametrize("fetch", [0, 1])
def test_power_iteration_matches_reference_kernels(oracle_lib, fetch):
    O = oracle_lib
    n, px, pa, ss = 64, 64, 90, 10
    ref = _ref(O, n, n, px, pa, ss)
    ang = np.arange(pa, dtype=np.float32) * np.float32(180.0 / pa)
    want = ref.power_iteration(ang, trials=4, work_group=1024, fetch_mode=fetch)
    got = O.power_iteration(ang, n, n, px, ss, trials=4, work_group=1024, fetch_mode=fetch)
    assert np.array_equal(got, want)
    assert np.all(got > 0)


def test_power_iteration_partial_work_groups(oracle_lib):
    """A work-group size that does not divide the image width: the reference's reductions
    visit only the first (nx / wg) * wg columns and rows, and its tree drops odd tails."""
    O = oracle_lib
    n, px, pa, ss = 64, 64, 90, 10
    ref = _ref(O, n, n, px, pa, ss)
    ang = np.arange(pa, dtype=np.float32) * np.float32(180.0 / pa)
    for wg in (48, 20):
        assert np.array_equal(O.power_iteration(ang, n, n, px, ss, trials=2, work_group=wg),
                              ref.power_iteration(ang, trials=2, work_group=wg))


@pytest.mark.parametrize("corr,it", [(0, 2), (2, 1)])
def test_fista_execution_matches_reference_kernels(oracle_lib, corr, it):
    O = oracle_lib
    n, px, pa, ss = 64, 64, 90, 10
    ref = _ref(O, n, n, px, pa, ss)
    ang, meas = _problem(O, n, px, pa, 70)
    L = O.power_iteration(ang, n, n, px, ss, trials=5)
    sub = O.subset_order(ss)
    want = ref.fista_execution(meas, ang, sub, it, L, alpha=1.0, correction_mode=corr)
    got = O.fista_run(np.zeros((3, n, n)), meas, ang, ss, it, L, alpha=1.0, cs_lambda_f32=1e-4,
                      correction_mode=corr, sub_order=sub)
    assert np.array_equal(got, want)
    assert np.all(np.isfinite(got)) and got.max() > 0


def test_fista_reference_image_is_the_first_cycle(oracle_lib):
    """The reference binds FISTA3D's x_{t+1} to the beta image (GPU.cpp:1867-1868), so its
    image after any number of cycles is the first cycle's ISTA3D step; with the output stored
    (flag 1) later cycles change it."""
    O = oracle_lib
    n, px, pa, ss = 48, 48, 60, 6
    ang, meas = _problem(O, n, px, pa, 80)
    L = O.power_iteration(ang, n, n, px, ss, trials=5)
    one = O.fista_run(np.zeros((3, n, n)), meas, ang, ss, 1, L)
    three = O.fista_run(np.zeros((3, n, n)), meas, ang, ss, 3, L)
    assert np.array_equal(one, three)
    upd = O.fista_run(np.zeros((3, n, n)), meas, ang, ss, 3, L, flags=1)
    assert not np.array_equal(upd, three)


def test_fista_golden_fixture(oracle_lib):
    """The committed fixture (written by tests/golden/make_golden.py only after the reference
    build reproduced it) pins the oracle where the reference checkout is absent."""
    O = oracle_lib
    f = dict(np.load(os.path.join(GOLDEN, "fista_64.npz")))
    nx, ny, px, pa, ss, it, trials = [int(v) for v in f["shape"]]
    L = O.power_iteration(f["angles"], nx, ny, px, ss, trials=trials)
    assert np.array_equal(L, f["L"])
    kw = dict(alpha=float(f["alpha"][0]), cs_lambda_f32=float(f["cs_lambda"][0]), sub_order=f["sub"])
    got = O.fista_run(np.zeros((f["meas"].shape[0], ny, nx)), f["meas"], f["angles"], ss, it, L, **kw)
    assert np.array_equal(got, f["fista"])
    upd = O.fista_run(np.zeros((f["meas"].shape[0], ny, nx)), f["meas"], f["angles"], ss, it, L, flags=1, **kw)
    assert np.array_equal(upd, f["fista_update_x"])
