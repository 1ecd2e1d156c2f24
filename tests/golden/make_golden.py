"""Generate the golden fixtures of tests/golden/ (run from the repository root).

The reference (NozomuIshiguro/CT-XAFS_analysis) ships no tests, fixtures or golden
vectors.  These fixtures are produced by the oracle's LITERAL evaluation order
(oracle/xct_oracle.c), and, when the reference checkout is present, every array is first
checked to be bit-identical to the reference's own OSEM.cl/reconstShare.cl kernels
compiled through oracle/ref_shim (oracle/build_ref.py) -- the script refuses to write a
fixture that the reference build does not reproduce.

Fixtures (np.savez_compressed):
  cfg1_256.npz   256x256 image, 180 angles over 180 deg, 256 bins, centre bin 128;
                 10 seeded ellipses (seed 1), I0 = 1e5 Poisson noise (seed 11),
                 10 subsets x 5 iterations from a uniform 1.0 image.
  small_64.npz   64x64, 90 angles, 64 bins, 10 subsets x 2 iterations; also the OSEM1
                 ratio and OSEM2 image of the first subset, and the projection/
                 backProjection kernels on their own.
  odd_48x40.npz  48x40 image, 56 bins, 36 angles, 4 subsets (power of two: bit-reversed
                 order) x 3 iterations: non-square image, px != nx.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "ct-xafs_analysis_gb300"))

import oracle as O  # noqa: E402
from xct import phantom as P  # noqa: E402

LIT = O.ORDER_LITERAL


def case(name, nx, ny, px, pa, ss, it, n_ell, seed, i0, noise_seed):
    m = max(nx, ny)
    img = P.rasterize_ellipses(P.ellipse_params(m, n_ell, seed, axes=(5 * m / 256, 60 * m / 256)), m, m)
    img = np.ascontiguousarray(img[(m - ny) // 2:(m - ny) // 2 + ny, (m - nx) // 2:(m - nx) // 2 + nx])
    ang = P.uniform_angles(pa)
    clean = O.projection(img, ang, px, order=LIT)
    meas = P.noisy_log_sinogram(clean, i0, noise_seed)
    x0 = np.ones((ny, nx), np.float32)
    sub = O.subset_order(ss)
    out = O.osem_run(x0, meas, ang, ss, it, sub_order=sub, order=LIT)
    out64 = O.osem_run(x0, meas, ang, ss, it, sub_order=sub, order=LIT, dtype=np.float64)
    ratio0 = O.osem1(x0, meas, ang, ss, int(sub[0]), order=LIT)
    upd0 = O.osem2(x0, ratio0, ang, ss, int(sub[0]), order=LIT)
    bp_all = O.backprojection(clean, ang, nx, ny, 1, 0, order=LIT)
    arrays = dict(phantom=img, angles=ang, clean=clean, meas=meas, x0=x0, sub=sub, osem=out, osem_f64=out64,
                  ratio0=ratio0, upd0=upd0, bp_all=bp_all,
                  shape=np.array([nx, ny, px, pa, ss, it], np.int32))
    if O.ref_available():
        ref = O.RefKernels(nx, ny, px, pa, ss)
        r_out = ref.osem_execution(x0[None], meas[None], ang, sub, it)[0]
        assert np.array_equal(r_out, out), name + ": oracle OS-EM differs from the reference kernels"
        rows = np.arange(0, (pa // ss) * ss, ss)
        r_prj = ref.projection(img, ang, 0)
        clean_s = O.projection(img, ang, px, ss=ss, sub=0, order=LIT)
        assert np.array_equal(r_prj[rows], clean_s[rows]), name + ": projection differs"
        arrays["pinned_by_reference_kernels"] = np.array([1], np.int32)
        print(name, "pinned: bit-identical to the reference kernels")
    else:
        arrays["pinned_by_reference_kernels"] = np.array([0], np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


if __name__ == "__main__":
    O.build()
    case("small_64", 64, 64, 64, 90, 10, 2, 10, 1, 1e5, 11)
    case("odd_48x40", 48, 40, 56, 36, 4, 3, 6, 5, 1e5, 12)
    case("cfg1_256", 256, 256, 256, 180, 10, 5, 10, 1, 1e5, 11)
