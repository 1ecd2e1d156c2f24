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
  fbp_64.npz     FBP (FBP.cl) of a 64x64 slice, 90 angles, 64 bins, zero padding 128: the
                 filtered sinogram, the image, the base-up image (order 4) and the hybrid
                 (FBP + base-up + 10 subsets x 2 iterations of OS-EM).
  fbp_odd.npz    the same for a 48x40 image, 57 bins, 37 angles (odd: the GPU filter pairs
                 rows across the end of a slice), zero padding 256, 1 subset x 2 iterations.
  rcs_64.npz     rotation-centre search (RotationCenterSearch/) on a 64x64 slice whose
                 sinogram (64 bins, 90 angles) is centred 1.0 bin right of px/2: 9 shifts
                 from -2.0 in steps of 0.5, one OS-EM iteration of 10 subsets from 1.0 each,
                 masks and focus indices (work-group of 64 items, and in double).
  reslice_small.npz  reslice (Reslice/reslice.cl) of 16 projections of 12 x 24 pixels
                 (uniform 0.5..1.5, seed 16) with per-angle shifts U[-2.5, 2.5] (x) and
                 U[-1.5, 1.5] (y), baseup 0.125, without and with the cosine correction,
                 and denoiseSinogram (threshold 0.3) of the first result with planted spikes.
  cs_64.npz      compressed-sensing OS-EM (FISTA_OSEM_execution with ISTA3D/FISTA3D) of a
                 batch of 3 slices of a 64x64x3 ellipsoid phantom (seed 4), 90 angles, 64 bins,
                 I0 = 1e4 (seeds 0..2), 10 subsets x 2 iterations, CSlambda 1e-4, from 1.0.
  fista_64.npz   FISTA with compressed sensing (powerIteration, 30 trials; FISTA_execution
                 with AART1, FISTAbackProjection, ISTA3D/FISTA3D) of 3 slices of a 64x64x3
                 ellipsoid phantom (seed 6), 90 angles, 64 bins, I0 = 1e4, 10 subsets x 2
                 iterations, CSlambda 1e-4, AART factor 1.0; also the run that stores
                 FISTA3D's x_{t+1}.
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


def fbp_case(name, nx, ny, px, pa, zp, ss, it, order, n_ell, seed, i0, noise_seed):
    m = max(nx, ny)
    img = P.rasterize_ellipses(P.ellipse_params(m, n_ell, seed, axes=(3, m / 4)), m, m)
    img = np.ascontiguousarray(img[(m - ny) // 2:(m - ny) // 2 + ny, (m - nx) // 2:(m - nx) // 2 + nx])
    ang = P.uniform_angles(pa)
    meas = P.noisy_log_sinogram(O.projection(img, ang, px, order=LIT), i0, noise_seed)
    fprj = O.fbp_filter(meas, zp)
    fbp = O.bp_fbp(fprj, ang, nx, ny)
    based, amin = O.base_up(fbp, order)
    sub = O.subset_order(ss)
    hybrid = O.osem_run(based, meas, ang, ss, it, sub_order=sub, order=LIT)
    arrays = dict(phantom=img, angles=ang, meas=meas, fprj=fprj, fbp=fbp, base_up=based,
                  minimum=np.array([amin], np.float32), sub=sub, hybrid=hybrid,
                  fprj_f64=O.fbp_filter(meas.astype(np.float64), zp, dtype=np.float64),
                  shape=np.array([nx, ny, px, pa, ss, it, zp, order], np.int32))
    if O.ref_available():
        ref = O.RefKernels(nx, ny, px, pa, ss, zp)
        r_fprj, r_img = ref.fbp(meas, ang)
        assert np.array_equal(r_fprj, fprj), name + ": filtered sinogram differs from FBP.cl"
        assert np.array_equal(r_img, fbp), name + ": FBP image differs from FBP.cl"
        r_based, r_min = ref.base_up(r_img, order)
        assert np.array_equal(r_based, based) and r_min[0] == amin, name + ": base-up differs"
        r_hyb = ref.osem_execution(r_based[None], meas[None], ang, sub, it)[0]
        assert np.array_equal(r_hyb, hybrid), name + ": hybrid OS-EM differs"
        arrays["pinned_by_reference_kernels"] = np.array([1], np.int32)
        print(name, "pinned: bit-identical to the reference kernels")
    else:
        arrays["pinned_by_reference_kernels"] = np.array([0], np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


def rcs_case(name, n_img, px, pa, ss, n, start, step, offset, seed, i0, noise_seed, L):
    img = P.rasterize_ellipses(P.ellipse_params(n_img, 6, seed, axes=(3, n_img / 4)), n_img, n_img)
    ang = P.uniform_angles(pa)
    sino = P.noisy_log_sinogram(O.projection(img, ang, px, cx=px / 2 + offset, order=LIT), i0, noise_seed)
    shifts = O.shift_values(start, step, n)
    shifted = np.stack([O.rot_center_shift(sino, s) for s in shifts])
    sub = O.subset_order(ss)
    x0 = np.ones((n_img, n_img), np.float32)
    imgs = np.stack([O.osem_run(x0, shifted[i], ang, ss, 1, sub_order=sub, order=LIT) for i in range(n)])
    masks = np.stack([O.set_mask(n_img, n_img, s, float(ang[0]), float(ang[-1])) for s in shifts])
    f_lit = np.array([O.focus_index(imgs[i], masks[i], L) for i in range(n)], np.float32)
    f_dbl = np.array([O.focus_index(imgs[i], masks[i], 0) for i in range(n)], np.float64)
    arrays = dict(phantom=img, angles=ang, sino=sino, shifted=shifted, sub=sub, imgs=imgs, masks=masks,
                  findex=f_lit, findex_f64=f_dbl,
                  shape=np.array([n_img, px, pa, ss, n, L], np.int32),
                  shift=np.array([start, step, offset], np.float32))
    if O.ref_available() and O.rcs_available():
        R = O.RefRotCenter(n_img, n_img)
        assert np.array_equal(R.rot_center_shift(sino, n, start, step), shifted), name + ": rotCenterShift differs"
        r_masks, r_fi = R.focus_index(imgs, L, start, step, float(ang[0]), float(ang[-1]))
        assert np.array_equal(r_masks, masks), name + ": setMask differs"
        assert np.array_equal(r_fi, f_lit), name + ": imgFocusIndex differs"
        ref = O.RefKernels(n_img, n_img, px, pa, ss)
        r_imgs = ref.osem_execution(np.repeat(x0[None], n, 0), shifted, ang, sub, 1)
        assert np.array_equal(r_imgs, imgs), name + ": OS-EM differs"
        arrays["pinned_by_reference_kernels"] = np.array([1], np.int32)
        print(name, "pinned: bit-identical to the reference kernels")
    else:
        arrays["pinned_by_reference_kernels"] = np.array([0], np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


def reslice_case(name, A, H, W, seed, baseup, threshold):
    rng = np.random.default_rng(seed)
    mt = rng.uniform(0.5, 1.5, (A, H, W)).astype(np.float32)
    xs = rng.uniform(-2.5, 2.5, A).astype(np.float32)
    ys = rng.uniform(-1.5, 1.5, A).astype(np.float32)
    out0 = O.reslice(mt, xs, ys, baseup, 0)
    out1 = O.reslice(mt, xs, ys, baseup, 1)
    spiky = out0.copy()
    spiky[:, 5, ::3] += 1.0
    spiky[:, 9, 1::4] -= 1.0
    den = O.denoise_sinogram(spiky, threshold)
    arrays = dict(mt=mt, xshift=xs, yshift=ys, sino=out0, sino_corr=out1, spiky=spiky, denoised=den,
                  params=np.array([baseup, threshold], np.float32))
    if O.reslice_available():
        R = O.RefReslice(W, H, A)
        assert np.array_equal(R.reslice(mt, xs, ys, baseup, 0), out0), name + ": reslice differs"
        assert np.array_equal(R.reslice(mt, xs, ys, baseup, 1), out1), name + ": corrected reslice differs"
        assert np.array_equal(R.denoise(spiky, threshold), den), name + ": denoiseSinogram differs"
        arrays["pinned_by_reference_kernels"] = np.array([1], np.int32)
        print(name, "pinned: bit-identical to the reference kernels")
    else:
        arrays["pinned_by_reference_kernels"] = np.array([0], np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


def cs_case(name, n, px, pa, ss, it, dN, lam, seed, i0):
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, dN, count=6, seed=seed)
    meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, px, order=LIT), i0, z)
                     for z in range(dN)])
    x0 = np.ones((dN, n, n), np.float32)
    sub = O.subset_order(ss)
    out = O.cs_osem_run(x0, meas, ang, ss, it, lam, sub, order=LIT)
    out_gpu_order = O.cs_osem_run(x0, meas, ang, ss, it, lam, sub, order=O.ORDER_GPU)
    arrays = dict(angles=ang, meas=meas, x0=x0, sub=sub, cs=out, cs_gpu_order=out_gpu_order,
                  shape=np.array([n, px, pa, ss, it, dN], np.int32), cs_lambda=np.array([lam], np.float32))
    if O.ref_available():
        ref = O.RefKernels(n, n, px, pa, ss)
        assert np.array_equal(ref.fista_osem_execution(x0, meas, ang, sub, it), out), name + ": CS OS-EM differs"
        arrays["pinned_by_reference_kernels"] = np.array([1], np.int32)
        print(name, "pinned: bit-identical to the reference kernels")
    else:
        arrays["pinned_by_reference_kernels"] = np.array([0], np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


def fista_case(name, n, px, pa, ss, it, dN, lam, alpha, trials, seed, i0):
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, dN, count=6, seed=seed)
    meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, px, order=LIT), i0, z)
                     for z in range(dN)])
    sub = O.subset_order(ss)
    L = O.power_iteration(ang, n, n, px, ss, trials=trials)
    out = O.fista_run(np.zeros((dN, n, n)), meas, ang, ss, it, L, alpha, lam, sub_order=sub)
    upd = O.fista_run(np.zeros((dN, n, n)), meas, ang, ss, it, L, alpha, lam, sub_order=sub, flags=1)
    arrays = dict(angles=ang, meas=meas, sub=sub, L=L, fista=out, fista_update_x=upd,
                  shape=np.array([n, n, px, pa, ss, it, trials], np.int32), cs_lambda=np.array([lam], np.float32),
                  alpha=np.array([alpha], np.float32))
    if O.ref_available():
        ref = O.RefKernels(n, n, px, pa, ss, cs_lambda="%g" % np.float32(lam))
        assert np.array_equal(ref.power_iteration(ang, trials=trials), L), name + ": power iteration differs"
        assert np.array_equal(ref.fista_execution(meas, ang, sub, it, L, alpha), out), name + ": FISTA differs"
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
    fbp_case("fbp_64", 64, 64, 64, 90, 128, 10, 2, 4, 8, 3, 1e5, 13)
    fbp_case("fbp_odd", 48, 40, 57, 37, 256, 1, 2, 4, 6, 7, 1e5, 14)
    rcs_case("rcs_64", 64, 64, 90, 10, 9, -2.0, 0.5, 1.0, 5, 1e5, 15, 64)
    reslice_case("reslice_small", 16, 12, 24, 16, 0.125, 0.3)
    cs_case("cs_64", 64, 64, 90, 10, 2, 3, 1.0e-4, 4, 1e4)
    fista_case("fista_64", 64, 64, 90, 10, 2, 3, 1.0e-4, 1.0, 30, 6, 1e4)
