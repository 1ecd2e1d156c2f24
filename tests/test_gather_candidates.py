"""The gather form of the exact adjoint (adj_gather_kernel in csrc/xct_tiled.cu) finds the
forward projector's samples per base texel instead of scattering them: for texel (i, j) and
one angle it tests only four candidates -- rays Xa, Xa + 1 with Xa = floor(u0 - 0.717) + 1,
indices Ya, Ya + 1 with Ya = floor(w0 - 0.717) + 1, where u0 and w0 are the lattice
coordinates of the texel's centre.  That is complete only if every sample whose base texel is
(i, j) is among them.  Checked here on the CPU with the kernels' float32 arithmetic (fused
multiply-adds emulated exactly: float32 products are exact in float64) over every sample of
a 256^2 geometry at 0, 45, 90, 135 degrees, random angles and an off-centre axis; also that
no texel holds more than two samples of one angle."""
import numpy as np
import pytest

f32 = np.float32


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


@pytest.mark.parametrize("cx_off", [0.0, 3.5])
def test_every_sample_is_a_candidate_of_its_base_texel(cx_off):
    n = px = D = 256
    hx = hy = f32(n * 0.5)
    hd = f32(D * 0.5)
    cx = f32(px * 0.5 + cx_off)
    rng = np.random.default_rng(11)
    deg = np.concatenate([[0.0, 45.0, 90.0, 135.0], rng.uniform(0.0, 180.0, 60)])
    X = np.arange(px)
    Y = np.arange(D)
    XX, YY = np.meshgrid(X, Y, indexing="ij")
    Xc = (XX.astype(f32) - cx).astype(f32)
    Yc = (YY.astype(f32) - hd).astype(f32)
    for t in deg:
        th = np.float64(t) * np.pi / 180.0
        c, s = f32(np.cos(th)), f32(np.sin(th))
        c_arr, s_arr = np.full_like(Xc, c), np.full_like(Xc, s)
        # the forward's sample coordinates: (ax, ay) = Xc (c, -s) + (hx, hy), then + Yc (s, c)
        ax = _fma(Xc, c_arr, np.full_like(Xc, hx))
        ay = _fma(Xc, -s_arr, np.full_like(Xc, hy))
        x = _fma(Yc, s_arr, ax)
        y = _fma(Yc, c_arr, ay)
        bi = np.floor(x).astype(np.int64)
        bj = np.floor(y).astype(np.int64)
        inside = (bi >= -1) & (bi < n) & (bj >= -1) & (bj < n)
        bi, bj, sx, sy = bi[inside], bj[inside], XX[inside], YY[inside]
        # the kernel's candidates of each sample's base texel
        di = ((bi.astype(f32) + f32(0.5)) - hx).astype(f32)
        dj = ((bj.astype(f32) + f32(0.5)) - hy).astype(f32)
        u0 = _fma(di, np.full_like(di, c), _fma(-dj, np.full_like(dj, s), np.full_like(di, cx)))
        w0 = (_fma(di, np.full_like(di, s), (dj * c).astype(f32)) + hd).astype(f32)
        Xa = np.floor((u0 - f32(0.717)).astype(f32)).astype(np.int64) + 1
        Ya = np.floor((w0 - f32(0.717)).astype(f32)).astype(np.int64) + 1
        ok = ((sx == Xa) | (sx == Xa + 1)) & ((sy == Ya) | (sy == Ya + 1))
        assert ok.all(), (t, int((~ok).sum()))
        key = (bj + 1) * (n + 2) + (bi + 1)
        assert np.bincount(key).max() <= 2, t
