"""The algorithmic work behind the benchmark's roofline: bench.algorithmic_counts gives, per
angle, T_fwd (bilinear samples whose 2x2 footprint meets the image: base texel in
[-1, nx-1] x [-1, ny-1], from each ray's exact chord) and T_bp ((pixel, angle) pairs whose
nearest bin lands on the detector).  Both are checked here against brute-force enumeration of
every sample and every pixel, in float64, on small odd geometries -- with 0, 45, 90, 135 and
180 degree angles, where sample coordinates fall exactly on texel boundaries (a direction
cosine below 1e-12 counts as 0, as in the helper), and an off-centre axis."""
import numpy as np
import pytest


def _brute(angles, nx, ny, px, cx):
    D = max(nx, ny)
    t_fwd, t_bp = [], []
    X = np.arange(px, dtype=np.float64)[:, None]
    Y = np.arange(D, dtype=np.float64)[None, :]
    xp = np.arange(nx, dtype=np.float64)[None, :] - nx * 0.5
    yp = np.arange(ny, dtype=np.float64)[:, None] - ny * 0.5
    for th in np.deg2rad(np.asarray(angles, np.float64)):
        c, s = np.cos(th), np.sin(th)
        # the counts' convention: a direction cosine below 1e-12 (cos 90, sin 180 in float64)
        # is exactly 0, so rays lying on a texel boundary count whole, as at 0 degrees
        c = 0.0 if abs(c) < 1e-12 else c
        s = 0.0 if abs(s) < 1e-12 else s
        x = (Y - D * 0.5) * s + (X - cx) * c + nx * 0.5
        y = (Y - D * 0.5) * c - (X - cx) * s + ny * 0.5
        t_fwd.append(int(np.count_nonzero((x >= -1) & (x < nx) & (y >= -1) & (y < ny))))
        b = np.floor(xp * c - yp * s + cx + 0.5)
        t_bp.append(int(np.count_nonzero((b >= 0) & (b < px))))
    return np.array(t_fwd), np.array(t_bp)


@pytest.mark.parametrize("nx,ny,px,cx_off", [(37, 37, 41, 0.0), (40, 27, 33, 2.75), (23, 45, 60, -3.5)])
def test_counts_match_brute_force(nx, ny, px, cx_off):
    from bench import algorithmic_counts
    rng = np.random.default_rng(nx * ny)
    angles = np.concatenate([[0.0, 45.0, 90.0, 135.0, 180.0], rng.uniform(0.0, 360.0, 12)])
    cx = px * 0.5 + cx_off
    t_fwd, t_bp = algorithmic_counts(angles, nx, ny, px, cx=cx)
    want_fwd, want_bp = _brute(angles, nx, ny, px, cx)
    assert np.array_equal(t_fwd.astype(np.int64), want_fwd), (t_fwd, want_fwd)
    assert np.array_equal(t_bp.astype(np.int64), want_bp), (t_bp, want_bp)


def _geometry_groups(n_energy, n_slices):
    """Sizes of the sets of items that share one geometry (width = bins, angle list) in the
    benchmark's CT-XAFS stack, items taken energy by energy."""
    from bench import ctxafs_stack_specs
    widths, angs, _ = ctxafs_stack_specs(n_energy, n_slices)
    groups = {}
    for e in range(n_energy):
        for w in widths:
            key = (w, angs[e].tobytes())
            groups[key] = groups.get(key, 0) + 1
    return sorted(groups.values())


def test_ctxafs_stacks_geometry_groups():
    """The 512-item stack (64 energies x 8 slices) has two slices per width and energy, below
    the batch plan's group size of eight, so its graph serves every item; the stack with whole
    energies (4 x 64) has 16 groups of 16, so every item is in a geometry group.  Widths
    512-2048 each appear equally often; angle counts stay within 360-1200 minus 10 %."""
    from bench import ctxafs_stack_specs
    assert _geometry_groups(64, 8) == [2] * 256
    assert _geometry_groups(4, 64) == [16] * 16
    widths, angs, grids = ctxafs_stack_specs(4, 64)
    assert sorted(set(widths)) == [512, 1024, 1536, 2048]
    assert all(widths.count(w) == 16 for w in (512, 1024, 1536, 2048))
    for a, (pa, keep) in zip(angs, grids):
        assert pa in (360, 720, 900, 1200) and 0.9 * pa <= len(a) <= pa
        assert np.array_equal(a, (keep * (180.0 / pa)).astype(np.float32))
