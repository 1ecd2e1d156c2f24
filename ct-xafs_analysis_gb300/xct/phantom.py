"""Seeded synthetic inputs for the OS-EM workloads.

No public dataset is involved; these generators produce inputs with the shapes, sizes and
value distributions of the workloads the library is measured on:

* ``ellipse_phantom``   -- additive 2-D ellipses (single-slice workload: 10 ellipses, centres
  in the inner 80% of the field of view, semi-axes 5-60 px, attenuation 0.01-0.2 /px);
* ``ellipsoid_volume``  -- a 3-D ellipsoid phantom sectioned into slices (per-slice workload at
  scale: 30 ellipsoids, attenuation 0.005-0.1 /px);
* ``xanes_mixture``     -- per-voxel mixtures of two synthetic XANES spectra (CT-XAFS stack);
* ``noisy_log_sinogram``-- transmission counts I = Poisson(I0 exp(-p)), then -ln(max(I,1)/I0).

Everything works on numpy arrays; the ``torch`` variants run the same formulas on a device
tensor for the large workloads (torch is used as an array library only).
"""
import math

import numpy as np


def uniform_angles(pa, span_deg=180.0):
    """pa angles k * span / pa, k = 0..pa-1, in degrees (float32), as in the log files the
    reference reads (one angle per line, CT_reconstruction/fileIO.cpp:11-23)."""
    return (np.arange(pa, dtype=np.float64) * (span_deg / pa)).astype(np.float32)


def ellipse_params(n, count=10, seed=1, axes=(5.0, 60.0), mu=(0.01, 0.2), inner=0.8):
    """Random ellipses for an n x n field of view: rows (cx, cy, a, b, angle, mu)."""
    rng = np.random.default_rng(seed)
    lo, hi = 0.5 * (1.0 - inner) * n, 0.5 * (1.0 + inner) * n
    cx = rng.uniform(lo, hi, count)
    cy = rng.uniform(lo, hi, count)
    a = rng.uniform(axes[0], axes[1], count)
    b = rng.uniform(axes[0], axes[1], count)
    ang = rng.uniform(0.0, math.pi, count)
    m = rng.uniform(mu[0], mu[1], count)
    return np.stack([cx, cy, a, b, ang, m], axis=1)


def rasterize_ellipses(params, nx, ny):
    """Sum of ellipse indicator functions sampled at pixel centres (x = i, y = j)."""
    img = np.zeros((ny, nx), dtype=np.float64)
    y, x = np.mgrid[0:ny, 0:nx].astype(np.float64)
    for cx, cy, a, b, ang, m in params:
        c, s = math.cos(ang), math.sin(ang)
        dx, dy = x - cx, y - cy
        u = (dx * c + dy * s) / a
        v = (-dx * s + dy * c) / b
        img += m * ((u * u + v * v) <= 1.0)
    return img.astype(np.float32)


def ellipse_phantom(n=256, count=10, seed=1, axes=(5.0, 60.0), mu=(0.01, 0.2)):
    return rasterize_ellipses(ellipse_params(n, count, seed, axes, mu), n, n)


def ellipsoid_params(n, nz, count=30, seed=2, mu=(0.005, 0.1), inner=0.8):
    """Random ellipsoids in an n x n x nz volume: rows (cx, cy, cz, a, b, c, angle, mu)."""
    rng = np.random.default_rng(seed)
    lo, hi = 0.5 * (1.0 - inner) * n, 0.5 * (1.0 + inner) * n
    cx = rng.uniform(lo, hi, count)
    cy = rng.uniform(lo, hi, count)
    cz = rng.uniform(0.0, nz, count)
    a = rng.uniform(0.04 * n, 0.3 * n, count)
    b = rng.uniform(0.04 * n, 0.3 * n, count)
    c = rng.uniform(0.2 * nz, 0.8 * nz, count)
    ang = rng.uniform(0.0, math.pi, count)
    m = rng.uniform(mu[0], mu[1], count)
    return np.stack([cx, cy, cz, a, b, c, ang, m], axis=1)


def ellipsoid_slice(params, z, nx, ny, torch_device=None):
    """Section z of an ellipsoid phantom, sampled at pixel centres."""
    if torch_device is not None:
        import torch
        y, x = torch.meshgrid(torch.arange(ny, device=torch_device, dtype=torch.float32),
                              torch.arange(nx, device=torch_device, dtype=torch.float32), indexing="ij")
        img = torch.zeros((ny, nx), device=torch_device, dtype=torch.float32)
    else:
        y, x = np.mgrid[0:ny, 0:nx].astype(np.float32)
        img = np.zeros((ny, nx), dtype=np.float32)
    for cx, cy, cz, a, b, c, ang, m in params:
        w = 1.0 - ((z + 0.5 - cz) / c) ** 2
        if w <= 0.0:
            continue
        r = math.sqrt(w)
        co, si = math.cos(ang), math.sin(ang)
        dx, dy = x - cx, y - cy
        u = (dx * co + dy * si) / (a * r)
        v = (-dx * si + dy * co) / (b * r)
        img += float(m) * ((u * u + v * v) <= 1.0)
    return img


def noisy_log_sinogram(p, i0, seed):
    """Poisson transmission noise on a line-integral sinogram p, then log conversion:
    y = -ln(max(I, 1) / I0) with I ~ Poisson(I0 exp(-p))."""
    rng = np.random.default_rng(seed)
    lam = i0 * np.exp(-np.asarray(p, dtype=np.float64))
    counts = rng.poisson(lam)
    return (-np.log(np.maximum(counts, 1) / i0)).astype(np.float32)


def noisy_log_sinogram_torch(p, i0, generator=None):
    import torch
    lam = i0 * torch.exp(-p.double())
    counts = torch.poisson(lam, generator=generator)
    return (-torch.log(torch.clamp(counts, min=1.0) / i0)).float()


# ------------------------------------------------------------------ CT-XAFS (XANES) stack
def xanes_spectrum(energies, e0=7112.0, wl_amp=1.0, wl_sigma=3.0, edge_width=1.5):
    """Arctan edge step at e0 plus a Gaussian white line just above the edge."""
    e = np.asarray(energies, dtype=np.float64)
    step = 0.5 + np.arctan((e - e0) / edge_width) / math.pi
    wl = wl_amp * np.exp(-0.5 * ((e - (e0 + 2.0 * wl_sigma)) / wl_sigma) ** 2)
    return step + wl


def xanes_mixture(n_energy=64, seed=3, e_range=(7080.0, 7180.0)):
    """Two random XANES spectra S1(E), S2(E) (white-line amplitude 0.2-1.5, sigma 2-5 eV)."""
    rng = np.random.default_rng(seed)
    e = np.linspace(e_range[0], e_range[1], n_energy)
    s = [xanes_spectrum(e, wl_amp=rng.uniform(0.2, 1.5), wl_sigma=rng.uniform(2.0, 5.0)) for _ in range(2)]
    return e, s[0], s[1]


def ctxafs_item_specs(n, seed=3, widths=(512, 1024, 1536, 2048), angles=(360, 720, 900, 1200), max_drop=0.10):
    """n slice shapes of a CT-XAFS stack: width w (bins = w) from `widths`, a projection count
    from `angles` over 180 deg with 0..max_drop of the angles dropped at random (seeded).
    Returns a list of (w, angle array in degrees)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        w = int(rng.choice(widths))
        pa = int(rng.choice(angles))
        drop = int(rng.integers(0, int(max_drop * pa) + 1))
        keep = np.sort(rng.choice(pa, pa - drop, replace=False))
        out.append((w, (keep * (180.0 / pa)).astype(np.float32)))
    return out


def xanes_fields(w, seed):
    """The energy-independent fields of one CT-XAFS slice: the sample's support (a few
    ellipses) and the seeded per-voxel fraction f of spectrum 1 (piecewise constant per
    16x16 voxel block), both [w][w] float64."""
    rng = np.random.default_rng(seed)
    support = rasterize_ellipses(ellipse_params(w, 4, seed, axes=(0.1 * w, 0.35 * w), mu=(1.0, 1.0)), w, w) > 0
    f = rng.uniform(0.0, 1.0, (w // 16 + 1, w // 16 + 1))
    f = np.kron(f, np.ones((16, 16)))[:w, :w]
    return support.astype(np.float64), f


def xanes_slice(w, energy_index, seed, spectra, mu_scale=0.02, torch_device=None, fields=None):
    """One slice of a CT-XAFS volume at one energy: inside a few ellipses, each voxel is the
    mixture f*S1(E) + (1-f)*S2(E) with a seeded per-voxel fraction f (smoothed noise), times
    mu_scale per pixel.  fields: xanes_fields(w, seed), computed once for many energies."""
    e, s1, s2 = spectra
    support, f = xanes_fields(w, seed) if fields is None else fields
    mu = support * (f * s1[energy_index] + (1.0 - f) * s2[energy_index]) * mu_scale
    mu = mu.astype(np.float32)
    if torch_device is not None:
        import torch
        return torch.from_numpy(mu).to(torch_device)
    return mu
