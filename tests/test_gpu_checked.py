"""The bounds-checked build (libxct_checked.so, -DXCT_CHECKED): every shared-memory access
whose address the kernels derive from geometry -- the forward tile's footprint loads and
accumulator rows (per-slice and slice-interleaved tiles), the adjoint's shared accumulator, the OS-EM and FBP backprojectors' bin
windows -- is tested against its buffer.  A child process runs those kernels through the
checked library on awkward shapes (every forward tile size, odd sizes, an off-centre
rotation axis, a 360-degree scan, batched mixed shapes) and must report no skipped access;
its results equal the standard library's."""
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "ct-xafs_analysis_gb300")

CASES = [  # nx, ny, px, pa, ss, span (deg), centre offset
    (97, 61, 120, 45, 5, 180.0, 0.0),
    (130, 130, 200, 64, 4, 360.0, 3.5),
    (200, 150, 171, 30, 3, 180.0, -7.25),
]

RUN = r"""
import sys, numpy as np, torch, xct
from xct import phantom as P
CASES = %r
ctx = xct.Context(0)
out = {}
for ci, (nx, ny, px, pa, ss, span, off) in enumerate(CASES):
    rng = np.random.default_rng(ci)
    ang = np.sort(rng.uniform(0, span, pa)).astype(np.float32)
    m = max(nx, ny)
    img = P.rasterize_ellipses(P.ellipse_params(m, 6, ci, axes=(3, m / 4)), m, m)[:ny, :nx] + np.float32(0.01)
    img = torch.from_numpy(np.ascontiguousarray(img, np.float32)).cuda()[None].contiguous()
    plan = xct.OSEMPlan(ctx, nx, ny, px, ang, ss, 2, center_bin=px * 0.5 + off, max_batch=2)
    meas = torch.empty((2, pa, px), device="cuda")
    plan.fwd(torch.cat([img, img.flip(1)]).contiguous(), meas)
    for T in (44, 60, 76, 92):
        for chunk in (16, 128):
            plan.set_tuning(T, chunk)
            x = torch.ones((2, ny, nx), device="cuda")
            plan.run_device(meas, x)
            out["osem_%%d_%%d_%%d" %% (ci, T, chunk)] = x.cpu().numpy()
    y = torch.from_numpy(rng.uniform(0, 1, (2, pa, px)).astype(np.float32)).cuda()
    a = torch.empty((2, ny, nx), device="cuda")
    plan.adj(y, a)
    out["adj_%%d" %% ci] = a.cpu().numpy()
    f = torch.empty((2, ny, nx), device="cuda")
    plan.fbp_backproject(y, f)
    out["fbpbp_%%d" %% ci] = f.cpu().numpy()
    plan.close()
    # the slice-interleaved forward projector: nine slices (a group of eight, then one)
    plan9 = xct.OSEMPlan(ctx, nx, ny, px, ang, ss, 2, center_bin=px * 0.5 + off, max_batch=9)
    img9 = torch.cat([img * (1.0 + 0.1 * j) for j in range(9)]).contiguous()
    for chunk in (16, 128):
        plan9.set_multislice(chunk)
        s9 = torch.empty((9, pa, px), device="cuda")
        plan9.fwd(img9, s9)
        out["msfwd_%%d_%%d" %% (ci, chunk)] = s9.cpu().numpy()
        x = torch.ones((9, ny, nx), device="cuda")
        plan9.run_device(s9, x)
        out["msosem_%%d_%%d" %% (ci, chunk)] = x.cpu().numpy()
    plan9.close()
# batched mixed shapes
geoms, sinos, imgs = [], [], []
for ci, (nx, ny, px, pa, ss, span, off) in enumerate(CASES):
    ang = np.sort(np.random.default_rng(10 + ci).uniform(0, span, pa)).astype(np.float32)
    geoms.append(xct.make_geom(nx, ny, px, ang, 3, 2))
    sinos.append(torch.from_numpy(np.random.default_rng(20 + ci).uniform(0.1, 2, (pa, px)).astype(np.float32)).cuda())
    imgs.append(torch.ones((ny, nx), device="cuda"))
bp = xct.BatchPlan(ctx, geoms, 2)
bp.run(sinos, imgs)
torch.cuda.synchronize()
for i, t in enumerate(imgs):
    out["batched_%%d" %% i] = t.cpu().numpy()
bp.close()
np.savez(sys.argv[1], **out)
if len(sys.argv) > 2:
    n, site, v, lo, hi = xct.check_report(ctx)
    print("CHECK", n, site, v, lo, hi)
""" % (CASES,)


def _run(tmp_path, variant):
    env = dict(os.environ)
    env["PYTHONPATH"] = PKG + os.pathsep + env.get("PYTHONPATH", "")
    env["XCT_LIB_VARIANT"] = variant
    res = tmp_path / (variant + ".npz")
    args = [sys.executable, "-c", RUN, str(res)] + (["report"] if variant == "checked" else [])
    r = subprocess.run(args, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return dict(np.load(res)), r.stdout


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_checked_build_finds_no_out_of_bounds_access(xct_lib, tmp_path):
    sys.path.insert(0, PKG)
    from xct import build
    build.build_lib(checked=True)
    checked, log = _run(tmp_path, "checked")
    line = [l for l in log.splitlines() if l.startswith("CHECK")][-1].split()
    assert int(line[1]) == 0, "skipped accesses: %s (site, index, lo, hi)" % line[1:]
    standard, _ = _run(tmp_path, "")
    assert set(checked) == set(standard)
    for k in checked:
        if k.startswith("fbpbp"):  # no atomics: the same sums in the same order
            assert np.array_equal(checked[k], standard[k]), k
        else:  # double (forward) and shared float (adjoint) atomics add in any order
            assert _rel(checked[k], standard[k]) <= 1e-6, k
