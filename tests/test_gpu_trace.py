"""XCT_TRACE: with the variable naming a file, every OS-EM call appends one JSON line with the
per-kernel totals and per-subset [forward, finalize, backprojection] milliseconds, and the
traced run gives the untraced run's result.  The variable is read once per process, so the
traced calls run in a child process."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "ct-xafs_analysis_gb300")

CHILD = r"""
import sys, numpy as np, torch, xct
from xct import phantom as P
n, px, pa, ss, it = 64, 72, 45, 5, 2
ang = P.uniform_angles(pa)
ctx = xct.Context(0)
out = {}
for kern, name in ((xct.KERNELS_TILED, "tiled"), (xct.KERNELS_PLAIN, "plain")):
    plan = xct.OSEMPlan(ctx, n, n, px, ang, ss, it, max_batch=2, kernels=kern)
    img = torch.from_numpy(P.rasterize_ellipses(P.ellipse_params(n, 4, 1, axes=(3, 16)), n, n)).cuda()
    sino = torch.empty((2, pa, px), device="cuda")
    plan.fwd(torch.stack([img, img.flip(0)]).contiguous(), sino)
    x = torch.ones((2, n, n), device="cuda")
    plan.run_device(sino, x)
    h = [np.zeros((n, n), np.float32) + 1]
    plan.run([sino[0].cpu().numpy().copy()], h)
    torch.cuda.synchronize()
    out[name] = (x.cpu().numpy(), h[0])
    plan.close()
np.savez(sys.argv[1], **{k + "_dev": v[0] for k, v in out.items()}, **{k + "_host": v[1] for k, v in out.items()})
"""


def _child(tmp_path, trace):
    env = dict(os.environ)
    env["PYTHONPATH"] = PKG + os.pathsep + env.get("PYTHONPATH", "")
    if trace:
        env["XCT_TRACE"] = str(trace)
    else:
        env.pop("XCT_TRACE", None)
    res = tmp_path / ("traced.npz" if trace else "plain.npz")
    r = subprocess.run([sys.executable, "-c", CHILD, str(res)], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return dict(np.load(res))


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_trace_lines_and_results(xct_lib, tmp_path):
    trace = tmp_path / "trace.jsonl"
    traced = _child(tmp_path, trace)
    plain = _child(tmp_path, None)
    lines = [json.loads(l) for l in open(trace)]
    assert [l["call"] for l in lines] == ["xct_osem_run_device", "xct_osem_run"] * 2
    assert [l["kernels"] for l in lines] == ["tiled", "tiled", "plain", "plain"]
    for l in lines:
        assert (l["nx"], l["px"], l["pa"], l["ss"], l["it"]) == (64, 72, 45, 5, 2)
        steps = l["subset_ms"]
        assert len(steps) == l["ss"] * l["it"] and all(len(s) == 3 for s in steps)
        for k, key in enumerate(("fwd", "finalize", "bp")):
            assert abs(sum(s[k] for s in steps) - l["ms"][key]) <= 1e-3 + 1e-3 * l["ms"][key]
        assert l["ms"]["total"] >= l["ms"]["fwd"] + l["ms"]["bp"] - 1e-3
        assert l["launches"] == l["ss"] * l["it"] * (3 if l["kernels"] == "tiled" else 2)
        assert l["slice_iters_per_s"] > 0
    assert [l["dN"] for l in lines] == [2, 1, 2, 1]
    for k in ("tiled_dev", "tiled_host", "plain_dev", "plain_host"):
        assert _rel(traced[k], plain[k]) <= 1e-6, k
    assert np.array_equal(traced["plain_dev"], plain["plain_dev"])  # plain kernels: no atomics
