"""Compressed-sensing OS-EM (FISTA_OSEM_execution: OS-EM + ISTA3D/FISTA3D) on the GPU.

The proximal kernels are element-wise and bit-exact for the same input; with the plain
OS-EM kernels (bit-exact companions of the oracle's GPU order) the whole run is bit-exact
against the oracle.  The tiled kernels carry the OS-EM parity bar (1e-4 rel-L2, max-abs
1e-3 of the peak); the proximal selection is piecewise constant in its input, so it can
only move a voxel where the OS-EM rounding lands next to a selection boundary."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _plan(ctx, f, kernels):
    import xct
    n, px, pa, ss, it, dN = [int(v) for v in f["shape"]]
    return xct.OSEMPlan(ctx, n, n, px, f["angles"], ss, it, max_batch=dN, kernels=kernels)


def test_cs_plain_bit_exact(gpu_ctx):
    import xct
    f = _load("cs_64")
    plan = _plan(gpu_ctx, f, xct.KERNELS_PLAIN)
    d_s = torch.from_numpy(f["meas"]).cuda()
    d_x = torch.from_numpy(f["x0"]).cuda()
    plan.cs_run_device(d_s, d_x, cs_lambda=float(f["cs_lambda"][0]), sub=f["sub"])
    torch.cuda.synchronize()
    assert np.array_equal(d_x.cpu().numpy(), f["cs_gpu_order"])
    plan.close()


def test_cs_tiled_matches_reference(gpu_ctx):
    import xct
    f = _load("cs_64")
    plan = _plan(gpu_ctx, f, xct.KERNELS_TILED)
    d_s = torch.from_numpy(f["meas"]).cuda()
    d_x = torch.from_numpy(f["x0"]).cuda()
    plan.cs_run_device(d_s, d_x, cs_lambda=float(f["cs_lambda"][0]), sub=f["sub"])
    torch.cuda.synchronize()
    got = d_x.cpu().numpy()
    assert _rel(got, f["cs"]) <= 1e-4
    assert np.abs(got - f["cs"]).max() <= 1e-3 * np.abs(f["cs"]).max()
    # host-buffer form, and a second run on the same plan (buffers reused)
    out = [f["x0"][z].copy() for z in range(f["x0"].shape[0])]
    plan.cs_run([f["meas"][z].copy() for z in range(len(out))], out, cs_lambda=float(f["cs_lambda"][0]), sub=f["sub"])
    assert _rel(np.stack(out), got) <= 1e-6
    plan.close()


def test_cs_argument_errors(gpu_ctx):
    import xct
    f = _load("cs_64")
    plan = _plan(gpu_ctx, f, xct.KERNELS_TILED)
    d_s = torch.from_numpy(f["meas"]).cuda()
    d_x = torch.from_numpy(f["x0"]).cuda()
    for lam in (-1.0, float("nan"), float("inf")):
        with pytest.raises(xct.XCTError):
            plan.cs_run_device(d_s, d_x, cs_lambda=lam)
    plan.close()


def test_hybrid_with_compressed_sensing(gpu_ctx, oracle_lib):
    """hybrid_thread with CSitBool (GPU.cpp:1569-1571): FBP, base-up, then the compressed-
    sensing OS-EM on the corrected sinogram; against the oracle's composition of the three
    (each pinned to the reference's kernels), the FBP filter's rounding carried through."""
    import xct
    O = oracle_lib
    f = _load("cs_64")
    n, px, pa, ss, it, dN = [int(v) for v in f["shape"]]
    lam = float(f["cs_lambda"][0])
    plan = _plan(gpu_ctx, f, xct.KERNELS_TILED)
    d_s = torch.from_numpy(f["meas"]).cuda()
    d_x = torch.zeros((dN, n, n), device="cuda")
    plan.hybrid_cs(d_s, d_x, zp=128, baseup_order=4, cs_lambda=lam, sub=f["sub"])
    torch.cuda.synchronize()
    x0 = np.stack([O.base_up(O.fbp(f["meas"][z], f["angles"], n, n, 128), 4)[0] for z in range(dN)])
    want = O.cs_osem_run(x0, f["meas"], f["angles"], ss, it, lam, f["sub"], order=O.ORDER_LITERAL)
    got = d_x.cpu().numpy()
    assert _rel(got, want) <= 1e-4
    out = [np.zeros((n, n), np.float32) for _ in range(dN)]
    plan.hybrid_cs_run([f["meas"][z].copy() for z in range(dN)], out, zp=128, baseup_order=4, cs_lambda=lam,
                       sub=f["sub"])
    assert _rel(np.stack(out), got) <= 1e-6
    plan.close()
