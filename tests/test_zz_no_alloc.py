"""The allocation-free OS-EM entry point, xct_osem_run_static.

It serves callers that cannot allocate device memory (an acquisition loop that must never
stall on cudaMalloc, an application whose device memory belongs to its own pool): they pass
their own device sinograms and images, and the scratch lives in one static device array
inside the library.  This test calls it through the C ABI twice in a row -- the second call
starts from whatever the first left in that shared array -- and checks both results against
the plan-based entry point xct_osem_run_device within the tolerance the parity tests use for
the tiled kernels.  It runs last (file name) and also passes on its own in a fresh process,
where its first call performs the per-device set-up.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

REL = 1e-6  # the GPU-order tolerance of the parity tests (tiled ray sums add partials in double)


def _geom(xct, nx, ny, px, ang, ss, it, subset_mode=None):
    return xct.Geom(nx, ny, nx, ny, px, len(ang), ss, it, ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                    -1.0, xct.FETCH_EXACT, xct.SUBSETS_REF if subset_mode is None else subset_mode, 0, 1,
                    xct.KERNELS_TILED)


# (subset count, subset mode, explicit order): a power-of-two count (bit-reversed order), a
# count that does not divide the 120 angles in both subset modes (ratio rows never written
# read as zero / every row projected), and a caller-supplied order
CASES = [(8, "ref", None), (7, "ref", None), (7, "cover", None), (8, "ref", [3, 0, 6, 1, 7, 2, 5, 4])]


@pytest.mark.parametrize("ss,mode,order", CASES, ids=["ss8", "ss7-ref", "ss7-cover", "ss8-order"])
def test_static_scratch_entry_matches_plan_entry(gpu_ctx, oracle_lib, ss, mode, order):
    import xct
    from xct import phantom as P
    O = oracle_lib
    lib = xct.load()
    n, px, pa, it, dN = 160, 176, 120, 2, 2
    smode = xct.SUBSETS_COVER if mode == "cover" else xct.SUBSETS_REF
    ang = P.uniform_angles(pa)
    meas = np.stack([P.noisy_log_sinogram(
        O.projection(P.rasterize_ellipses(P.ellipse_params(n, 6, 20 + z, axes=(4, 40)), n, n), ang, px), 1e5, z)
        for z in range(dN)])
    x0 = np.ones((dN, n, n), np.float32)
    d_sino = torch.from_numpy(meas).cuda().contiguous()

    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, subset_mode=smode, max_batch=dN, kernels=xct.KERNELS_TILED)
    want = torch.from_numpy(x0).cuda().contiguous()
    plan.run_device(d_sino, want, dN=dN, sub=order)
    torch.cuda.synchronize()
    want = want.cpu().numpy().astype(np.float64)
    plan.close()

    g = _geom(xct, n, n, px, ang, ss, it, smode)
    sub = None if order is None else (ctypes.c_int * ss)(*order)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        got = torch.from_numpy(x0).cuda().contiguous()
        rc = lib.xct_osem_run_static(ctypes.byref(g), dN, d_sino.data_ptr(), got.data_ptr(), sub, -1, stream)
        assert rc == xct.XCT_OK, lib.xct_last_error()
        torch.cuda.synchronize()
        got = got.cpu().numpy()
        assert np.all(np.isfinite(got))
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel <= REL, "call %d: rel-L2 %.3e" % (call, rel)


def test_static_scratch_refuses_stream_capture(gpu_ctx):
    """Each call uploads its angle table from host stack memory, which a graph replay could
    not read, so a call on a capturing stream is refused before it enqueues anything."""
    import xct
    lib = xct.load()
    n, px, pa, ss = 64, 64, 30, 5
    ang = np.linspace(0, 180, pa, endpoint=False).astype(np.float32)
    g = _geom(xct, n, n, px, ang, ss, 1)
    sino = torch.ones((1, pa, px), device="cuda")
    img = torch.ones((1, n, n), device="cuda")
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        graph.capture_begin()
        rc = lib.xct_osem_run_static(ctypes.byref(g), 1, sino.data_ptr(), img.data_ptr(), None, -1, s.cuda_stream)
        img.add_(0.0)  # the captured graph is not empty
        graph.capture_end()
    assert rc == xct.XCT_E_UNSUPPORTED
    assert b"captured" in lib.xct_last_error()
    # outside a capture the same call runs
    rc = lib.xct_osem_run_static(ctypes.byref(g), 1, sino.data_ptr(), img.data_ptr(), None, -1,
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == xct.XCT_OK, lib.xct_last_error()
    torch.cuda.synchronize()
    assert bool(torch.isfinite(img).all())


def test_static_scratch_rejects_oversized_problems(gpu_ctx):
    import xct
    lib = xct.load()
    ang = np.linspace(0, 180, 1500, endpoint=False).astype(np.float32)
    g = _geom(xct, 2048, 2048, 2048, ang, 15, 1)
    d = torch.zeros(1, device="cuda")
    # two 2048^2 slices with 1500 angles need ~28 MB of scratch
    rc = lib.xct_osem_run_static(ctypes.byref(g), 2, d.data_ptr(), d.data_ptr(), None, -1, None)
    assert rc == xct.XCT_E_INVALID
    assert b"static scratch holds" in lib.xct_last_error()
