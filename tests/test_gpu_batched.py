"""Batched OS-EM over slices of different shapes (xct_batch_plan_*): one CUDA graph of
persistent launches fed by a device work queue.  Each slice must come out as the single-plan
path computes it (same kernels and tiles; only the order of the double-precision partial-sum
atomics may differ) and within the parity bar of the reference."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SS, IT = 5, 3


def _items():
    rng = np.random.default_rng(21)
    spec = [  # nx, ny, px, pa, drop, centre offset, cover
        (64, 64, 64, 90, 0, 0.0, False),
        (96, 80, 110, 60, 5, 0.0, False),
        (40, 40, 48, 36, 0, 0.0, True),
        (130, 130, 150, 72, 3, 2.5, False),
        (256, 256, 256, 180, 9, 0.0, False),
        (50, 70, 80, 45, 2, 0.0, True),
    ]
    out = []
    for k, (nx, ny, px, pa, drop, off, cover) in enumerate(spec):
        ang = np.arange(pa) * (180.0 / pa)
        keep = np.sort(rng.choice(pa, pa - drop, replace=False))
        out.append((nx, ny, px, ang[keep].astype(np.float32), px * 0.5 + off, cover, 30 + k))
    return out


def test_batched_graph_matches_single_plans(gpu_ctx, oracle_lib):
    import xct
    from xct import phantom as P
    O = oracle_lib
    items = _items()
    geoms, sinos, x0s, singles, refs = [], [], [], [], []
    for nx, ny, px, ang, cx, cover, seed in items:
        m = max(nx, ny)
        img = P.rasterize_ellipses(P.ellipse_params(m, 6, seed, axes=(2, m / 4)), m, m)[:ny, :nx].copy()
        meas = P.noisy_log_sinogram(O.projection(img, ang, px, cx=cx), 1e5, seed)
        mode = xct.SUBSETS_COVER if cover else xct.SUBSETS_REF
        geoms.append(xct.make_geom(nx, ny, px, ang, SS, IT, center_bin=cx, subset_mode=mode))
        sinos.append(torch.from_numpy(meas).cuda().contiguous())
        x0 = np.ones((ny, nx), np.float32)
        x0s.append(x0)
        plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, ang, SS, IT, center_bin=cx, subset_mode=mode)
        d_x = torch.from_numpy(x0).cuda().reshape(1, ny, nx).contiguous()
        plan.run_device(sinos[-1].reshape(1, *meas.shape), d_x)
        torch.cuda.synchronize()
        singles.append(d_x[0].cpu().numpy().astype(np.float64))
        plan.close()
        refs.append(O.osem_run(x0, meas, ang, SS, IT, cx=cx, cover=cover, order=O.ORDER_LITERAL))
    bp = xct.BatchPlan(gpu_ctx, geoms, IT)
    for replay in range(2):  # capture, then replay with fresh image buffers
        imgs = [torch.from_numpy(x).cuda().contiguous() for x in x0s]
        bp.run(sinos, imgs)
        torch.cuda.synchronize()
        for k, (d_x, single, ref) in enumerate(zip(imgs, singles, refs)):
            got = d_x.cpu().numpy().astype(np.float64)
            assert np.linalg.norm(got - single) / np.linalg.norm(single) <= 1e-6, (replay, k)
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-4, (replay, k)
            assert np.abs(got - ref).max() <= 1e-3 * np.abs(ref).max(), (replay, k)
    bp.close()


def test_batched_rejects_mixed_subset_counts(gpu_ctx):
    import xct
    g1 = xct.make_geom(32, 32, 32, np.arange(20, dtype=np.float32) * 9, 4, 1)
    g2 = xct.make_geom(32, 32, 32, np.arange(20, dtype=np.float32) * 9, 5, 1)
    with pytest.raises(xct.XCTError) as e:
        xct.BatchPlan(gpu_ctx, [g1, g2], 1)
    assert "same subset count" in str(e.value)


def test_volume_stream_matches_batches(gpu_ctx, oracle_lib):
    """xct_osem_run_volume over 7 slices in batches of 3 (two staging sets, overlapped
    copies from page-locked host tensors) gives each slice the single-batch result; the
    rotation centre is off px/2 by +3.5 bins (the full-volume workload's offset)."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, ss, it, nz = 96, 100, 72, 6, 2, 7
    cx = px / 2 + 3.5
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, nz, count=8, seed=6)
    sinos = [P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, px, cx=cx), 2e4, z)
             for z in range(nz)]
    plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, center_bin=cx, max_batch=3)
    hs = [torch.from_numpy(s).pin_memory() for s in sinos]
    hi = [torch.ones((n, n)).pin_memory() for _ in range(nz)]
    plan.run_volume(hs, hi)
    x0 = np.ones((n, n), np.float32)
    for z in range(nz):
        ref = O.osem_run(x0, sinos[z], ang, ss, it, cx=cx, order=O.ORDER_LITERAL)
        got = hi[z].numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-4, z
    # pageable numpy buffers: same results
    out = [np.ones((n, n), np.float32) for _ in range(nz)]
    plan.run_volume([s.copy() for s in sinos], out)
    for z in range(nz):
        assert np.linalg.norm(out[z] - hi[z].numpy()) / np.linalg.norm(hi[z].numpy()) <= 1e-6
    plan.close()
