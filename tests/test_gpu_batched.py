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


def test_batched_sinogram_correction_modes(gpu_ctx, oracle_lib):
    """Per-slice sinogram correction in a batch (modes 0-4 on slices of different shapes):
    each slice is corrected once per run, as OSEM_execution does with prjCorrection set
    (GPU.cpp:175-186), then reconstructed; against the oracle on the corrected sinogram and
    against the single-plan path with the same mode."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    ss, it = 5, 2
    spec = [(64, 64, 90, 0), (72, 80, 60, 1), (48, 56, 45, 2), (80, 64, 70, 3), (56, 60, 50, 4)]
    geoms, sinos, want, singles, host = [], [], [], [], []
    for k, (n, px, pa, mode) in enumerate(spec):
        ang = P.uniform_angles(pa)
        img = P.rasterize_ellipses(P.ellipse_params(n, 5, 40 + k, axes=(2, n / 4)), n, n)
        meas = P.noisy_log_sinogram(O.projection(img, ang, px), 1e5, k).astype(np.float32)
        geoms.append(xct.make_geom(n, n, px, ang, ss, it, correction_mode=mode))
        host.append(meas)
        sinos.append(torch.from_numpy(meas).cuda().contiguous())
        used = O.sino_correction(meas, ang, mode) if mode else meas
        want.append(O.osem_run(np.ones((n, n), np.float32), used, ang, ss, it, order=O.ORDER_LITERAL))
        plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, correction_mode=mode)
        x = torch.ones((1, n, n), device="cuda")
        plan.run_device(sinos[-1].reshape(1, pa, px), x)
        torch.cuda.synchronize()
        singles.append(x[0].cpu().numpy().astype(np.float64))
        plan.close()
    bp = xct.BatchPlan(gpu_ctx, geoms, it)
    for replay in range(2):
        imgs = [torch.ones((n, n), device="cuda") for n, _, _, _ in spec]
        bp.run(sinos, imgs)
        torch.cuda.synchronize()
        for k, (x, ref, single) in enumerate(zip(imgs, want, singles)):
            got = x.cpu().numpy().astype(np.float64)
            assert np.linalg.norm(got - single) / np.linalg.norm(single) <= 1e-6, (replay, k)
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-4, (replay, k)
            assert np.abs(got - ref).max() <= 1e-3 * np.abs(ref).max(), (replay, k)
    # the caller's sinograms are not modified (the corrected copies live in the plan)
    for k in range(len(spec)):
        assert np.array_equal(sinos[k].cpu().numpy(), host[k])
    bp.close()


def test_batched_compressed_sensing_stacks(gpu_ctx, oracle_lib):
    """Compressed-sensing OS-EM in a batch plan over three stacks of different image sizes
    (3 x 64^2, 2 x 48^2, 1 x 40^2; each stack's images one array), against the oracle's
    FISTA_OSEM_execution of each stack and against the single-plan call."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    ss, it, lam = 5, 2, 1.0e-4
    stacks = [(64, 64, 90, 3), (48, 50, 60, 2), (40, 40, 45, 1)]
    geoms, sinos, want, singles, arrays = [], [], [], [], []
    for s_i, (n, px, pa, dN) in enumerate(stacks):
        ang = P.uniform_angles(pa)
        prm = P.ellipsoid_params(n, dN, count=5, seed=50 + s_i)
        meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, px), 1e4, z)
                         for z in range(dN)]).astype(np.float32)
        for z in range(dN):
            geoms.append(xct.make_geom(n, n, px, ang, ss, it))
            sinos.append(torch.from_numpy(meas[z]).cuda().contiguous())
        want.append(O.cs_osem_run(np.ones((dN, n, n), np.float32), meas, ang, ss, it, lam))
        plan = xct.OSEMPlan(gpu_ctx, n, n, px, ang, ss, it, max_batch=dN)
        x = torch.ones((dN, n, n), device="cuda")
        plan.cs_run_device(torch.from_numpy(meas).cuda(), x, cs_lambda=lam)
        torch.cuda.synchronize()
        singles.append(x.cpu().numpy().astype(np.float64))
        plan.close()
    bp = xct.BatchPlan(gpu_ctx, geoms, it)
    bp.set_cs([d for _, _, _, d in stacks], cs_lambda=lam)
    for replay in range(2):
        arrays = [torch.ones((dN, n, n), device="cuda") for n, _, _, dN in stacks]
        imgs = [a[z] for a in arrays for z in range(a.shape[0])]
        bp.run(sinos, imgs)
        torch.cuda.synchronize()
        for s_i, a in enumerate(arrays):
            got = a.cpu().numpy().astype(np.float64)
            assert np.linalg.norm(got - singles[s_i]) / np.linalg.norm(singles[s_i]) <= 1e-6, (replay, s_i)
            ref = want[s_i]
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-4, (replay, s_i)
    # a stack whose images are not one array is refused
    loose = [torch.ones((n, n), device="cuda") for n, _, _, dN in stacks for _ in range(dN)]
    with pytest.raises(xct.XCTError):
        bp.run(sinos, loose)
    bp.close()


def test_uniform_batch_route(gpu_ctx, oracle_lib):
    """A batch of 16 slices of one geometry (512^2, 90 angles; the slice-interleaved forward
    projector's shape) is one geometry group: in one pair of arrays it runs in place through
    a single-shape plan, 16 slices per call, and gives the single-plan result; with the
    images in separate allocations it runs through the plan's scratch pair; with groups off
    the same plan replays its graph of persistent launches; all against the oracle."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, pa, ss, it, dn = 512, 90, 5, 2, 16
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, dn, count=8, seed=61)
    meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, n), 1e5, z)
                     for z in range(dn)]).astype(np.float32)
    d_s = torch.from_numpy(meas).cuda()
    geoms = [xct.make_geom(n, n, n, ang, ss, it) for _ in range(dn)]
    bp = xct.BatchPlan(gpu_ctx, geoms, it)
    assert bp.uniform() == dn
    assert bp.groups() == (1, dn)
    plan = xct.OSEMPlan(gpu_ctx, n, n, n, ang, ss, it, max_batch=dn)
    x1 = torch.ones((dn, n, n), device="cuda")
    plan.run_device(d_s, x1)
    arr = torch.ones((dn, n, n), device="cuda")
    bp.run([d_s[z] for z in range(dn)], [arr[z] for z in range(dn)])
    loose_s = [d_s[z].clone() for z in reversed(range(dn))][::-1]
    sep = [torch.ones((n, n), device="cuda") for _ in range(dn)]
    bp.run(loose_s, sep)
    bp.set_grouping(False)
    gsep = [torch.ones((n, n), device="cuda") for _ in range(dn)]
    bp.run([d_s[z] for z in range(dn)], gsep)
    torch.cuda.synchronize()
    single = x1.cpu().numpy().astype(np.float64)
    routed = arr.cpu().numpy().astype(np.float64)
    scratch = torch.stack(sep).cpu().numpy().astype(np.float64)
    graph = torch.stack(gsep).cpu().numpy().astype(np.float64)
    assert np.linalg.norm(scratch - routed) / np.linalg.norm(routed) <= 1e-6
    assert np.linalg.norm(routed - single) / np.linalg.norm(single) <= 1e-6
    assert np.linalg.norm(graph - single) / np.linalg.norm(single) <= 1e-6
    for z in (0, dn - 1):
        ref = O.osem_run(np.ones((n, n), np.float32), meas[z], ang, ss, it, order=O.ORDER_LITERAL)
        for got in (routed[z], graph[z]):
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-4, z
            assert np.abs(got - ref).max() <= 1e-3 * np.abs(ref).max(), z
    plan.close()
    bp.close()
    # different angle lists: not uniform
    g2 = [xct.make_geom(64, 64, 64, ang, ss, it), xct.make_geom(64, 64, 64, ang + 0.5, ss, it)]
    bp2 = xct.BatchPlan(gpu_ctx, g2, it)
    assert bp2.uniform() == 0
    assert bp2.groups() == (0, 0)
    bp2.close()


def test_uniform_batch_route_with_correction(gpu_ctx, oracle_lib):
    """A uniform batch whose geometry carries a sinogram correction (mode 3): the geometry
    group corrects inside its single-shape plan, the graph (groups off) in its own correction
    launch; both give the oracle's OS-EM of the corrected sinogram."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    n, pa, ss, it, dn, mode = 128, 90, 5, 2, 9, 3
    ang = P.uniform_angles(pa)
    prm = P.ellipsoid_params(n, dn, count=6, seed=71)
    meas = np.stack([P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z, n, n), ang, n), 1e5, z)
                     for z in range(dn)]).astype(np.float32)
    d_s = torch.from_numpy(meas).cuda()
    geoms = [xct.make_geom(n, n, n, ang, ss, it, correction_mode=mode) for _ in range(dn)]
    bp = xct.BatchPlan(gpu_ctx, geoms, it)
    assert bp.uniform() == dn
    arr = torch.ones((dn, n, n), device="cuda")
    bp.run([d_s[z] for z in range(dn)], [arr[z] for z in range(dn)])
    bp.set_grouping(False)
    sep = [torch.ones((n, n), device="cuda") for _ in range(dn)]
    bp.run([d_s[z] for z in range(dn)], sep)
    torch.cuda.synchronize()
    routed = arr.cpu().numpy().astype(np.float64)
    graph = torch.stack(sep).cpu().numpy().astype(np.float64)
    assert np.linalg.norm(routed - graph) / np.linalg.norm(graph) <= 1e-6
    for z in (0, dn - 1):
        ref = O.osem_run(np.ones((n, n), np.float32), O.sino_correction(meas[z], ang, mode), ang, ss, it,
                         order=O.ORDER_LITERAL)
        assert np.linalg.norm(routed[z] - ref) / np.linalg.norm(ref) <= 1e-4, z
    # the caller's sinograms are not modified
    assert np.array_equal(d_s.cpu().numpy(), meas)
    bp.close()


def test_geometry_groups_in_a_mixed_batch(gpu_ctx, oracle_lib):
    """A batch of 27 slices in interleaved order: 16 of geometry A (512^2, 90 angles: the
    slice-interleaved kernels' shape), 8 of geometry B (80x72 image, 88 bins, 45 angles with
    3 dropped, centre +1.5 bins, correction mode 2) and 3 of shapes of their own.  A and B
    are geometry groups (single-shape plans, their slices copied through the scratch pair),
    the 3 others run in the graph; every slice agrees with the graph serving all 27 (groups
    off), and slices of each kind with the oracle.  The caller's sinograms are unchanged."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    ss, it = 5, 2
    rng = np.random.default_rng(77)
    angA = P.uniform_angles(90)
    keepB = np.sort(rng.choice(45, 42, replace=False))
    angB = (keepB * 4.0).astype(np.float32)
    kinds = ["A"] * 16 + ["B"] * 8 + ["C0", "C1", "C2"]
    order = list(rng.permutation(len(kinds)))
    prmA = P.ellipsoid_params(512, 16, count=8, seed=78)
    specs, geoms, sinos, host = [], [], [], []
    za = zb = 0
    for k in order:
        kind = kinds[k]
        if kind == "A":
            nx = ny = px = 512
            ang, cx, mode = angA, None, 0
            img = P.ellipsoid_slice(prmA, za, nx, ny)
            za += 1
        elif kind == "B":
            nx, ny, px, ang, cx, mode = 80, 72, 88, angB, 44 + 1.5, 2
            m = max(nx, ny)
            img = P.rasterize_ellipses(P.ellipse_params(m, 4, 90 + zb, axes=(2, m / 4)), m, m)[:ny, :nx].copy()
            zb += 1
        else:
            c = int(kind[1])
            nx = ny = 40 + 16 * c
            px, ang, cx, mode = nx + 8, P.uniform_angles(30 + 10 * c), None, 0
            img = P.rasterize_ellipses(P.ellipse_params(nx, 4, 95 + c, axes=(2, nx / 4)), nx, nx)
        ccx = px * 0.5 if cx is None else cx
        meas = P.noisy_log_sinogram(O.projection(img, ang, px, cx=ccx), 1e5, len(specs)).astype(np.float32)
        specs.append((kind, nx, ny, px, ang, ccx, mode))
        geoms.append(xct.make_geom(nx, ny, px, ang, ss, it, center_bin=ccx, correction_mode=mode))
        host.append(meas)
        sinos.append(torch.from_numpy(meas).cuda().contiguous())
    bp = xct.BatchPlan(gpu_ctx, geoms, it)
    assert bp.groups() == (2, 24)
    assert bp.uniform() == 0
    grouped = [torch.ones((ny, nx), device="cuda") for _, nx, ny, _, _, _, _ in specs]
    bp.run(sinos, grouped)
    bp.set_grouping(False)
    graph = [torch.ones((ny, nx), device="cuda") for _, nx, ny, _, _, _, _ in specs]
    bp.run(sinos, graph)
    torch.cuda.synchronize()
    checked = set()
    for i, (kind, nx, ny, px, ang, cx, mode) in enumerate(specs):
        a = grouped[i].cpu().numpy().astype(np.float64)
        b = graph[i].cpu().numpy().astype(np.float64)
        assert np.all(np.isfinite(a)), i
        assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-6, (i, kind)
        if kind[0] not in checked:
            checked.add(kind[0])
            used = O.sino_correction(host[i], ang, mode) if mode else host[i]
            ref = O.osem_run(np.ones((ny, nx), np.float32), used, ang, ss, it, cx=cx, order=O.ORDER_LITERAL)
            assert np.linalg.norm(a - ref) / np.linalg.norm(ref) <= 1e-4, (i, kind)
            assert np.abs(a - ref).max() <= 1e-3 * np.abs(ref).max(), (i, kind)
    assert checked == {"A", "B", "C"}
    for i in range(len(specs)):
        assert np.array_equal(sinos[i].cpu().numpy(), host[i])
    bp.close()
