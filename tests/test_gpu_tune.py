"""The forward projector's tile autotuner: every (tile side, angles per CTA) candidate gives
the same OS-EM (only the order of the per-tile double partial sums changes), the autotuner
keeps a valid choice, and its JSON cache is read back by later plans."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_every_tile_candidate_gives_the_same_osem(gpu_ctx):
    import xct
    f = dict(np.load(os.path.join(GOLDEN, "cfg1_256.npz")))
    nx, ny, px, pa, ss, it = [int(v) for v in f["shape"]]
    d_s = torch.from_numpy(f["meas"]).cuda()[None].contiguous()
    plan = xct.OSEMPlan(gpu_ctx, nx, ny, px, f["angles"], ss, it)
    results = {}
    for T in (44, 60, 76, 92):
        for chunk in (8, 16, 128):
            plan.set_tuning(T, chunk)
            assert plan.tuning() == (T, chunk)
            d_x = torch.ones((1, ny, nx), device="cuda")
            plan.run_device(d_s, d_x, sub=f["sub"])
            torch.cuda.synchronize()
            results[(T, chunk)] = d_x[0].cpu().numpy()
    ref = results[(92, 128)]
    for k, v in results.items():
        assert _rel(v, ref) <= 1e-6, k
        assert _rel(v, f["osem"]) <= 1e-4, k
    with pytest.raises(xct.XCTError):
        plan.set_tuning(50, 16)
    with pytest.raises(xct.XCTError):
        plan.set_tuning(92, 200)
    plan.close()


def test_autotune_and_cache_file(gpu_ctx, tmp_path):
    import xct
    cache = tmp_path / "tune.json"
    ang = np.arange(180, dtype=np.float32)
    plan = xct.OSEMPlan(gpu_ctx, 256, 256, 256, ang, 10, 1, max_batch=2)
    T, c = plan.autotune(dN=2, cache_path=cache)
    assert T in (44, 60, 76, 92) and 1 <= c <= 128
    data = json.loads(cache.read_text())
    assert data["xct_tune_cache"] == 1 and len(data["entries"]) == 1
    (key, entry), = data["entries"].items()
    assert entry["fwd_tile"] == T and entry["ang_chunk"] == c and entry["ms"] > 0
    assert "|256x256|256x180|ss10|dN2" in key
    plan.close()
    # a later plan of the same shape starts with the cached choice (file named by the
    # environment; the in-process copy is bypassed by a different key's lookup order)
    data["entries"][key]["fwd_tile"] = 44
    data["entries"][key]["ang_chunk"] = 8
    cache.write_text(json.dumps(data))
    os.environ["XCT_TUNE_CACHE"] = str(cache)
    try:
        p2 = xct.OSEMPlan(gpu_ctx, 256, 256, 256, ang, 10, 1, max_batch=2)
        assert p2.tuning() in ((T, c), (44, 8))  # the process cache may answer first
        p2.autotune(dN=2, cache_path=cache, force=True)
        assert p2.tuning()[0] in (44, 60, 76, 92)
        p2.close()
    finally:
        del os.environ["XCT_TUNE_CACHE"]


def test_batch_autotune_keeps_results(gpu_ctx, oracle_lib):
    import xct
    from xct import phantom as P
    O = oracle_lib
    specs = [(64, 64, 40), (128, 128, 90), (96, 96, 60)]
    geoms, sinos, x0s = [], [], []
    for k, (n, px, pa) in enumerate(specs):
        ang = P.uniform_angles(pa)
        img = P.ellipse_phantom(n, 5, 10 + k, axes=(3, n / 4))
        meas = P.noisy_log_sinogram(O.projection(img, ang, px), 1e5, k)
        geoms.append(xct.make_geom(n, n, px, ang, 5, 2))
        sinos.append(torch.from_numpy(meas).cuda())
        x0s.append(np.ones((n, n), np.float32))
    bp = xct.BatchPlan(gpu_ctx, geoms, 2)
    imgs0 = [torch.from_numpy(x).cuda() for x in x0s]
    bp.run(sinos, imgs0)
    torch.cuda.synchronize()
    T, c = bp.autotune(force=True)
    assert T in (44, 60, 76, 92) and 1 <= c <= 128
    imgs1 = [torch.from_numpy(x).cuda() for x in x0s]
    bp.run(sinos, imgs1)
    torch.cuda.synchronize()
    for a, b in zip(imgs0, imgs1):
        assert _rel(b.cpu().numpy(), a.cpu().numpy()) <= 1e-6
    bp.close()
