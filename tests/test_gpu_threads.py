"""Concurrent plans from host threads.  The reference runs one reconstruction thread per
device beside its input and output threads (CT_reconstruction/GPU.cpp:629-658); the ABI keeps
no shared mutable state between plans, so two host threads, each with its own plan on one
context, run blocking host-buffer OS-EM calls at the same time (ctypes releases the GIL for
the call).  Every result equals the same call made alone: bit for bit with the plain kernels,
to 1e-6 rel-L2 with the tiled ones (their per-tile partial sums meet in double atomics)."""
import threading

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernels", ["plain", "tiled"])
def test_two_threads_two_plans(gpu_ctx, kernels):
    import xct
    from xct import phantom as P
    kk = xct.KERNELS_PLAIN if kernels == "plain" else xct.KERNELS_TILED
    shapes = [(256, 256, 180, 10), (192, 200, 150, 5)]  # (n, px, pa, ss) per thread
    rng = np.random.default_rng(12)
    jobs = []
    for (n, px, pa, ss) in shapes:
        calls = []
        for _ in range(3):
            sinos = [rng.uniform(0.1, 1.0, (pa, px)).astype(np.float32) for _ in range(2)]
            calls.append(sinos)
        jobs.append(((n, px, pa, ss), calls))

    def make(shape):
        n, px, pa, ss = shape
        return xct.OSEMPlan(gpu_ctx, n, n, px, P.uniform_angles(pa), ss, 2, max_batch=2, kernels=kk)

    def run_all(plan, shape, calls):
        n = shape[0]
        out = []
        for sinos in calls:
            imgs = [np.ones((n, n), np.float32) for _ in sinos]
            plan.run(sinos, imgs)
            out.append(imgs)
        return out

    plans = [make(shape) for shape, _ in jobs]
    alone = [run_all(p, shape, calls) for p, (shape, calls) in zip(plans, jobs)]

    together = [None, None]
    errors = []
    start = threading.Barrier(2, timeout=60)

    def worker(k):
        try:
            start.wait()
            together[k] = run_all(plans[k], jobs[k][0], jobs[k][1])
        except Exception as e:  # reported below
            errors.append(repr(e))

    ts = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not errors, errors
    for k in range(2):
        for a_call, b_call in zip(alone[k], together[k]):
            for a, b in zip(a_call, b_call):
                assert np.isfinite(b).all()
                if kernels == "plain":
                    assert np.array_equal(a, b)
                else:
                    assert np.linalg.norm(a - b) / np.linalg.norm(a) <= 1e-6
    for p in plans:
        p.close()
