"""Serving loop on the GPU: a stream of frames for uneven patches, two lanes, batches of
two; every result must equal the same patch's solve alone (same warm start), within
relative L2 1e-5 (the batch kernels keep each patch's arithmetic separate, so the
results are expected to be bit-identical)."""
import numpy as np
import pytest

from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu

GEO = [((75, 60), (0, 7)), ((45, 105), (2, 4)), ((60, 60), (0, 7)), ((30, 45), (1, 5))]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def frames(H, n_frames=3, seed=0):
    rng = np.random.default_rng(seed)
    out = {}
    for p, ((xr, xc), (z0, nz)) in enumerate(GEO):
        vol = synth.make_volume(xr, xc, nz, 8, 3.0, "uniform", 0.01, seed=seed + p)
        base = synth.forward_project_full(H[:, :, :, :, z0:z0 + nz], vol)
        for f in range(n_frames):
            lam = np.clip(base, 0, None) * (500.0 / base.max()) * rng.uniform(0.8, 1.2)
            out[p, f] = np.asfortranarray(rng.poisson(lam).astype(np.float32))
    return out


def test_results_same_alone_and_in_the_mix(cuda):
    import time

    import torch
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    from mesolf_gb300.api import _fortran
    from mesolf_gb300.serve import SolveServer

    H, Ht = synth.make_psf(61, 15, np.arange(7) - 3, seed=1)
    psf = PhaseSpacePSF(H, Ht)
    lfs = frames(H)
    srv = SolveServer(psf, GEO, iters=2, precision="bf16x2", lanes=2, max_batch=2)
    futs = {}
    t0 = time.perf_counter()
    order = [(p, f) for f in range(3) for p in (2, 0, 3, 1)]
    for k, (p, f) in enumerate(order):
        futs[p, f] = srv.submit(p, f, lfs[p, f], t_arrival=t0 + 0.001 * k)
        if k % 3 == 2:
            time.sleep(0.02)
    mix = {k: np.array(v.result(timeout=300)) for k, v in futs.items()}
    srv.drain(timeout=60)
    rep = srv.report()
    srv.close()
    assert rep["requests"] == 12 and rep["voxels"] > 0 and rep["p99_ms"] >= rep["p50_ms"] > 0
    assert rep["mean_batch"] > 1.0          # patches were batched together

    def dev(x):
        return _fortran(torch.as_tensor(np.ascontiguousarray(x)).cuda())[0]

    for p, ((xr, xc), planes) in enumerate(GEO):
        alone = BatchSolver(psf, [(xr, xc)], [planes])
        prev = None
        for f in range(3):
            out = alone.run([dev(lfs[p, f])], 2, precision="bf16x2",
                            warm=None if prev is None else [dev(prev)])[0].cpu().numpy()
            assert out.shape == (xr, xc, planes[1])
            assert rel_l2(mix[p, f], out) <= 1e-5, (p, f, rel_l2(mix[p, f], out))
            prev = mix[p, f]
        alone.close()


def test_plan_bytes_bounds_the_allocation(cuda):
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    H, Ht = synth.make_psf(61, 15, np.arange(7) - 3, seed=1)
    psf = PhaseSpacePSF(H, Ht)
    shapes = [g[0] for g in GEO]
    planes = [g[1] for g in GEO]
    plan = BatchSolver.plan_bytes(psf, shapes, planes)
    b = BatchSolver(psf, shapes, planes)
    assert b.device_bytes <= plan
    # members build their filter plans and scratch on the first solve
    import torch
    b.run([torch.rand((xc, xr), device="cuda").t() for xr, xc in shapes], 1)
    assert b.device_bytes <= plan <= 1.05 * b.device_bytes + (1 << 20), (plan, b.device_bytes)
