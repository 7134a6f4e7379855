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


def test_batch_run_leaves_patches_out(cuda):
    """A run with some images None (the serving loop's slots): the other patches' results
    are bit-identical to a run with every patch, and the left-out patches' outputs are not
    touched."""
    import torch
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    from mesolf_gb300.api import _fortran
    H, Ht = synth.make_psf(61, 15, np.arange(7) - 3, seed=1)
    psf = PhaseSpacePSF(H, Ht)
    lfs = frames(H, n_frames=1)
    shapes = [g[0] for g in GEO]
    planes = [g[1] for g in GEO]
    b = BatchSolver(psf, shapes, planes)
    imgs = [_fortran(torch.as_tensor(np.ascontiguousarray(lfs[p, 0])).cuda())[0] for p in range(len(GEO))]
    full = [o.cpu().numpy() for o in b.run(imgs, 2, precision="bf16x2")]
    for left_out in ([1], [0, 3]):
        outs = [torch.full((nz, xc, xr), -7.0, device="cuda").permute(2, 1, 0) for (xr, xc), (_, nz) in GEO]
        got = b.run([None if p in left_out else imgs[p] for p in range(len(GEO))], 2, precision="bf16x2",
                    outs=outs)
        for p in range(len(GEO)):
            g = got[p].cpu().numpy()
            if p in left_out:
                assert np.all(g == -7.0)
            else:
                assert np.array_equal(g, full[p]), (left_out, p)
    b.close()


def _long_batch(torch):
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    H, Ht = synth.make_psf(91, 15, np.arange(21) - 10, seed=3)
    psf = PhaseSpacePSF(H, Ht)
    shapes = [(600, 600), (450, 600), (600, 525)]
    b = BatchSolver(psf, shapes)
    imgs = [torch.rand((xc, xr), device="cuda").t() * 100 + 10 for xr, xc in shapes]
    return psf, b, shapes, imgs


def test_cancel_stops_a_running_batch_between_view_steps(cuda):
    """mlf_batch_cancel from another thread while a long synchronous run is on the GPU: the
    run returns MLF_ERR_CANCELLED early, its outputs are untouched, and the work set and the
    context keep working (the next run equals an uncancelled one)."""
    import threading
    import time

    import torch
    from mesolf_gb300 import MesoLFError, _lib
    psf, b, shapes, imgs = _long_batch(torch)
    ref = [o.cpu().numpy() for o in b.run(imgs, 2, precision="bf16x2")]   # warm-up: tuning, graphs
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run(imgs, 2, precision="bf16x2")
    t_two = time.perf_counter() - t0
    iters = max(20, int(2 * 2.0 / max(t_two, 1e-3)))                       # about two seconds
    outs = [torch.full((psf.Z, xc, xr), -3.0, device="cuda").permute(2, 1, 0) for xr, xc in shapes]
    box = {}

    def run():
        try:
            b.run(imgs, iters, precision="bf16x2", outs=outs)
            box["rc"] = 0
        except MesoLFError as e:
            box["rc"] = e.code
        box["t"] = time.perf_counter()

    th = threading.Thread(target=run)
    t_start = time.perf_counter()
    th.start()
    time.sleep(0.2)
    b.cancel()
    th.join(timeout=120)
    assert box.get("rc") == _lib.MLF_ERR_CANCELLED, box
    assert b.cancelled
    assert box["t"] - t_start < 0.5 * iters / 2 * t_two + 0.3          # stopped well before the end
    for o in outs:
        assert torch.all(o == -3.0)
    again = [o.cpu().numpy() for o in b.run(imgs, 2, precision="bf16x2")]
    assert not b.cancelled
    for a, r in zip(again, ref):
        assert np.array_equal(a, r)
    b.close()


def test_cancel_stops_a_plain_fp32_solve(cuda):
    import threading
    import time

    import torch
    from mesolf_gb300 import MesoLFError, PhaseSpacePSF, RLSolver, _lib
    H, Ht = synth.make_psf(91, 15, np.arange(21) - 10, seed=3)
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, (600, 600))
    lf = torch.rand((600, 600), device="cuda").t() * 100 + 10
    ref = s.run(lf, 1).cpu().numpy()
    out = torch.full((21, 600, 600), -5.0, device="cuda").permute(2, 1, 0)
    box = {}

    def run():
        try:
            s.run(lf, 200, out=out)
            box["rc"] = 0
        except MesoLFError as e:
            box["rc"] = e.code

    th = threading.Thread(target=run)
    th.start()
    time.sleep(0.2)
    s.cancel()
    th.join(timeout=300)
    assert box.get("rc") == _lib.MLF_ERR_CANCELLED and s.cancelled
    assert torch.all(out == -5.0)
    assert np.array_equal(s.run(lf, 1).cpu().numpy(), ref) and not s.cancelled


def test_server_cancel_queued_and_running(cuda):
    """SolveServer.cancel: a queued request is withdrawn at once; a running batch whose
    requests are all withdrawn stops, and its patches' next frames still equal a solve from
    the previous frame's volume."""
    import concurrent.futures
    import time

    import torch
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    from mesolf_gb300.api import _fortran
    from mesolf_gb300.serve import SolveServer
    H, Ht = synth.make_psf(61, 15, np.arange(7) - 3, seed=1)
    psf = PhaseSpacePSF(H, Ht)
    lfs = frames(H, n_frames=3)
    srv = SolveServer(psf, GEO, iters=400, precision="bf16x2", lanes=1, max_batch=len(GEO))
    f0 = [srv.submit(p, 0, lfs[p, 0]) for p in range(len(GEO))]
    first = [np.array(f.result(timeout=300)) for f in f0]
    f1 = [srv.submit(p, 1, lfs[p, 1]) for p in range(len(GEO))]
    time.sleep(0.25)                                          # well inside the 400-iteration batch
    assert all(srv.cancel(p, 1) for p in range(len(GEO)))     # running (or still queued)
    f2q = srv.submit(0, 2, lfs[0, 2])
    for f in f1:
        try:
            f.result(timeout=300)
            raised = False
        except concurrent.futures.CancelledError:
            raised = True
        assert raised
    res2 = np.array(f2q.result(timeout=300))
    srv.drain(timeout=120)
    srv.close()

    def dev(x):
        return _fortran(torch.as_tensor(np.ascontiguousarray(x)).cuda())[0]
    (xr, xc), planes = GEO[0]
    alone = BatchSolver(psf, [(xr, xc)], [planes])
    want = alone.run([dev(lfs[0, 2])], 400, precision="bf16x2", warm=[dev(first[0])])[0].cpu().numpy()
    assert rel_l2(res2, want) <= 1e-5
    alone.close()
