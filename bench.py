"""Throughput benchmark of the phase-space RL deconvolution on GB300.

One step = one complete solve (all RL iterations) of one synthetic light-field patch:
Nnum 15, 67 x 67 lenslets (1005 x 1005 px), 51 planes, PSF side 231 (phase-space side
225), 3 iterations, plain FP32 -- the "full single patch" workload.  `value` is
deconvolved voxels/s with the image already in HBM; `e2e` is the same solve through the
C ABI (mlf_solver_run) with pinned host buffers, the image copy in and the volume copy
out inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: patches are independent (replicas); each rank solves its own patch, no
collective on the data path; value = all ranks' voxels / max rank time.
The reference arm (--impl reference) times the CPU restatement of the reference's
algorithm (the oracle port; the MATLAB original cannot run here) on the host cores.

At N = 1 the line also carries: `roofline` (the fused view kernel against the FP32 FMA rate
measured live), `clocks`, `convergence` (the last iteration's FP64 relative change),
`mixed` (the same workload on the tensor cores, bf16x2, timed on iteration graphs without
timing nodes; its kernel times come from one instrumented solve after the timed region),
`precision_vs_fp64_oracle`, `serving` (36-patch carpet at 18 Hz), `batched` (64 uneven
patches), `mex_projector`, `seed_library`, `summary_image`, `rectification` and
`cpu_baseline`.

    python bench.py --profile --iters 1 [--planes P] [--precision bf16x2]   # one solve, for ncu
    python bench.py --only summary|rectify --frames F                      # one block, for ncu
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("deconvolved voxels/s, plain FP32 vs batched mixed-prec @≤1e-3 rel L2; p99 ms")
WORKLOAD = "lf1005x1005x51_k231_it3"
WORKLOAD_DESC = ("Nnum 15, 67x67 lenslets (1005x1005 px), 51 planes (0-200 um at 4 um), "
                 "PSF 231 px (phase-space 225), 2000 somas, 2000-photon Poisson image, 3 RL iterations")


KVIEW_DRAM_BYTES = 393.3e6     # k_view MODE_STEP launch, 1005x1005x51, FP32 (ncu, 2 launches: 229.9 + 163.4 MB)
# per launch, same workload, bf16x2 (ncu): the fused view step (back projection + next forward),
# and the two-kernel form it replaces (MLF_FUSED=0)
KTC_DRAM_BYTES = {"k_tc_bwdfwd": 412.4e6, "two_kernel_form": {"k_tc_bwd": 390.7e6, "k_tc_fwd": 220.5e6}}


def max_over_ranks(x, ws, dev=None):
    """The largest value over all ranks (the whole job takes as long as its slowest rank).
    Works on NCCL (device tensor) and gloo (host tensor) process groups."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    on_dev = dist.get_backend() == "nccl"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev if on_dev else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, ws, ms_max):
    """Whole-job throughput of independent replicas: all ranks' units / the slowest time."""
    return ws * units_per_rank / (ms_max * 1e-3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = [r.split(", ") for r in open(self.path).read().strip().splitlines() if r.strip()]
        try:
            os.unlink(self.path)
        except OSError:
            pass
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(device, rank, planes=None):
    import torch
    from mesolf_gb300 import synth
    w = synth.config2(seed=rank)
    if planes:
        # the deepest planes of the same workload: lateral size, PSF array side and the
        # per-plane kernel windows unchanged, fewer planes (and somas in proportion)
        k = w.z_idx[-planes:]
        w = synth.Workload(f"lf1005x1005x{planes}_k231_it3_deepest", w.N, w.lenslets, w.K0, k,
                           np.asarray(w.plane_sides)[-planes:], max(1, w.n_obj * planes // len(w.z_idx)),
                           w.sigma, w.peaks, w.background, w.photons, w.iters, w.seed)
    H, Ht = w.psf()
    lf = workload_image(w, H, device)
    return w, H, Ht, lf


def algorithmic_flop_per_view(Xr, Xc, Z, S, N):
    # forward (sampled outputs) + back projection (lattice-sparse input), 2 flop per MAC:
    # 2 * [(Xr/N)(Xc/N) Z S^2 + Xr Xc Z S^2 / N^2] = 4 Xr Xc Z S^2 / N^2
    return 4.0 * Xr * Xc * Z * S * S / (N * N)


def cpu_baseline_sample(H, Ht, lf, u=3, v=5, planes=None):
    """Time one RL view step of the C/OpenMP oracle port (FP64, all host threads) on the
    full workload (or its first `planes` planes).  Returns (seconds, threads, planes)."""
    from oracle import cbuild
    from oracle import mesolf_ref as R
    Z = H.shape[4] if planes is None else planes
    h, t = R.phasespace_view(H[:, :, :, :, :Z], Ht[:, :, :, :, :Z], u, v)
    X = np.full(lf.shape + (Z,), float(lf.sum()) / (lf.size * H.shape[4]))
    t0 = time.perf_counter()
    cbuild.view_step(h, t, lf.astype(np.float64), X, u, v, 0.3, 15)
    return time.perf_counter() - t0, cbuild.threads(), Z


def cpu_fft_sample(Xr, Xc, S, calls=3):
    """Seconds per conv2FFT call of the reference's GPU-branch formulation (conv2FFT.m:1-22 on
    the exsize grid of recon_…_with_filter.m:78-83), FP64 numpy (pocketfft, one thread).  One
    view step makes 3 Z such calls (forward per plane, C and D per plane)."""
    from oracle import mesolf_ref as R
    rng = np.random.default_rng(0)
    x = rng.random((Xr, Xc))
    m = rng.random((S, S))
    E = R.ex_size((Xr, Xc), S)
    R.conv2fft(x, m, E)
    t0 = time.perf_counter()
    for _ in range(calls):
        R.conv2fft(x, m, E)
    return (time.perf_counter() - t0) / calls, E


def progress(what):
    """One line per finished block on stderr: elapsed time and the process's peak host memory."""
    import resource
    rss = resource.getrusage(resource.RUSAGE_SELF).ru_maxrss / 1024.0
    print(f"[bench {time.perf_counter() - _T0:7.1f} s] {what} (peak RSS {rss:.0f} MB)", file=sys.stderr, flush=True)


_T0 = time.perf_counter()


def workload_config(ws, n_views):
    """The `config` of both arms' lines (the workload, not the implementation)."""
    return {"workload": WORKLOAD, "desc": WORKLOAD_DESC, "views_per_iteration": int(n_views),
            "parallelism": f"replicas x{ws}"}


def workload_image(w, H, device=None):
    """The workload's measured image.  For seed 0 (rank 0, and the reference arm) this is the
    image stored with the FP64 oracle fixture of the workload, so both arms and the error
    table solve the very same image; other seeds generate their own (replicas)."""
    if w.seed == 0 and os.path.exists(GOLDEN_C2) and w.name == WORKLOAD:
        return np.asfortranarray(np.load(GOLDEN_C2)["lf"].astype(np.float32))
    return w.measured(H, w.volume(), device=str(device) if device is not None else "cpu")


def active_views(H):
    """(u, v) of the views with non-zero weight in spiral order, and the weights, from the
    FP64 oracle (recon_..._with_filter.m:20-40 and :156-188)."""
    from oracle import mesolf_ref as R
    N = H.shape[2]
    wt = R.view_weights_from_sums(R.view_sums(H))
    i_idx, j_idx = R.gen_spiral(N)
    order = [(int(i_idx[k]) - 1, int(j_idx[k]) - 1) for k in range(N * N)]
    return [(u, v) for u, v in order if wt[u, v] != 0], wt


def run_reference(args):
    """CPU arm: the C/OpenMP port of the reference's per-view RL step (the MATLAB original
    cannot run here) on all host cores.  One step = one full RL view step (forward
    projection, ratio, back projection, D, update) of the workload's own image, over the
    active views in spiral order; `ms_per_step` is that view step's time.  `value` is the
    solve throughput it implies (a solve is views x iterations view steps plus the filter,
    whose cost is below 1 %), stated with the extrapolation in `extrapolated_solve`."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from mesolf_gb300 import synth
    w = synth.config2()
    H, Ht = w.psf()
    lf = workload_image(w, H).astype(np.float64)
    views, _ = active_views(H)
    n_views = len(views)
    for _ in range(args.warmup):
        cpu_baseline_sample(H, Ht, lf, planes=2)
    ts = []
    for k in range(args.steps):
        u, v = views[k % n_views]
        t, thr, planes = cpu_baseline_sample(H, Ht, lf, u=u, v=v)
        ts.append(t)
    t_view = float(np.mean(ts))
    t_solve = t_view * n_views * w.iters
    val = w.voxels / t_solve
    sample = (f"{args.steps} RL view steps (forward, ratio, back projection, D, update; views in spiral order) of "
              f"the full {w.image_shape[0]}x{w.image_shape[1]}x{w.Z} workload, FP64 C/OpenMP port of the oracle, "
              f"{thr} threads, {t_view:.2f} s per view step; value = one solve's voxels / ({n_views} views x "
              f"{w.iters} iterations x that time)")
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "voxels/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_view * 1e3,
            "step": "one RL view step", "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator, see mesolf_gb300/synth.py)",
            "config": workload_config(ws, n_views),
            "extrapolated_solve": {"view_steps_per_solve": n_views * w.iters, "ms_per_solve": t_solve * 1e3,
                                   "voxels_per_solve": int(w.voxels),
                                   "note": "value = voxels_per_solve / ms_per_solve; not timed as a whole"},
            "cpu_baseline": {"value": val, "unit": "voxels/s", "cores": thr, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="one solve of --iters iterations and exit (for ncu captures)")
    ap.add_argument("--iters", type=int, default=None)
    ap.add_argument("--planes", type=int, default=None,
                    help="with --profile: the deepest PLANES planes of the workload only (a smaller "
                         "device footprint for full ncu captures; same lateral size and kernel widths)")
    ap.add_argument("--mixed", default="bf16x2", help="tensor-core precision timed beside plain FP32 ('' to skip)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="seconds of each leg of the 36-patch 18 Hz serving stream (0 to skip)")
    ap.add_argument("--batched-steps", type=int, default=1,
                    help="timed steps of the 64-patch batched workload (0 to skip)")
    ap.add_argument("--only", choices=["summary", "rectify", "mex"], default=None,
                    help="run only that block (summary image / frame rectification on --frames frames; the "
                         "direct MEX projector on --frames slices of the fixture shape), 2 timed calls, no CPU "
                         "or host leg, and exit (for ncu captures)")
    ap.add_argument("--frames", type=int, default=2000)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        import torch
        import __graft_entry__
        __graft_entry__.build()
        dev0 = torch.device("cuda", 0)
        if args.only == "summary":
            blk = summary_block(dev0, T=args.frames, steps=2, cpu=False, e2e=False)
        elif args.only == "mex":
            blk = mex_direct_block(dev0, n=args.frames)
        else:
            blk = rectify_block(dev0, T=args.frames, steps=2, cpu=False, e2e=False)
        print(json.dumps({"only": args.only, "block": blk}), flush=True)
        return

    import torch
    import __graft_entry__
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    __graft_entry__.build()
    from mesolf_gb300 import PhaseSpacePSF, RLSolver, _lib
    from mesolf_gb300.api import _fortran

    w, H, Ht, lf = make_workload(dev, rank, args.planes if args.profile else None)
    torch.cuda.empty_cache()
    Xr, Xc = w.image_shape
    Z = w.Z
    psf = PhaseSpacePSF(H, Ht)
    solver = RLSolver(psf, (Xr, Xc))
    lf_dev = _fortran(torch.as_tensor(np.ascontiguousarray(lf)).to(dev))[0]
    out_dev = torch.empty((Z, Xc, Xr), dtype=torch.float32, device=dev).permute(2, 1, 0)
    if args.profile:
        torch.cuda.synchronize()
        solver.run(lf_dev, args.iters or w.iters, precision=args.precision, out=out_dev, want_stats=True)
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": solver.last_stats}), flush=True)
        return

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        solver.run(lf_dev, w.iters, precision=args.precision, out=out_dev, want_stats=False)
    barrier()
    clk = ClockSampler(local)
    clk.start()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        solver.run(lf_dev, w.iters, precision=args.precision, out=out_dev, want_stats=False)
    e1.record(stream)
    barrier()
    clocks = clk.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, ws, dev)
    # the per-launch kernel times (CUDA events around each view launch), the launch count and
    # the convergence monitor from one more, instrumented solve after the timed region: the
    # timed solves run as in production, without per-launch events or the FP64 monitor
    solver.run(lf_dev, w.iters, precision=args.precision, out=out_dev, want_stats=True)
    st = solver.last_stats
    launches = st["kernel_launches"] * args.steps
    vk_ms = st["view_kernel_ms"] * args.steps
    vk_n = st["view_kernel_launches"] * args.steps
    n_views = st["n_views"]
    value = replica_value(w.voxels, ws, ms)

    # mixed precision (tensor cores) on the same workload, error vs the plain FP32 volume
    mixed = None
    if args.mixed:
        ref_vol = out_dev.clone()
        mix_out = torch.empty_like(out_dev)
        for _ in range(max(1, args.warmup)):
            solver.run(lf_dev, w.iters, precision=args.mixed, out=mix_out, want_stats=False)
        barrier()
        m0 = torch.cuda.Event(enable_timing=True)
        m1 = torch.cuda.Event(enable_timing=True)
        mk_ms = 0.0
        mk_n = 0
        mlaunch = 0
        # throughput from graphs without timing-event nodes; the kernel times of the roofline
        # from one more solve of the instrumented graph, after the timed region
        m0.record(stream)
        for _ in range(args.steps):
            solver.run(lf_dev, w.iters, precision=args.mixed, out=mix_out, want_stats=False)
        m1.record(stream)
        barrier()
        mms = max_over_ranks(m0.elapsed_time(m1) / args.steps, ws, dev)
        solver.run(lf_dev, w.iters, precision=args.mixed, out=mix_out, want_stats=True)
        st2 = solver.last_stats
        mk_ms = st2["view_kernel_ms"] * args.steps
        mk_n = st2["view_kernel_launches"] * args.steps
        mlaunch = st2["kernel_launches"] * args.steps
        d = (mix_out.double() - ref_vol.double()).norm() / ref_vol.double().norm()
        mflop = algorithmic_flop_per_view(Xr, Xc, Z, psf.S, psf.N) * n_views * w.iters * args.steps
        mixed = {"precision": args.mixed, "value": replica_value(w.voxels, ws, mms), "unit": "voxels/s",
                 "ms_per_step": mms, "speedup_vs_plain_fp32": ms / mms,
                 "rel_l2_vs_plain_fp32": float(d),
                 "rel_change_last_iteration": st2.get("rel_change"),
                 "gpu_launches": int(mlaunch),
                 "launch_config": {k: st2[k] for k in ("fwd_splits", "fwd_stages", "bwd_xbufs", "tuned")},
                 "view_kernels_ms_per_view": mk_ms / max(1, mk_n),
                 "roofline": {"bound": "tensor", "achieved": mflop / (mk_ms * 1e-3) / 1e12,
                              "traffic": KTC_DRAM_BYTES if (Xr, Xc, Z) == (1005, 1005, 51) else None,
                              "peak": _measured_bf16(), "unit": "TFLOP/s",
                              "frac": (mflop / (mk_ms * 1e-3) / 1e12) / _measured_bf16() if _measured_bf16() else None,
                              "note": "algorithmic flop of the projections / time of the view-step GEMM kernels "
                                      "(fused back projection + update + next-view forward, k_tc_bwdfwd); "
                                      "peak = measured bf16 burst"}}

    # e2e: pinned host image in, pinned host volume out, through mlf_solver_run
    lf_host = torch.empty((Xc, Xr), dtype=torch.float32, pin_memory=True).t()
    lf_host.copy_(torch.as_tensor(np.ascontiguousarray(lf)))
    out_host = torch.empty((Z, Xc, Xr), dtype=torch.float32, pin_memory=True).permute(2, 1, 0)
    solver.run(lf_host, w.iters, precision=args.precision, out=out_host, want_stats=False)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solver.run(lf_host, w.iters, precision=args.precision, out=out_host, want_stats=False)
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, ws, dev)
    e2e = {"value": replica_value(w.voxels, ws, e2e_ms), "unit": "voxels/s",
           "h2d_bytes_per_step": int(Xr * Xc * 4), "d2h_bytes_per_step": int(Xr * Xc * Z * 4),
           "ms_per_step": e2e_ms, "path": "mlf_solver_run, pinned host buffers"}

    # roofline of the dominant kernel (the per-view projector/update kernel)
    peak = ctypes_peak = None
    import ctypes
    pk = ctypes.c_double()
    if _lib.load().mlf_probe_fp32_peak(200.0, ctypes.byref(pk), ctypes.c_void_p(stream.cuda_stream)) == 0:
        ctypes_peak = pk.value
    peak = ctypes_peak
    flop_view = algorithmic_flop_per_view(Xr, Xc, Z, psf.S, psf.N)
    mean_launch_ms = vk_ms / max(1, vk_n)
    # the launches of one iteration do n_views views' worth of work in n_views + 1 launches
    achieved = flop_view * n_views * w.iters * args.steps / (vk_ms * 1e-3) / 1e12
    # dram__bytes_read.sum + dram__bytes_write.sum of one fused view launch at this workload
    # (ncu capture on GB300); algorithmic bytes per view are 8 B per voxel = 412 MB
    traffic = KVIEW_DRAM_BYTES if (Xr, Xc, Z) == (1005, 1005, 51) else None
    roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if peak else None, "traffic": traffic,
                "kernel": "k_view (fused back projection + update + next forward projection)",
                "flop_per_view": flop_view, "mean_launch_ms": mean_launch_ms,
                "peak_source": "measured live: mlf_probe_fp32_peak (register-only FP32 FMA kernel)",
                "hbm_peak_gbs_measured": _measured_hbm()}

    line = {"metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, see mesolf_gb300/synth.py)",
            "config": workload_config(ws, n_views), "precision": args.precision,
            "l2": "inputs larger than L2 (projector taps 4.6 GB, volume 206 MB)",
            "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline, "clocks": clocks,
            "impl": "ours", "mixed": mixed,
            "convergence": {"rel_change_last_iteration": st.get("rel_change"),
                            "note": "||X_k - X_(k-1)|| / ||X_k|| of the last RL iteration, FP64 on the device"}}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        t, thr, planes = cpu_baseline_sample(H, Ht, lf.astype(np.float64))
        t_solve = t * n_views * w.iters
        line["cpu_baseline"] = {"value": w.voxels / t_solve, "unit": "voxels/s", "cores": thr, "kind": "port",
                                "sample": f"one full RL view step ({Xr}x{Xc}x{planes}) of the FP64 C/OpenMP oracle "
                                          f"port on {thr} host threads ({t:.2f} s), extrapolated to "
                                          f"{n_views} views x {w.iters} iterations"}
        tc_s, E = cpu_fft_sample(Xr, Xc, psf.S)
        t_fft = tc_s * 3 * Z * n_views * w.iters
        line["cpu_baseline"]["fft_variant"] = {
            "value": w.voxels / t_fft, "unit": "voxels/s", "cores": 1, "kind": "port",
            "sample": f"3 conv2FFT calls ({Xr}x{Xc} image, {psf.S}x{psf.S} kernel, {E[0]}x{E[1]} grid, FP64 "
                      f"numpy, {tc_s:.3f} s each), extrapolated to 3 x {Z} calls per view x {n_views} views x "
                      f"{w.iters} iterations"}
    # the single-GPU extras (error table, MEX projector, serving stream, batched workload) run
    # at N = 1 only
    if ws == 1:
        progress("main solve, mixed, e2e, CPU baseline")
        line["config1"] = config1_block(dev, cpu=not args.no_cpu_baseline)
        progress("config1")
        line["fft_formulation"] = fft_formulation_block(H, Ht, lf, psf, dev)
        progress("fft_formulation")
        line["mex_projector"] = mex_block(dev, peak)
        progress("mex_projector")
        line["seed_library"] = seed_block(Ht, dev)
        progress("seed_library")
        line["summary_image"] = summary_block(dev, cpu=not args.no_cpu_baseline)
        progress("summary_image")
        line["rectification"] = rectify_block(dev, cpu=not args.no_cpu_baseline)
        progress("rectification")
        solver.close()
        torch.cuda.empty_cache()
        line["precision_vs_fp64_oracle"] = precision_block(psf, dev)
        progress("precision_vs_fp64_oracle")
    if ws == 1 and args.serve_seconds > 0 and args.mixed:
        solver.close()
        del out_dev, lf_dev
        torch.cuda.empty_cache()
        line["serving"] = serve_block(psf, args.serve_seconds, args.mixed, dev)
        progress("serving")
    if ws == 1 and args.batched_steps > 0 and args.mixed:
        solver.close()
        psf.close()
        torch.cuda.empty_cache()
        line["batched"] = batched_block(args.mixed, dev, steps=args.batched_steps)
        progress("batched")
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()
    psf.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


SERVE_DESC = ("6x6 patch carpet (36 patches, 45-71 lenslets per side, 51 planes, the same PSF), frames at "
              "18 Hz +-10% jitter for 60 s, AR(1) (rho 0.95) soma intensities, 2000-photon Poisson images, warm "
              "start from the previous frame, 3 RL iterations")


def serve_block(psf, seconds, precision, dev, pool=12, rate_hz=18.0, paced_frac=0.8):
    """The serving stream through SolveServer (two lanes, each with a work set sized once for
    the whole carpet; continuous batching; warm start).  Two legs of `seconds` each:

    * `stream_18hz`: frames of the carpet arrive at 18 Hz +-10 % jitter.  One GB300 serves
      far fewer carpet frames per second than that (the HBM bound below), so the server runs
      with the latest-frame policy (a patch with several frames waiting takes the newest; the
      older ones are dropped and counted) and the latency of the served frames stays bounded.
    * `paced`: the same stream at `paced_frac` of the rate the first leg sustained, nothing
      dropped: the steady-state latency (and its first / second half, to show it is flat).

    Latency = scheduled arrival -> volume in pinned host memory.  Frames cycle through a
    pool of `pool` distinct frames of the AR(1) soma stream (rendering and projecting 1080
    distinct carpet frames would take longer than the stream).  The plain FP32 drop-in rate
    is taken on the carpet's own 36 patches (one cold 3-iteration solve each), and the mixed
    results' error against it on the same cold solves."""
    import torch
    from mesolf_gb300 import BatchSolver, RLSolver, synth
    from mesolf_gb300.api import _fortran
    from mesolf_gb300.serve import SolveServer
    N, Z = psf.N, psf.Z
    shapes = synth.carpet_geometry()
    P = len(shapes)
    geo = [(sh, (0, Z)) for sh in shapes]
    density = 2000.0 / (1005 * 1005 * 51)
    streams = [synth.SomaStream(sh, Z, int(round(density * sh[0] * sh[1] * Z)), seed=100 + k, device=dev)
               for k, sh in enumerate(shapes)]
    gen = BatchSolver(psf, shapes)
    rng = torch.Generator(device=dev)
    rng.manual_seed(11)
    frames, scale = [], None
    t_gen = time.perf_counter()
    for f in range(pool):
        vols = [st.step() for st in streams]
        lfs = gen.forward_project(vols, raw_psf=True, precision="bf16x3")
        if scale is None:
            scale = [2000.0 / float(lf.max()) for lf in lfs]
        frames.append([torch.poisson((lf.clamp(min=0) * sc).contiguous(), generator=rng).cpu().numpy()
                       for lf, sc in zip(lfs, scale)])
        del vols, lfs
    gen.close()
    del streams
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t_gen
    torch.cuda.empty_cache()
    frame_vox = sum(a * b * Z for a, b in shapes)
    srv = SolveServer(psf, geo, iters=3, precision=precision, lanes=2, drop_stale=True)
    # frame 0 warms the server up (autotuning, graph captures, cold-started volumes); not timed
    for p in range(P):
        srv.submit(p, 0, frames[0][p])
    srv.drain()
    srv.reset_stats()
    fno = [1]

    def stream(period_s, jitter, seconds_):
        rng_j = np.random.default_rng(3 + fno[0])
        t0 = time.perf_counter() + 0.01
        t_next, n = t0, 0
        while t_next < t0 + seconds_:
            while time.perf_counter() < t_next:
                time.sleep(max(0.0, min(0.002, t_next - time.perf_counter())))
            fr = frames[fno[0] % pool]
            for p in range(P):
                # the futures are not kept: a served volume is freed once its lane is done with it
                srv.submit(p, fno[0], fr[p], t_arrival=t_next)
            fno[0] += 1
            n += 1
            t_next += period_s * (1.0 + (rng_j.uniform(-jitter, jitter) if jitter else 0.0))
        srv.drain()
        return n

    n_over = stream(1.0 / rate_hz, 0.1, seconds)
    rep = srv.report()
    sustained = rep["voxels_per_s"] / frame_vox
    srv.reset_stats()
    slow_period = 1.0 / (paced_frac * sustained)
    n_paced = stream(slow_period, 0.0, seconds)
    rep_slow = srv.report()
    # latencies of the paced leg in completion order: first and second half
    srv_lat = np.array(srv.latencies_ms())
    half = len(srv_lat) // 2
    lat_first, lat_second = srv_lat[:half], srv_lat[half:]
    srv.close()
    torch.cuda.empty_cache()
    # plain FP32 drop-in on the carpet's own patches, and the mixed results' error against it
    fp32_t, errs = 0.0, []
    mixed = BatchSolver(psf, shapes)
    imgs = [_fortran(torch.as_tensor(np.ascontiguousarray(frames[1][p])).to(dev))[0] for p in range(P)]
    mix = mixed.run(imgs, 3, precision=precision, want_stats=False)
    torch.cuda.synchronize()
    for p in range(P):
        s = RLSolver(psf, shapes[p])
        s.run(imgs[p], 1, precision="fp32", want_stats=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = s.run(imgs[p], 3, precision="fp32", want_stats=False)
        torch.cuda.synchronize()
        fp32_t += time.perf_counter() - t0
        errs.append(float((mix[p].double() - out.double()).norm() / out.double().norm()))
        s.close()
        del out
    mixed.close()
    fp32_rate = frame_vox / fp32_t
    return {"workload": "carpet6x6_lenslets45-71_z51_k231_it3_18hz", "desc": SERVE_DESC,
            "precision": precision, "seconds_per_leg": seconds, "frame_pool": pool,
            "voxels_per_frame": frame_vox, "frame_period_ms": 1000.0 / rate_hz,
            "stream_18hz": {"frames_offered": n_over, "requests_served": rep["requests"],
                            "requests_dropped": rep["dropped"], "p50_ms": rep["p50_ms"], "p99_ms": rep["p99_ms"],
                            "max_ms": rep["max_ms"], "voxels_per_s": rep["voxels_per_s"],
                            "frames_per_s_sustained": sustained, "batches": rep["batches"],
                            "mean_batch_patches": rep["mean_batch"], "lanes": rep["lanes"],
                            "policy": "latest frame per patch (older waiting frames dropped)"},
            "paced": {"frame_period_ms": 1e3 * slow_period, "fraction_of_sustained": paced_frac,
                      "frames_offered": n_paced, "requests_served": rep_slow["requests"],
                      "requests_dropped": rep_slow["dropped"], "p50_ms": rep_slow["p50_ms"],
                      "p99_ms": rep_slow["p99_ms"], "max_ms": rep_slow["max_ms"],
                      "voxels_per_s": rep_slow["voxels_per_s"],
                      "p50_ms_first_half": float(np.percentile(lat_first, 50)) if lat_first.size else None,
                      "p50_ms_second_half": float(np.percentile(lat_second, 50)) if lat_second.size else None},
            "voxels_per_s": rep["voxels_per_s"], "p50_ms": rep["p50_ms"], "p99_ms": rep["p99_ms"],
            "plain_fp32_voxels_per_s": fp32_rate, "speedup_vs_plain_fp32": rep["voxels_per_s"] / fp32_rate,
            "plain_fp32_ms_per_frame": 1e3 * frame_vox / fp32_rate,
            "plain_fp32_sample": "one cold 3-iteration FP32 solve of each of the 36 carpet patches",
            "rel_l2_vs_plain_fp32_cold_solve": {"max": max(errs), "median": float(np.median(errs))},
            "frame_generation_s": t_gen,
            "note": "the carpet needs >= 8 B per voxel per view step of HBM traffic: one frame of 3 iterations "
                    "moves >= 4.6 TB, so 18 Hz is out of reach on one GPU and the 18 Hz leg is overloaded by "
                    "design; the paced leg shows the latency under a load the server keeps up with"}


BATCH_DESC = ("64 independent patches, Nnum 15, lenslets per side uniform in [31, 71], planes uniform in "
              "[26, 101] of one 101-plane PSF (plane k window 31+4k capped at 255, K0 255), soma density 5e-4 "
              "per voxel, 2000-photon Poisson images, 5 RL iterations, one persistent launch per view step for "
              "all patches under a captured CUDA graph per iteration")


def batched_block(precision, dev, steps=1, warmup=1, n_patches=64):
    """The batched uneven-patch workload: all patches in one work set, each RL iteration one
    CUDA graph.  Deconvolved voxels/s with the images resident in HBM."""
    import torch
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF, synth
    t0 = time.perf_counter()
    z_idx = np.arange(101)
    sides = np.minimum(31 + 4 * z_idx, 255)
    H, Ht = synth.make_psf(int(sides.max()), 15, z_idx, seed=4, plane_sides=sides)
    psf = PhaseSpacePSF(H, Ht)
    shapes, planes = synth.uneven_batch_geometry(n=n_patches)
    b = BatchSolver(psf, shapes, planes)
    vols = []
    for k, (sh, (z0, nz)) in enumerate(zip(shapes, planes)):
        st = synth.SomaStream(sh, nz, int(round(5e-4 * sh[0] * sh[1] * nz)), seed=200 + k, device=dev)
        vols.append(st.step())
    lf_clean = b.forward_project(vols, raw_psf=True, precision="bf16x3")
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    imgs = []
    for lf in lf_clean:
        sc = 2000.0 / float(lf.max())
        x = torch.poisson((lf.clamp(min=0) * sc).contiguous(), generator=g)
        imgs.append(x.t().contiguous().t())          # column-major (Xr, Xc)
    del vols, lf_clean
    t_setup = time.perf_counter() - t0
    voxels = sum(a * c * nz for (a, c), (_, nz) in zip(shapes, planes))
    outs = None
    for _ in range(warmup):
        outs = b.run(imgs, 5, precision=precision, outs=outs, want_stats=False)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream()
    e0.record(stream)
    for _ in range(steps):
        outs = b.run(imgs, 5, precision=precision, outs=outs, want_stats=False)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # kernel times and launch counts from one instrumented solve after the timed region
    outs = b.run(imgs, 5, precision=precision, outs=outs, want_stats=True)
    launches = b.last_stats["kernel_launches"] * steps
    vk_ms = b.last_stats["view_kernel_ms"] * steps
    vk_n = b.last_stats["view_kernel_launches"] * steps
    finite = all(bool(torch.isfinite(o).all()) for o in outs)
    # the plain FP32 drop-in on two of the patches (PSF cut to each patch's planes), and the
    # batched results' error against it
    from mesolf_gb300 import RLSolver
    fp32_t, fp32_vox, errs = 0.0, 0, []
    for k in range(2):
        (xr, xc), (z0, nz) = shapes[k], planes[k]
        sub = PhaseSpacePSF(np.asfortranarray(H[:, :, :, :, z0:z0 + nz]), np.asfortranarray(Ht[:, :, :, :, z0:z0 + nz]))
        s1 = RLSolver(sub, (xr, xc))
        o = s1.run(imgs[k], 5, precision="fp32", want_stats=False)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        o = s1.run(imgs[k], 5, precision="fp32", want_stats=False)
        torch.cuda.synchronize()
        fp32_t += time.perf_counter() - t1
        fp32_vox += xr * xc * nz
        errs.append(float((outs[k].double() - o.double()).norm() / o.double().norm()))
        s1.close()
        sub.close()
    del H, Ht
    fp32_rate = fp32_vox / fp32_t
    res = {"workload": "batch64_lenslets31-71_z26-101_k255_it5", "desc": BATCH_DESC, "precision": precision,
           "patches": n_patches, "voxels": int(voxels), "value": voxels / (ms * 1e-3), "unit": "voxels/s",
           "ms_per_step": ms, "steps": steps, "warmup": warmup, "views_per_iteration": b.last_stats["n_views"],
           "gpu_launches": int(launches), "view_kernels_ms_per_view": vk_ms / max(1, vk_n),
           "device_bytes_work_set": b.device_bytes, "all_finite": finite, "setup_s": t_setup,
           "plain_fp32_voxels_per_s": fp32_rate, "speedup_vs_plain_fp32": voxels / (ms * 1e-3) / fp32_rate,
           "rel_l2_vs_plain_fp32": errs,
           "plain_fp32_sample": "single FP32 solves (5 iterations) of patches 0 and 1 with the PSF cut to their planes"}
    b.close()
    psf.close()
    return res


GOLDEN_C1 = os.path.join(ROOT, "tests", "golden", "lf165x165x21_k61.npz")
CONFIG1_DESC = ("Nnum 15, 11x11 lenslets (165x165 px), 21 planes (-40..40 um at 4 um), PSF 61 px (phase-space 45), "
                "40 spheres, 1000-photon Poisson image, 8 RL iterations")


def config1_block(dev, steps=10, warmup=3, cpu=True):
    """The plain CPU-runnable workload (165 x 165 x 21, 8 iterations), timed whole on both
    sides with nothing extrapolated: the FP32 drop-in and the bf16x2 tensor-core solve on the
    GPU (image in HBM, CUDA events; and end to end from pinned host memory), and the whole
    FP64 oracle solve on the host cores (normalisation, realignment, weights, filter bank,
    8 iterations of C/OpenMP view steps and numpy sample_filter).  Errors against the
    oracle's committed 8-iteration volume."""
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver, synth
    from mesolf_gb300.api import _fortran
    w = synth.config1()
    H, Ht = w.psf()
    g = dict(np.load(GOLDEN_C1))
    lf = g["lf"]
    ref = g["x8"].astype(np.float64)
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, lf.shape)
    lf_dev = _fortran(torch.as_tensor(np.ascontiguousarray(lf)).to(dev))[0]
    out = torch.empty((w.Z, lf.shape[1], lf.shape[0]), dtype=torch.float32, device=dev).permute(2, 1, 0)
    stream = torch.cuda.current_stream()
    res = {"workload": "lf165x165x21_k61_it8", "desc": CONFIG1_DESC, "voxels": int(w.voxels), "iterations": 8}
    for prec in ("fp32", "bf16x2"):
        for _ in range(warmup):
            s.run(lf_dev, 8, precision=prec, out=out, want_stats=False)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            s.run(lf_dev, 8, precision=prec, out=out, want_stats=False)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        got = out.cpu().numpy().astype(np.float64)
        res[prec] = {"value": w.voxels / (ms * 1e-3), "unit": "voxels/s", "ms_per_solve": ms, "steps": steps,
                     "rel_l2_vs_fp64_oracle": float(np.linalg.norm(got - ref) / np.linalg.norm(ref))}
    lf_host = torch.empty((lf.shape[1], lf.shape[0]), dtype=torch.float32, pin_memory=True).t()
    lf_host.copy_(torch.as_tensor(np.ascontiguousarray(lf)))
    out_host = torch.empty((w.Z, lf.shape[1], lf.shape[0]), dtype=torch.float32, pin_memory=True).permute(2, 1, 0)
    s.run(lf_host, 8, precision="fp32", out=out_host, want_stats=False)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.run(lf_host, 8, precision="fp32", out=out_host, want_stats=False)
    t_e2e = (time.perf_counter() - t0) / steps
    res["fp32"]["e2e"] = {"value": w.voxels / t_e2e, "unit": "voxels/s", "ms_per_solve": t_e2e * 1e3,
                          "h2d_bytes_per_step": int(lf.size * 4), "d2h_bytes_per_step": int(w.voxels * 4),
                          "path": "mlf_solver_run, pinned host buffers"}
    s.close()
    psf.close()
    if cpu:
        from oracle import cbuild
        from oracle import mesolf_ref as R
        t0 = time.perf_counter()
        X = R.recon_phase_space(lf.astype(np.float64), H, Ht, 8, view_step=cbuild.view_step)
        t_cpu = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": w.voxels / t_cpu, "unit": "voxels/s", "s_per_solve": t_cpu,
                               "cores": cbuild.threads(), "kind": "port",
                               "sample": "the whole 8-iteration solve, timed once, not extrapolated: FP64 C/OpenMP "
                                         "view steps on all host threads, the rest FP64 numpy",
                               "rel_l2_vs_committed_oracle_volume": float(np.linalg.norm(X - ref) /
                                                                          np.linalg.norm(ref))}
        res["speedup_fp32_vs_cpu"] = res["fp32"]["value"] / res["cpu_baseline"]["value"]
        res["e2e_speedup_fp32_vs_cpu"] = res["fp32"]["e2e"]["value"] / res["cpu_baseline"]["value"]
    return res


GOLDEN_C2 = os.path.join(ROOT, "tests", "golden", "lf1005x1005x51_k231.npz")


def precision_block(psf, dev):
    """Error of every precision against the FP64 oracle of the 1005 x 1005 x 51 workload
    (fixture: the oracle's volume on a fixed sample of 131072 voxels after 3 and 10
    iterations, and the measured image it was computed from)."""
    if not os.path.exists(GOLDEN_C2):
        return {"available": False, "why": "oracle fixture not generated"}
    import torch
    from mesolf_gb300 import RLSolver
    from mesolf_gb300.api import _fortran
    g = dict(np.load(GOLDEN_C2))
    s = RLSolver(psf, g["lf"].shape)
    lf = _fortran(torch.as_tensor(g["lf"].astype(np.float32)).to(dev))[0]
    rows = []
    stream = torch.cuda.current_stream()
    for prec in ("fp32", "bf16x3", "fp16x3", "bf16x2", "fp16x2", "bf16", "fp16"):
        for it in (3, 10):
            if f"x{it}" not in g:
                continue
            vol = s.run(lf, it, precision=prec, want_stats=False)
            row = {"precision": prec, "iterations": it}
            if it == 3:
                # device time of this solve (image in HBM), 3 timed solves after this one
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(3):
                    s.run(lf, it, precision=prec, out=vol, want_stats=False)
                e1.record(stream)
                torch.cuda.synchronize()
                row["ms_per_solve"] = e0.elapsed_time(e1) / 3
            vol = vol.cpu().numpy()
            ref = g[f"x{it}"].astype(np.float64)
            got = vol.astype(np.float64).reshape(-1, order="F")[g["idx"]]
            row.update({"rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                        "max_abs": float(np.abs(got - ref).max()), "ref_max": float(np.abs(ref).max())})
            rows.append(row)
    s.close()
    return {"available": True, "sample_voxels": int(g["idx"].size), "vs": "FP64 oracle", "rows": rows}


def fft_formulation_block(H, Ht, lf, psf, dev, steps=5):
    """The reference's GPU-branch formulation of one RL view step (recon_..._with_filter.m:
    109-137 with conv2FFT.m:1-22 on the exsize grid) on this GPU with cuFFT (torch.fft) and
    the PSF spectra of the view precomputed (the reference recomputes them every call):
    forward = Z R2C transforms of the volume planes, the spectral product summed over z, one
    C2R; back projection = one R2C of the sparse ratio image, Z C2R for C and Z for D
    (= bwd(ones), recomputed per view as the reference does).  A comparison measurement, not a
    product path: the FP32 time per view, the bytes its transforms and spectra move, and the
    error of its updated volume against the FP32 direct view step (mlf_rl_view_step) from the
    same start -- in FP32 and, as a check of the formulation, in FP64, over all voxels and
    over those where D is not round-off -- for the active view nearest the centre and for the
    view of largest weight (a corner view, where D is exactly 0 near the image edge).
    Spectra of all views would need 2 x 225 x Z x E x (E/2+1) x 8 B of HBM."""
    import torch
    from mesolf_gb300 import RLSolver
    from mesolf_gb300.api import _fortran
    from oracle import mesolf_ref as R
    N = psf.N
    Xr, Xc = lf.shape
    Z = H.shape[4]
    S = psf.S
    E = R.ex_size((Xr, Xc), S)
    m = S // 2
    c0 = (N + 1) // 2 - 1
    lf64 = torch.as_tensor(np.ascontiguousarray(lf), dtype=torch.float64, device=dev)
    X0 = torch.full((Z, Xr, Xc), float(lf.sum()) / (lf.size * Z), dtype=torch.float64, device=dev)
    X0 *= 1.0 + 0.1 * torch.rand(X0.shape, generator=torch.Generator(device=dev).manual_seed(3), device=dev,
                                 dtype=torch.float64)
    X0 = X0.float().double()                         # the same start, representable in FP32
    s = RLSolver(psf, (Xr, Xc))
    lf_d = _fortran(torch.as_tensor(np.ascontiguousarray(lf), dtype=torch.float32).to(dev))[0]

    def view_case(u, v, timed):
        h, t = R.phasespace_view(H, Ht, u, v)
        w_uv = float(psf.weights[u, v])
        kp = np.zeros((2, Z) + E)
        kp[0, :, :S, :S] = np.moveaxis(h, 2, 0)
        kp[1, :, :S, :S] = np.moveaxis(t, 2, 0)
        kp = np.roll(kp, (-m, -m), axis=(2, 3))     # conv2FFT's circular re-centring
        res = {"view": [u, v], "weight": w_uv}
        ref = s.view_step(lf_d, _fortran(X0.float().permute(1, 2, 0).contiguous())[0], u, v, w_uv)
        ref = ref.permute(2, 0, 1).double()
        for dt, name in ((torch.float32, "fp32"), (torch.float64, "fp64")):
            spec = torch.fft.rfft2(torch.as_tensor(kp, dtype=dt, device=dev))
            Hs, Ts = spec[0], spec[1]
            Xp = torch.zeros((Z,) + E, dtype=dt, device=dev)
            Bp = torch.zeros(E, dtype=dt, device=dev)
            Op = torch.zeros(E, dtype=dt, device=dev)
            Op[u:Xr:N, v:Xc:N] = 1.0
            ones_s = torch.fft.rfft2(Op)
            X = X0.to(dt)
            lft = lf64.to(dt)

            def step():
                Xp[:, :Xr, :Xc] = X
                P = torch.fft.irfft2((torch.fft.rfft2(Xp) * Hs).sum(0), s=E)[:Xr, :Xc]
                Rr = lft[u::N, v::N] / P[c0::N, c0::N]
                Rr = torch.where(torch.isfinite(Rr), Rr, torch.zeros_like(Rr))
                Bp.zero_()
                Bp[u:Xr:N, v:Xc:N] = Rr
                C = torch.fft.irfft2(torch.fft.rfft2(Bp) * Ts, s=E)[:, :Xr, :Xc]
                D = torch.fft.irfft2(ones_s * Ts, s=E)[:, :Xr, :Xc]
                Xn = X * C / D
                Xn = torch.where(torch.isfinite(Xn) & (Xn >= 0), Xn, torch.zeros_like(Xn))
                return torch.clamp(w_uv * Xn + (1 - w_uv) * X, min=0), D

            out, D = step()
            if name == "fp64":
                # where the exact D is 0 (no sampled lenslet's kernel reaches the voxel) the
                # transforms leave round-off of ~1e-16 of the peak, and C/D is a ratio of two
                # round-off values; the direct form has exact zeros there (0/0 -> 0)
                keep = D.abs() > 1e-9 * float(D.abs().max())
                res["voxels_with_D_roundoff_only"] = float(1.0 - keep.double().mean())
            if timed and name == "fp32":
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(steps):
                    out, D = step()
                e1.record()
                torch.cuda.synchronize()
                res["ms_per_view_fp32"] = e0.elapsed_time(e1) / steps
            res[f"rel_l2_{name}_vs_fp32_direct"] = float((out.double() - ref).norm() / ref.norm())
            if name == "fp64":
                for nm, o in (("fp64", out.double()), ("fp32", out32.double())):
                    d = torch.where(keep, o - ref, torch.zeros_like(ref))
                    r = torch.where(keep, ref, torch.zeros_like(ref))
                    res[f"rel_l2_{nm}_vs_fp32_direct_where_D_nonzero"] = float(d.norm() / r.norm())
            else:
                out32 = out
            del spec, Hs, Ts, Xp, out, D
            torch.cuda.empty_cache()
        return res

    W = psf.weights
    h0 = (N - 1) // 2
    act = [(abs(a - h0) + abs(b - h0), a, b) for a in range(N) for b in range(N) if W[a, b] != 0]
    _, ua, va = min(act)                             # the active view nearest the centre
    cases = [view_case(ua, va, True)]
    uc, vc = (int(k) for k in np.unravel_index(int(np.argmax(W)), W.shape))
    if (uc, vc) != (ua, va):
        cases.append(view_case(uc, vc, False))
    s.close()
    spec_bytes = 2 * Z * E[0] * (E[1] // 2 + 1) * 8
    ntrans = 3 * Z + 2
    trans_bytes = ntrans * E[0] * (E[1] // 2 + 1) * 8 * 2
    return {"exsize": list(E), "views": cases, "transforms_per_view": ntrans,
            "spectra_bytes_per_view": spec_bytes, "transform_bytes_per_view_min": trans_bytes,
            "hbm_bound_ms_per_view": (spec_bytes + trans_bytes + 8 * Xr * Xc * Z) / (_measured_hbm() or 6800) / 1e6,
            "spectra_bytes_all_views": 225 * spec_bytes,
            "note": "cuFFT (torch.fft) on this GPU, spectra of the view precomputed; comparison only"}


def mex_direct_block(dev, n=8, kw=241, steps=2):
    """The direct MEX kernel alone on n slices of the fixture shape (376 x 376, kw 241):
    time per call and TFLOP/s (algorithmic 2*W*H*n*kw^2); for ncu captures."""
    import torch
    from mesolf_gb300 import mex_lfm_convolution_vec
    W = Hh = 376
    g = torch.Generator(device=dev)
    g.manual_seed(9)
    bm = torch.rand((n, Hh, W), generator=g, device=dev).permute(2, 1, 0)
    K = torch.rand((15, 15, kw, kw), generator=g, device=dev).permute(3, 2, 1, 0)
    mex_lfm_convolution_vec(bm, K, method="direct")
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        mex_lfm_convolution_vec(bm, K, method="direct")
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"W": W, "H": Hh, "n": n, "kw": kw, "ms_per_call": ms, "tflops": 2.0 * W * Hh * n * kw * kw / ms / 1e9}


def mex_block(dev, fp32_peak, steps=2):
    """The MEX projector (mex_lfm_convolution_vec) on the reference's fixture shape: a
    376 x 376 x 77 single bitmap (vols_slice.mat) and 241 x 241 x 15 x 15 kernels (the demo's
    width), seeded random values (the fixture's PSF is not available).  Algorithmic flop
    2*W*H*n*kw^2 = 1.26 T per call.  The default call takes the tensor-core route; the direct
    CUDA-core kernel is timed beside it.  Checked against the FP64 oracle on sampled pixels."""
    import torch
    from mesolf_gb300 import mex_lfm_convolution_vec
    from oracle import mesolf_ref as R
    W, Hh, n, kw = 376, 376, 77, 241
    g = torch.Generator(device=dev)
    g.manual_seed(9)
    bm = torch.rand((n, Hh, W), generator=g, device=dev).permute(2, 1, 0)      # column-major W x H x n
    K = torch.rand((15, 15, kw, kw), generator=g, device=dev).permute(3, 2, 1, 0)
    out = mex_lfm_convolution_vec(bm, K)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream()
    e0.record(stream)
    for _ in range(steps):
        out = mex_lfm_convolution_vec(bm, K)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    flop = 2.0 * W * Hh * n * kw * kw
    e0.record(stream)
    direct = mex_lfm_convolution_vec(bm, K, method="direct")
    e1.record(stream)
    torch.cuda.synchronize()
    ms_direct = e0.elapsed_time(e1)
    d_rel = float((direct.double() - out.double()).norm() / direct.double().norm())
    rng = np.random.default_rng(1)
    pts = [(int(rng.integers(W)), int(rng.integers(Hh)), int(rng.integers(n))) for _ in range(64)]
    ref = R.lfm_conv_vec_points(bm.cpu().numpy(), K.cpu().numpy(), pts)
    got = np.array([float(out[x, y, i]) for x, y, i in pts])
    ach = flop / (ms * 1e-3) / 1e12
    bf16 = _measured_bf16()
    return {"workload": "mex376x376x77_kw241", "route": "tensor cores (forward-projection recast, bf16x3)",
            "ms_per_call": ms, "tflops_algorithmic": ach,
            "roofline": {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                         "frac": ach / bf16 if bf16 else None,
                         "frac_of_fp32_peak": ach / fp32_peak if fp32_peak else None,
                         "note": "algorithmic flop of the correlation / call time including the per-call PSF and "
                                 "batch set-up; peak = measured bf16 burst"},
            "direct_kernel_ms_per_call": ms_direct, "speedup_vs_direct": ms_direct / ms,
            "rel_l2_tensor_vs_direct": d_rel,
            "rel_l2_vs_fp64_oracle_64_pixels": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            "data": "seeded uniform bitmap and kernels of the fixture's shape"}


def seed_block(Ht, dev, n_seg=128, side=396, depth=9):
    """The seed library's "collect and forward-project" section on a synthetic segment set:
    n_seg segments of side x side pixels, each `depth` consecutive planes of the PSF, four
    kinds of slices (sample, mask, ring, ring mask), projected with Ht in one pass
    (seed_library_projections).  The reference makes 4 MEX calls per depth over the slices at
    that depth; its time is estimated from one direct MEX slice projection."""
    import torch
    from mesolf_gb300 import mex_lfm_convolution_vec, seed_library_projections
    Z = Ht.shape[4]
    rng = np.random.default_rng(21)
    ua, vols = [], [[] for _ in range(4)]
    for i in range(n_seg):
        z0 = int(rng.integers(0, Z - depth + 1))
        ua.append(list(range(z0 + 1, z0 + depth + 1)))
        base = rng.random((side, side, depth)).astype(np.float32)
        for k in range(4):
            vols[k].append(base if k % 2 == 0 else (base > 0.7).astype(np.float32))
    seed_library_projections(Ht, *vols, ua)      # warm (PSF set-up paths, allocations)
    t0 = time.perf_counter()
    out = seed_library_projections(Ht, *vols, ua)
    t_pass = time.perf_counter() - t0
    one = torch.as_tensor(vols[0][0][:, :, :1]).to(dev)
    Kz = torch.as_tensor(np.ascontiguousarray(Ht[:, :, :, :, 0])).to(dev)
    mex_lfm_convolution_vec(one, Kz, method="direct")
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    mex_lfm_convolution_vec(one, Kz, method="direct")
    torch.cuda.synchronize()
    t_slice = time.perf_counter() - t1
    n_proj = 4 * n_seg * depth
    kw = Ht.shape[0]
    return {"workload": f"seed_library_{n_seg}seg_{side}px_{depth}planes_kw{kw}", "segments": n_seg,
            "slice_projections": n_proj, "one_pass_s": t_pass,
            "per_depth_mex_loop_estimate_s": t_slice * n_proj,
            "speedup_vs_per_depth_loop": t_slice * n_proj / t_pass,
            "tflops_algorithmic": 2.0 * side * side * kw * kw * n_proj / t_pass / 1e12,
            "all_finite": bool(all(np.isfinite(o).all() for o in out)),
            "note": "host arrays in and out, as the reference gathers its accumulators; the loop estimate is the "
                    "direct MEX kernel's time for one slice times the number of slice projections"}


def summary_block(dev, side=1005, T=2000, steps=3, cpu=True, cpu_pixels=8192, e2e=True):
    """The step before the reconstruction: the summary image (LFIMG) of a side x side-pixel,
    T-frame sensor movie with the reference's default parameters (pixelwise detrend,
    bg_iter 5, windows 100 and 20 frames, poly_index 3), movie resident in HBM (`value`) and
    from pinned host memory (`e2e`).  The movie is 4 B x pixels x frames (8.08 GB at 1005^2 x
    2000, larger than L2); every pass streams it once: 2 x bg_iter passes per call."""
    import torch
    from mesolf_gb300 import synth
    from mesolf_gb300.api import summary_image
    from oracle import mesolf_ref as R
    P = side * side
    prm = ("pixelwise", 5, 100, 20, 3)
    Y = synth.sensor_movie(P, T, seed=17, device=dev)
    img, _, _ = summary_image(Y, *prm)  # warm
    pm, acc = np.zeros(5), np.zeros(5)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        img, bs, bt = summary_image(Y, *prm, pass_ms=pm)
        acc += pm
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    acc /= steps
    movie_bytes = 4.0 * P * T
    passes = 2 * prm[1]
    hbm = _measured_hbm()
    gbs = lambda t_ms: movie_bytes / (t_ms * 1e-3) / 1e9 if t_ms > 0 else None
    last_gbs = gbs(acc[3])
    t_e2e, same = float("nan"), None
    if e2e:
        # end to end from pinned host memory: H2D of the movie, D2H of the three outputs
        host = torch.empty((T, P), dtype=torch.float32, pin_memory=True)
        host.copy_(Y.T)
        hmov = host.T
        summary_image(hmov, *prm)
        t0 = time.perf_counter()
        for _ in range(2):
            himg, _, _ = summary_image(hmov, *prm)
        t_e2e = (time.perf_counter() - t0) / 2
        same = bool(torch.equal(himg, img.cpu()))
        del host, hmov
    out = {"workload": f"summary_image_{side}x{side}px_{T}frames_pixelwise_bg5_w100_w20_p3",
           "value": T / (ms * 1e-3), "unit": "frames/s", "ms_per_call": ms,
           "movie_gb": movie_bytes / 1e9, "movie_passes": passes,
           "pass_ms": {"first_column_with_max": acc[0], "column": acc[1], "row": acc[2],
                       "last_pixelwise": acc[3], "finalise": acc[4]},
           "stream_gbs": {"column": gbs(acc[1]), "row": gbs(acc[2]), "last_pixelwise": last_gbs,
                          "whole_call": movie_bytes * passes / (ms * 1e-3) / 1e9},
           "roofline": {"bound": "hbm", "kernel": "k_si_pixelwise (last pass: s, moving means, power, std)",
                        "achieved": last_gbs, "peak": hbm, "unit": "GB/s",
                        "frac": last_gbs / hbm if (hbm and last_gbs) else None,
                        "algorithmic_bytes_per_launch": movie_bytes, "traffic": None,
                        "note": "achieved = movie bytes / last-pass time (CUDA events around the launch); "
                                "peak = measured copy bandwidth"},
           "e2e": {"value": T / t_e2e, "unit": "frames/s", "s_per_call": t_e2e,
                   "h2d_bytes_per_step": int(movie_bytes), "d2h_bytes_per_step": int(4 * (2 * P + T)),
                   "same_result_as_device_input": same},
           "kernel_launches_per_call": 3 * prm[1] + 2,
           "data": "synthetic: per-pixel baselines, 20% bleaching trend, calcium-like transients, noise "
                   "(mesolf_gb300/synth.py sensor_movie)"}
    if cpu:
        idx = torch.arange(0, P, P // cpu_pixels, device=dev)[:cpu_pixels]
        sub = Y[idx].cpu().numpy()
        t0 = time.perf_counter()
        ri, _, _ = R.summary_image(sub, *prm)
        t_cpu = time.perf_counter() - t0
        got = img[idx].double().cpu().numpy()
        scale = float(np.dot(got, ri) / np.dot(ri, ri))
        out["cpu_baseline"] = {"value": T / (t_cpu * P / len(idx)), "unit": "frames/s", "cores": 1,
                               "kind": "port",
                               "sample": f"the FP64 numpy oracle on {len(idx)} of the {P} pixels, all {T} frames "
                                         f"({t_cpu:.2f} s), scaled by the pixel count"}
        out["rel_l2_vs_fp64_oracle_sampled_pixels"] = float(np.linalg.norm(got / scale - ri) / np.linalg.norm(ri))
    del Y
    torch.cuda.empty_cache()
    return out


def rectify_block(dev, frame=1100, T=2000, steps=3, cpu=True, e2e=True):
    """The input step: raw uint16 frames (frame x frame pixels, T frames) cut and rectified onto
    the lenslet grid (image_load_module_aug: Nnum 15, pitch 15.27 px, one patch with a
    one-lenslet border crop, 1050 x 1050 rectified pixels), movie left unnormalised in HBM for
    the summary image.  `value`: frames resident in HBM; `e2e`: frames from pinned host memory
    (cut region copied per frame inside the timed region), movie in HBM.  Algorithmic bytes per
    frame: the raw cut read once (2 B/px) + the rectified frame written (4 B/px)."""
    import torch
    from mesolf_gb300 import rectify as RC
    from oracle import mesolf_ref as R
    SI = dict(Nnum=15, frames_dx=15.27, frames_x_offset=frame / 2 + 0.3, frames_y_offset=frame / 2 - 0.4,
              frames_crop_border_microlenses=[1, 1, 1, 1], patch_mode="carpet", n_patches=1)
    info = RC.determine_patch_info_aug(SI, (frame, frame))[0]
    g = torch.Generator(device=dev)
    g.manual_seed(23)
    fr16 = (torch.rand((T, frame, frame), generator=g, device=dev) * 4000).to(torch.int16)
    fr = fr16.view(torch.uint16)                       # values < 4000: the same bits
    frames = fr.permute(2, 1, 0)                       # (rows, cols, T), column-major
    mov = RC.image_load_module_aug(info, SI, frames, normalize=False)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        mov = RC.image_load_module_aug(info, SI, frames, normalize=False)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    (y0, y1), (x0, x1) = info["raw_cut"]
    h, w = info["size"]
    alg = T * (2.0 * (y1 - y0 + 1) * (x1 - x0 + 1) + 4.0 * h * w)
    hbm = _measured_hbm()
    ach = alg / (ms * 1e-3) / 1e9
    t_e2e, same = float("nan"), None
    if e2e:
        host = fr16.cpu().pin_memory().view(torch.uint16).permute(2, 1, 0)
        RC.image_load_module_aug(info, SI, host, normalize=False, out_device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hm = RC.image_load_module_aug(info, SI, host, normalize=False, out_device=dev)
        torch.cuda.synchronize()
        t_e2e = time.perf_counter() - t0
        same = bool(torch.equal(hm, mov))
        del host, hm
    out = {"workload": f"rectify_{frame}x{frame}_u16_{T}frames_to_{h}x{w}", "value": T / (ms * 1e-3),
           "unit": "frames/s", "ms_per_call": ms,
           "roofline": {"bound": "hbm", "kernel": "k_rectify", "achieved": ach, "peak": hbm, "unit": "GB/s",
                        "frac": ach / hbm if hbm else None, "algorithmic_bytes_per_launch": alg, "traffic": None,
                        "note": "achieved = (raw cut read + rectified movie written) / call time"},
           "e2e": {"value": T / t_e2e, "unit": "frames/s", "s_per_call": t_e2e,
                   "h2d_bytes_per_step": int(2 * T * (y1 - y0 + 1) * (x1 - x0 + 1)), "d2h_bytes_per_step": 0,
                   "same_result_as_device_input": same, "note": "movie kept in HBM for the summary image"},
           "data": "seeded uniform uint16 frames"}
    if cpu:
        sub = 8
        fh = fr16[:sub].permute(2, 1, 0).cpu().numpy().astype(np.uint16)
        t0 = time.perf_counter()
        ref = R.image_load(fh, info, dict(SI, frames_end=sub))
        t_cpu = time.perf_counter() - t0
        got = mov[:, :sub].cpu().numpy()
        out["cpu_baseline"] = {"value": sub / t_cpu, "unit": "frames/s", "cores": 1, "kind": "port",
                               "sample": f"the FP64 numpy oracle (bilinear on the same grids) on {sub} frames "
                                         f"({t_cpu:.2f} s)"}
        out["rel_l2_vs_fp64_oracle_8_frames"] = float(np.linalg.norm(got / got.max() - ref) / np.linalg.norm(ref))
    del frames, fr, fr16, mov
    torch.cuda.empty_cache()
    return out


def _measured_bf16():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"]
    except Exception:
        return None


def _measured_hbm():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except Exception:
        return None


if __name__ == "__main__":
    main()
