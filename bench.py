"""Benchmark of the GB300 multifit engine (one JSON line on rank 0).

Metric: channels fitted per second on one GB300. A step is one fit of the
whole workload batch (every channel of it) already resident in HBM; `value`
is channels / device time (CUDA events on the launching stream, L2 flushed
between steps, max over ranks). `e2e` is the same fit through the host-pointer
C-ABI entry (mf_fit_host): pinned host inputs copied in, results copied back,
synchronised, every step inside the timed region.

`--impl reference` times the reference's CPU path instead: the reference
needs Eigen, which is absent, so its CPU implementation is the FP64 oracle
restatement (oracle/), run on all host cores over a bounded sample.

Multi-GPU: channels are independent, so N ranks each fit their own shard of
the channel stream with no collective on the data path ("replicas"; weak
scaling); the only collectives are the timing barrier and max-reduce.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "test-regression_gb300")
METRIC = "channels fitted/s on 1 GB300: MLP-warm FP32 vs plain FNNLS FP64, ≤1e-4 amp err"
UNIT = "channels/s"


def load_pkg():
    if "multifit_gb300" in sys.modules:
        return sys.modules["multifit_gb300"]
    spec = importlib.util.spec_from_file_location("multifit_gb300", os.path.join(PKG_DIR, "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["multifit_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def build_pkg():
    spec = importlib.util.spec_from_file_location("multifit_gb300_build", os.path.join(PKG_DIR, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    """One process per GPU (torchrun env). NCCL for our arm on GPUs; gloo for the
    CPU reference arm and wherever CUDA is absent (the CPU tests of this logic)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if args.impl != "reference" and torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def shard_range(rank: int, per_rank: int):
    """Channels [first, first + per_rank) of the seeded channel stream that a
    rank fits: channels are independent, so ranks fit disjoint contiguous
    shards with no collective on the data path (weak scaling)."""
    return rank * per_rank, per_rank


def max_over_ranks(x: float, world: int, device=None) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


WORKLOAD_DESC = {
    "ecal-1m-pu2": "1,000,000 ECAL 10x10 channels, CRRC4 tau=43ns, sigma=0.044, rho=0.7, in-time U[1,100], "
                   "pileup Poisson(2)xExp(1 GeV) per out-of-time BX, seed 2",
    "ecal-10k-pu0.5": "10,000 ECAL 10x10 channels, pileup 0.5, seed 1",
    "ecal-10m-logamp-pu4": "10,000,000 ECAL channels, in-time log-uniform [0.1,1000], pileup 4, seed 3",
    "mixed-10m-ecal-hcal": "10,000,000 channels, 40% HCAL 8x8, pileup U[0,8] per channel, seed 4",
    "warm-eval-10m": "10,000,000 ECAL channels, log-uniform [0.1,1000], pileup 4, seed 6",
}


FORM_DESC = {
    "fp64": "plain-fp64 drop-in (bit-identical to the oracle)",
    "mixed": "mixed precision: FP32 active-set search + double-float screen + FP64 judge (solve, residual, "
             "chi2), KKT-converged",
    "fp32": "FP32: FP32 active-set search + double-float screen and judge (FP32 error-free transforms), "
            "FP64 repair of the rare rejects, KKT-converged",
    "warm": "learned warm start: BF16 tensor-core MLP + the FP32 form (double-float judge) to KKT",
    "fp32-cov": "per-channel form of the FP32 precision (a pulse covariance makes the covariance "
                "amplitude-dependent): the outer loop's first iteration through the passive-set tables (FP32 "
                "search, double-float judge), then the FP64 fit from it, KKT-converged",
}
# the pulse covariance of the fp32-cov workload: 1e-4 exp(-|i-j| / 3) over the
# template's samples 7..18 of the 19-sample fullpulse (a pulse-shape jitter)
FPC_SCALE, FPC_LENGTH = 1e-4, 3.0


def pulse_covariance():
    import numpy as np

    F = np.zeros((19, 19))
    idx = np.arange(7, 19)
    F[np.ix_(idx, idx)] = FPC_SCALE * np.exp(-np.abs(np.subtract.outer(idx, idx)) / FPC_LENGTH)
    return F


def default_workload(form: str) -> str:
    return {"fp64": "ecal-1m-pu2", "fp32-cov": "ecal-1m-pu2"}.get(form, "warm-eval-10m")
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per channel of a
# launch, measured by ncu on the kernel of the form named (a capture of one
# 2,000,000-channel launch; the bytes grow with the channels, so a launch's
# traffic is this times its channels); the summary with the command is the
# profiles/ file given
NCU_DRAM_BYTES_PER_CHANNEL = {
    ("judge_kernel", "warm"): (180.8, "profiles/judge_kernel_fp32_warm-2m.md"),
    ("fit_fp64_kernel", "fp64"): (9016.8, "profiles/fit_fp64_kernel_ecal-1m-pu2.md"),  # both passes
}
# useful FLOPs of one warm-start prediction: 12 inputs -> 128 -> 128 -> 20
# outputs, 2 per multiply-add (the network pads to 16 inputs and 32 outputs)
MLP_FLOPS_PER_CHANNEL = 2 * (12 * 128 + 128 * 128 + 128 * 20)


def schedule_of(mf, args, mixed_sets):
    if args.schedule == "auto":  # persistent work stealing pays for batches of several condition sets
        return mf.SCHED_PERSISTENT if mixed_sets and args.form != "fp64" else mf.SCHED_GRID
    return {"grid": mf.SCHED_GRID, "persistent": mf.SCHED_PERSISTENT}[args.schedule]


def form_options(mf, args, mixed_sets=False):
    if args.form == "fp64":
        return mf.default_options(max_iter_nnls=args.max_iter, nnls_start=args.start)
    sched = schedule_of(mf, args, mixed_sets)
    if args.form == "mixed":
        return mf.default_options(precision=mf.PREC_MIXED, max_iter_nnls=1000, schedule=sched)
    if args.form == "fp32":
        return mf.default_options(precision=mf.PREC_FP32, max_iter_nnls=1000, schedule=sched)
    if args.form == "fp32-cov":
        return mf.default_options(precision=mf.PREC_FP32, max_iter_nnls=1000)
    return mf.default_options(precision=mf.PREC_FP32, warm_start=mf.WARM_MLP, max_iter_nnls=1000, schedule=sched)


def train_warm_start(mf, eng, torch, args, rank):
    """Trains the warm-start MLP on the GPU: 5,000,000 channels of the
    log-uniform pileup-4 generator (seed 5), fitted by the plain FP64 kernel to
    KKT convergence (the targets). Untimed; returns a summary."""
    p = mf.WORKLOADS["warm-train-5m"]()
    n = int(args.train_channels or p.n)
    t0 = time.perf_counter()
    s = torch.zeros((n, 10), dtype=torch.float64, device="cuda")
    pe = torch.zeros(n, dtype=torch.float64, device="cuda")
    a = torch.zeros((n, 10), dtype=torch.float64, device="cuda")
    c = torch.zeros(n, dtype=torch.float64, device="cuda")
    mf.synth_generate_device(p, 0, n, s.data_ptr(), pe.data_ptr(), None)
    b = mf.Engine._batch(n, 10, 10, s.data_ptr(), pe.data_ptr(), None, a.data_ptr(), c.data_ptr())
    eng.fit_device(b, mf.default_options(max_iter_nnls=1000, nnls_start=mf.START_SUPPORT))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    eng.mlp_init(0, seed=7)
    tp = mf.mlp_params(epochs=args.train_epochs, batch=8192, lr=2e-3)
    losses = eng.mlp_train(b, tp)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    del s, pe, a, c
    return {"channels": n, "generator": "log-uniform [0.1,1000] GeV, pileup 4, seed 5", "epochs": tp.epochs,
            "batch": tp.batch, "lr": tp.lr, "epoch_loss": [float(x) for x in losses],
            "target_fit_s": t1 - t0, "train_s": t2 - t1}


def fp32_peak_tflops(torch) -> float:
    """cuBLAS SGEMM (TF32 off) measured in this run: the FP32-pipe roofline."""
    n = 8192
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn((n, n), dtype=torch.float32, device="cuda")
    b = torch.randn((n, n), dtype=torch.float32, device="cuda")
    best = 0.0
    for _ in range(3):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    return best


def judge_fp64_flops(N, active) -> float:
    """FP64 flops of the FP64 judge summed over channels with passive sets
    `active` (int tensor of bit masks): the whitening N(N+1), per passive
    column the table row and the residual column (2N each, FMA = 2), and
    chi2 (2N + 2); the judge loops over the passive set only."""
    import torch

    bits = active.to(torch.int32)
    cols = sum(int(((bits >> k) & 1).sum().item()) for k in range(16))
    n = int(active.numel())
    return float(n * (N * (N + 1) + 2 * N + 2) + 4 * N * cols)


def judge_df_flops(P, active) -> float:
    """FP32 flops of the double-float judge summed over channels of a set
    with pulse matrix P (N x K), given their passive sets `active` (int
    tensor of bit masks): 17 per emulated FMA (TwoProduct 3, two cross FMAs
    4, renormalised sum 10) over the whitening N(N+1)/2 and, per passive
    column k, the table solve row (N) and the residual over G_k's structural
    non-zeros (nnz_k); plus the FP32 KKT screen of the other columns
    (4 N each) and the double-float chi2 (15 N). The judge loops over the
    passive set only, so this is the work it has to do, not a dense K-column
    count."""
    import numpy as np
    import torch

    N, K = P.shape
    nnz = [N - int(np.argmax(P[:, k] != 0)) if (P[:, k] != 0).any() else 0 for k in range(K)]
    bits = active.to(torch.int32)
    cols = 0  # passive columns, summed over the channels
    rows = 0  # table rows and G non-zeros of the passive columns, summed
    for k in range(K):
        c = int(((bits >> k) & 1).sum().item())
        cols += c
        rows += c * (N + nnz[k])
    n = int(active.numel())
    return float(17 * (n * N * (N + 1) // 2 + rows) + 4 * N * (n * K - cols) + 15 * N * n)


def fp64_peak_tflops(torch) -> float:
    """cuBLAS DGEMM throughput measured in this run: the FP64-pipe roofline."""
    n = 4096
    a = torch.randn((n, n), dtype=torch.float64, device="cuda")
    b = torch.randn((n, n), dtype=torch.float64, device="cuda")
    best = 0.0
    for _ in range(3):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def run_ours(args, world, rank, local):
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    build_pkg()
    mf = load_pkg()
    eng = mf.Engine(local)
    wl = args.workload or default_workload(args.form)
    p = mf.WORKLOADS[wl]()
    n = int(args.channels or p.n)
    p.n = n
    mixed = p.hcal_fraction > 0
    ecal, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    if args.form == "fp32-cov":
        P, R, bxs, _ = mf.conditions_arrays(ecal)
        ecal = mf.make_conditions(P, R, bxs, fullpulsecov=pulse_covariance())
    eng.set_conditions(0, ecal)
    if mixed:
        hcal, _ = mf.synth_conditions(mf.SYNTH_HCAL)
        eng.set_conditions(1, hcal)
    opt = form_options(mf, args, mixed)

    dev = "cuda"
    samples = torch.zeros((n, 10), dtype=torch.float64, device=dev)
    pederr = torch.zeros(n, dtype=torch.float64, device=dev)
    ctype = torch.zeros(n, dtype=torch.uint8, device=dev) if mixed else None
    amp = torch.zeros((n, 10), dtype=torch.float64, device=dev)
    chi2 = torch.zeros(n, dtype=torch.float64, device=dev)
    intime = torch.zeros(n, dtype=torch.float64, device=dev)
    mask = torch.zeros(n, dtype=torch.int16, device=dev)
    status = torch.zeros(n, dtype=torch.uint8, device=dev)
    first, _ = shard_range(rank, n)  # each rank fits its own shard of the channel stream
    mf.synth_generate_device(p, first, n, samples.data_ptr(), pederr.data_ptr(),
                             ctype.data_ptr() if mixed else None)
    batch = mf.Engine._batch(n, 10, 10, samples.data_ptr(), pederr.data_ptr(),
                             ctype.data_ptr() if mixed else None, amp.data_ptr(), chi2.data_ptr(),
                             intime.data_ptr(), None, mask.data_ptr(), status.data_ptr(), None)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    torch.cuda.synchronize()

    training = None
    if args.form == "warm":
        training = train_warm_start(mf, eng, torch, args, rank)

    # algorithmic work of one launch: the plain FP64 algorithm's executed flops
    # on these channels (instrumented kernel, untimed) -- the same useful work
    # whatever form runs
    flops = torch.zeros(n, dtype=torch.float64, device=dev)
    eng.fit_count_flops(batch, flops.data_ptr(), mf.default_options(), stream.cuda_stream)
    torch.cuda.synchronize()
    flops_per_launch = float(flops.sum().item())
    # the FP64 work the timed form itself executes (its bound is the FP64 pipe)
    form_fp64_flops = flops_per_launch
    if args.form != "fp64":
        flops.zero_()
        eng.fit_count_flops(batch, flops.data_ptr(), opt, stream.cuda_stream)
        torch.cuda.synchronize()
        form_fp64_flops = float(flops.sum().item())
    del flops

    tune = None
    if args.autotune and opt.schedule == mf.SCHED_PERSISTENT:
        t0 = time.perf_counter()
        pts = eng.autotune(batch, opt)
        best = min(pts, key=lambda q: q[2])
        tune = {"seconds": time.perf_counter() - t0, "best": {"block_size": best[0], "channels_per_warp": best[1]},
                "points_ms": {f"b{q[0]}_cpw{q[1]}": round(q[2], 4) for q in pts}}

    def step():
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.fit_device(batch, opt, stream.cuda_stream)
            e1.record(stream)
        return e0, e1

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    eng.profile(True)  # per-kernel CUDA events on the launch stream, inside the timed region
    torch.cuda.nvtx.range_push("timed_region")  # lets ncu --nvtx-include select exactly these launches
    evs = [step() for _ in range(args.steps)]
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    kernels = eng.profile_read()
    eng.profile(False)
    times = [e0.elapsed_time(e1) for e0, e1 in evs]
    graph_ms = None
    if opt.schedule == mf.SCHED_PERSISTENT:
        # the same steps replayed as the captured CUDA graph (per-kernel timing
        # off, which is what makes the engine use the graph)
        step()
        torch.cuda.synchronize()
        gev = [step() for _ in range(args.steps)]
        torch.cuda.synchronize()
        graph_ms = sum(e0.elapsed_time(e1) for e0, e1 in gev) / len(gev)
    step_ms = sum(times) / len(times)
    step_ms_max = max_over_ranks(step_ms, world, device=dev)
    value = n * world / (step_ms_max * 1e-3)

    iters_out = None
    baseline = None
    accuracy = None
    if args.form != "fp64":
        torch.cuda.synchronize()
        form_amp = amp.clone()
        form_mask = mask.clone()
        form_chi2 = chi2.clone()
        # the clones run on torch's default stream and the fits below on `stream`
        # (non-blocking): let the copies finish before anything overwrites amp/mask
        torch.cuda.synchronize()
        # the plain FP64 drop-in on the same inputs (the denominator of the headline ratio)
        popt = mf.default_options()
        eng.fit_device(batch, popt, stream.cuda_stream)
        torch.cuda.synchronize()
        bts = []
        for _ in range(max(1, min(3, args.steps))):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                eng.fit_device(batch, popt, stream.cuda_stream)
                e1.record(stream)
            e1.synchronize()
            bts.append(e0.elapsed_time(e1))
        bms = max_over_ranks(sum(bts) / len(bts), world, device=dev)
        baseline = {"form": "plain-fp64 drop-in (reference start, max_iter 10)", "value": n * world / (bms * 1e-3),
                    "ms_per_step": bms, "speedup_of_form": (n * world / (step_ms_max * 1e-3)) / (n * world / (bms * 1e-3))}
        # the form against multifit_cpu's own result: `amp` now holds the plain FP64
        # fit with multifit_cpu's settings (reference start, max_iter 10)
        torch.cuda.synchronize()
        err_c = (form_amp - amp).abs().amax(dim=1) / amp.abs().amax(dim=1).clamp_min(1e-300)
        d_chi2 = (chi2 - form_chi2) / form_chi2.abs().clamp_min(1.0)
        vs_cpu = {"reference": "plain FP64 GPU kernel with multifit_cpu's settings (reference start, max_iter 10; "
                               "bit-identical to the oracle)",
                  "channels": n,
                  "frac_within_1e-5": float((err_c <= 1e-5).double().mean().item()),
                  "frac_within_1e-4": float((err_c <= 1e-4).double().mean().item()),
                  "support_identical_frac": float((form_mask == mask).double().mean().item()),
                  "chi2_multifit_cpu_above_frac": float((d_chi2 > 1e-9).double().mean().item()),
                  "chi2_multifit_cpu_below_frac": float((d_chi2 < -1e-9).double().mean().item()),
                  "chi2_note": "(chi2_cpu - chi2_form) / max(chi2_form, 1) beyond +-1e-9: where multifit_cpu's "
                               "chi2 is above, it stopped short of the NNLS optimum the form returns"}
        # accuracy of the form against the plain FP64 kernel run to KKT convergence, whole batch on the GPU
        eng.fit_device(batch, mf.default_options(max_iter_nnls=1000, nnls_start=mf.START_SUPPORT),
                       stream.cuda_stream)
        torch.cuda.synchronize()
        scale = amp.abs().amax(dim=1).clamp_min(1e-300)
        err = (form_amp - amp).abs().amax(dim=1) / scale
        same = (form_mask == mask)
        chi2_err = ((form_chi2 - chi2).abs() / chi2.abs().clamp_min(1.0))[same]
        accuracy = {"reference": "plain FP64 GPU kernel, support start, max_iter 1000 (bit-identical to the oracle)",
                    "channels": n, "rel_amp_err_median": float(err.median().item()),
                    "rel_amp_err_p999": float(torch.quantile(err[: min(n, 4_000_000)].float(), 0.999).item()),
                    "rel_amp_err_max": float(err.max().item()),
                    "frac_within_1e-4": float((err <= 1e-4).double().mean().item()),
                    "chi2_rel_err_median": float(chi2_err.median().item()) if chi2_err.numel() else None,
                    "chi2_rel_err_max": float(chi2_err.max().item()) if chi2_err.numel() else None,
                    "chi2_note": "|chi2 - chi2_ref| / max(chi2_ref, 1) on channels whose active sets agree",
                    "active_set_identical_frac": float(same.double().mean().item()),
                    "vs_multifit_cpu": vs_cpu}
        amp.copy_(form_amp)
        mask.copy_(form_mask)
        chi2.copy_(form_chi2)
        torch.cuda.synchronize()

    # parity spot check of this run's output against the oracle
    parity = None
    if rank == 0 and not args.no_parity:
        sys.path.insert(0, ROOT)
        import oracle

        m = min(n, 2000)
        inp_s = samples[:m].cpu().numpy()
        inp_p = pederr[:m].cpu().numpy()
        ct = ctype[:m].cpu().numpy() if mixed else np.zeros(m, np.uint8)
        a_gpu = amp[:m].cpu().numpy()
        ok = True
        worst = 0.0
        for t, cond in eng.conditions.items():
            sel = np.nonzero(ct == t)[0]
            if sel.size == 0:
                continue
            P, R, bxs, F = mf.conditions_arrays(cond)
            if args.form == "fp64":
                ref = oracle.fit_batch(inp_s[sel], inp_p[sel], P, R, bxs, fullpulsecov=F, max_iter_nnls=args.max_iter,
                                       start=args.start)
                ok = ok and bool(np.array_equal(a_gpu[sel, : P.shape[1]], ref["amplitudes"]))
            else:
                ref = oracle.fit_batch(inp_s[sel], inp_p[sel], P, R, bxs, fullpulsecov=F, max_iter_nnls=1000, start=1)
                r = ref["amplitudes"]
                e = np.abs(a_gpu[sel, : P.shape[1]] - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-300)
                worst = max(worst, float(e.max())) if sel.size else worst
        if args.form == "fp64":
            parity = {"sample_channels": m, "bitwise_equal_to_oracle": ok}
        else:
            parity = {"sample_channels": m, "oracle": "FP64 oracle, support start, max_iter 1000",
                      "max_rel_amp_err": worst, "tolerance": 1e-4, "ok": worst <= 1e-4}

    # end to end through the host-pointer entry point (pinned buffers)
    h_s = torch.empty((n, 10), dtype=torch.float64).pin_memory()
    h_p = torch.empty(n, dtype=torch.float64).pin_memory()
    h_s.copy_(samples)
    h_p.copy_(pederr)
    h_ct = None
    if mixed:
        h_ct = torch.empty(n, dtype=torch.uint8).pin_memory()
        h_ct.copy_(ctype)
    h_amp = torch.empty((n, 10), dtype=torch.float64).pin_memory()
    h_chi2 = torch.empty(n, dtype=torch.float64).pin_memory()
    h_int = torch.empty(n, dtype=torch.float64).pin_memory()
    h_mask = torch.empty(n, dtype=torch.int16).pin_memory()
    h_st = torch.empty(n, dtype=torch.uint8).pin_memory()
    hb = mf.Engine._batch(n, 10, 10, h_s.data_ptr(), h_p.data_ptr(), h_ct.data_ptr() if mixed else None,
                          h_amp.data_ptr(), h_chi2.data_ptr(), h_int.data_ptr(), None, h_mask.data_ptr(),
                          h_st.data_ptr(), None)
    import ctypes as C

    def e2e_step():
        rc = eng.lib.mf_fit_host(eng.h, C.byref(hb), C.byref(opt))
        if rc:
            raise RuntimeError(f"mf_fit_host rc={rc}")

    for _ in range(args.warmup):
        e2e_step()
    barrier(world)
    e2e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    # the median step: the host side of these machines is shared, and a step
    # that waited on someone else's host-memory traffic says nothing of the engine
    e2e_sorted = sorted(e2e_times)
    e2e_s = max_over_ranks(e2e_sorted[len(e2e_sorted) // 2], world, device=dev)
    e2e_mean_s = max_over_ranks(sum(e2e_times) / len(e2e_times), world, device=dev)
    h2d = n * (10 * 8 + 8 + (1 if mixed else 0))
    d2h = n * (10 * 8 + 8 + 8 + 2 + 1)

    peaks, peak_src = measured_peaks()
    fp64_peak = fp64_peak_tflops(torch)
    fp32_peak = fp32_peak_tflops(torch)
    bytes_per_launch = n * (10 * 8 + 8) + n * (10 * 8 + 8 + 8 + 2 + 1)
    hbm_gbs = bytes_per_launch / (step_ms * 1e-3) / 1e9
    kernel_table = kernel_rooflines(mf, eng, kernels, args, n, ctype, flops_per_launch, form_fp64_flops,
                                    fp64_peak, fp32_peak, peaks, peak_src, step_ms, mask)
    dominant = max(kernel_table, key=lambda k: kernel_table[k]["ms_per_step"])
    roof = dict(kernel_table[dominant])
    roof["kernel"] = dominant

    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(args, wl, n, budget_s=args.cpu_seconds)
        out = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": step_ms_max,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": {"fp64": "f64", "mixed": "f32+f64", "fp32": "f32 (double-float judge; f64 repair)",
                      "warm": "f32 (double-float judge; f64 repair; bf16 MLP)",
                      "fp32-cov": "f32 first iteration (double-float judge); f64 from the second"}[args.form],
            "data": "synthetic (seeded Philox generator; the workload's shapes and value distributions)",
            "config": workload_config(args, wl, n, world),
            "engine": {
                "form": FORM_DESC[args.form],
                "max_iter_nnls": opt.max_iter_nnls,
                "nnls_start": ["reference", "support"][opt.nnls_start] if args.form == "fp64" else "KKT-converged",
                "schedule": ["grid", "persistent work-stealing"][opt.schedule],
                "launch_shape": {"block_size": opt.block_size or "tuned/default",
                                 "channels_per_warp": opt.channels_per_warp or "tuned/default"},
                "autotune": tune,
                "graph_replay_ms_per_step": graph_ms,
                "timed_region_launches": "direct (per-kernel CUDA events on)" if graph_ms else "direct",
            },
            "e2e": {"value": n * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "entry": "mf_fit_host (pinned host buffers, pipelined copies)",
                    "statistic": "median step wall time",
                    "value_mean": n * world / e2e_mean_s, "ms_mean": e2e_mean_s * 1e3,
                    "step_ms": {"median": e2e_s * 1e3, "min": e2e_sorted[0] * 1e3, "max": e2e_sorted[-1] * 1e3,
                                "mean": sum(e2e_times) / len(e2e_times) * 1e3}},
            "roofline": roof,
            "kernels": kernel_table,
            "roofline_hbm": {"bound": "hbm", "achieved": hbm_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                             "frac": hbm_gbs / peaks["hbm_gbs"], "peak_source": peak_src,
                             "algorithmic_bytes_per_launch": bytes_per_launch},
            "cpu_baseline": cpu,
            "plain_fp64_same_inputs": baseline,
            "accuracy": accuracy,
            "mlp_training": training,
            "gpu_launches": sum(v[0] for v in kernels.values()),
            "clocks": clk,
            "parity": parity,
        }
        print(json.dumps(out), flush=True)
    eng.close()
    return out


def kernel_rooflines(mf, eng, kernels, args, n, ctype, plain_flops, form_fp64_flops, fp64_peak, fp32_peak, peaks,
                     peak_src, step_ms, active):
    """Roofline of every kernel launched in the timed region: its algorithmic
    work per launch over its mean launch time (CUDA events from mf_profile).

    fit_fp64_kernel: the plain fit's executed FP64 flops (instrumented count).
    judge_kernel: the FP64 judge's FP64 flops (judge_fp64_flops) and the
      double-float judge's FP32 flops (judge_df_flops), both summed over each
      channel's passive set (the form's active masks `active`).
    repair_kernel: the rest of the form's counted FP64 flops.
    mlp_infer_tc_kernel: MLP_FLOPS_PER_CHANNEL on the tensor cores (BF16, tcgen05).
    search_kernel: FP32 and latency-bound; its HBM bytes (samples, pederr,
      warm start in; hand-off out) against the copy bandwidth.
    fix_kernel, judge_fixed_kernel: run on the queued channels only; time and
      share, no roofline."""
    import numpy as np

    counts = {0: n}
    if ctype is not None:
        ct = np.bincount(ctype.cpu().numpy(), minlength=2)
        counts = {0: int(ct[0]), 1: int(ct[1])}
    judge = 0.0      # FP64 flops of the FP64 judge
    judge_df = 0.0   # FP32 flops of the double-float judge
    for t, m in counts.items():
        c = eng.conditions.get(t)
        if c is None:
            continue
        N, K = c.nsamples, c.npulses
        sel = active if ctype is None else active[ctype == t]
        judge += judge_fp64_flops(N, sel)
        judge_df += judge_df_flops(mf.conditions_arrays(c)[0], sel)
    df_form = args.form in ("fp32", "warm", "fp32-cov")
    warm = args.form == "warm"
    out = {}
    for name, (launches, total) in kernels.items():
        per_step = launches / args.steps
        ms = total / args.steps
        mean_s = total / launches * 1e-3
        if name == "fit_fp64_kernel" and args.form == "fp32-cov":
            # the per-channel form's FP64 continuation: its own counted FP64 flops
            work, bound, peak, unit = form_fp64_flops / per_step, "fp64", fp64_peak, "TFLOP/s"
        elif name == "fit_fp64_kernel":
            work, bound, peak, unit = plain_flops / per_step, "fp64", fp64_peak, "TFLOP/s"
        elif name == "judge_kernel" and df_form:
            work, bound, peak, unit = judge_df / per_step, "fp32", fp32_peak, "TFLOP/s"
        elif name == "judge_kernel":
            work, bound, peak, unit = judge / per_step, "fp64", fp64_peak, "TFLOP/s"
        elif name == "repair_kernel" and args.form == "fp32-cov":
            # the per-channel form's FP64 count is its continuation's: the repair's is not counted
            # apart -- time and share without a roofline
            out[name] = {"bound": None, "achieved": None, "peak": None, "unit": None, "frac": None,
                         "traffic": None, "launches_per_step": per_step, "ms_per_step": ms,
                         "share": ms / step_ms, "work_per_launch": None, "peak_source": None}
            continue
        elif name == "repair_kernel":
            # the FP64 judge's share of the counted FP64 flops belongs to the judge (its repairs redo it)
            rest = form_fp64_flops - (0.0 if df_form else judge)
            work, bound, peak, unit = max(rest, 0.0) / per_step, "fp64", fp64_peak, "TFLOP/s"
        elif name == "mlp_infer_tc_kernel":
            work = n * MLP_FLOPS_PER_CHANNEL / per_step
            bound, peak, unit = "tensor", peaks["bf16_tflops"], "TFLOP/s"
        elif name == "screen_kernel":  # samples + hand-off in, refined hand-off out (FP32 double-float)
            work = n * (10 * 8 + 44 + 40) / per_step
            bound, peak, unit = "hbm", peaks["hbm_gbs"], "GB/s"
        elif name in ("fix_kernel", "judge_fixed_kernel"):
            # second-pass kernels on the queued channels only (their count is not recorded):
            # time and share without a roofline
            out[name] = {"bound": None, "achieved": None, "peak": None, "unit": None, "frac": None,
                         "traffic": None, "launches_per_step": per_step, "ms_per_step": ms,
                         "share": ms / step_ms, "work_per_launch": None, "peak_source": None}
            continue
        elif name == "partition_kernel":  # ctype in, channel lists out
            work = n * (1 + 4) / per_step
            bound, peak, unit = "hbm", peaks["hbm_gbs"], "GB/s"
        else:  # search_kernel
            work = n * (10 * 8 + 8 + (2 + 40 if warm else 0) + 2 + 2 + 40) / per_step
            bound, peak, unit = "hbm", peaks["hbm_gbs"], "GB/s"
        achieved = work / mean_s / (1e12 if unit == "TFLOP/s" else 1e9)
        measured = NCU_DRAM_BYTES_PER_CHANNEL.get((name, args.form))
        out[name] = {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
                     "traffic": measured[0] * n / per_step if measured else None,
                     "traffic_unit": "bytes per launch" if measured else None,
                     "traffic_source": f"{measured[1]} ({measured[0]} B/channel x channels per launch)"
                     if measured else None,
                     "launches_per_step": per_step, "ms_per_step": ms,
                     "share": ms / step_ms, "work_per_launch": work,
                     "peak_source": ("cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe)" if bound == "fp64"
                                     else "cuBLAS SGEMM 8192^3, TF32 off, measured in this run (FP32 pipe)"
                                     if bound == "fp32" else f"MEASURED_PEAKS.json ({peak_src})")}
    return out


def reference_fit_setting(args):
    """(max_iter_nnls, nnls start, label) of the fit both arms compute: the
    warm/mixed/FP32 forms return each channel's NNLS optimum (KKT point), which
    the reference path reaches with max_iter 1000 and the support start; the
    FP64 form is timed with the settings given on the command line."""
    if args.form == "fp64":
        return args.max_iter, args.start, ("multifit_cpu literal (reference start, max_iter %d)" % args.max_iter
                                           if args.start == 0 else "support start, max_iter %d" % args.max_iter)
    return 1000, 1, "NNLS to KKT convergence (support start, max_iter 1000)"


def workload_config(args, wl: str, n: int, world: int) -> dict:
    """The `config` both arms print: the workload and the fit it asks for,
    nothing that depends on which arm runs it."""
    _, _, fit = reference_fit_setting(args)
    cfg = {"workload": wl, "description": WORKLOAD_DESC.get(wl, wl), "channels_per_step": n, "fit": fit,
           "l2": "inputs (88 B/channel) exceed every cache; the GPU arm also flushes its L2 between steps "
                 "(256 MB write)",
           "parallelism": f"replicas x{world}"}
    if args.form == "fp32-cov":
        cfg["fullpulsecov"] = f"{FPC_SCALE:g} exp(-|i-j|/{FPC_LENGTH:g}) over fullpulse samples 7..18"
    return cfg


class CpuReference:
    """The reference's CPU path on this host: the oracle restatement of
    multifit_cpu's fit (oracle/, C++), fed by the oracle's own seeded
    generator. Loads nothing of the engine."""

    def __init__(self, wl: str, n: int, fullpulsecov=None):
        sys.path.insert(0, ROOT)
        import numpy as np

        import oracle

        self.oracle, self.np = oracle, np
        self.fpc = fullpulsecov
        self.nt = oracle.hardware_threads()
        self.wl, self.n = wl, n
        sets = [0, 1] if oracle.WORKLOADS[wl].get("hcal_fraction", 0.0) > 0 else [0]
        self.conds = {t: oracle.synth_conditions(t) for t in sets}
        d = oracle.synth_generate(wl, 0, n)
        # channels of each condition set in contiguous arrays (the fits are per set)
        self.parts = {}
        for t in sets:
            sel = np.nonzero(d["ctype"] == t)[0]
            self.parts[t] = (np.ascontiguousarray(d["samples"][sel]), np.ascontiguousarray(d["pederr"][sel]))

    def fit(self, max_iter: int, start: int, nthreads: int = 0, m: int | None = None) -> float:
        """Fits the first m channels of every set; returns the wall seconds."""
        t0 = time.perf_counter()
        for t, (s, pe) in self.parts.items():
            k = s.shape[0] if m is None else min(s.shape[0], m)
            if k == 0:
                continue
            P, R, bxs, _ = self.conds[t]
            self.oracle.fit_batch(s[:k], pe[:k], P, R, bxs, fullpulsecov=self.fpc if t == 0 else None,
                                  max_iter_nnls=max_iter, start=start, nthreads=nthreads or self.nt)
        return time.perf_counter() - t0

    def channels(self, m: int | None) -> int:
        return sum(s.shape[0] if m is None else min(s.shape[0], m) for s, _ in self.parts.values())

    def rate(self, max_iter: int, start: int, nthreads: int, budget_s: float, cap: int | None = None) -> dict:
        """Channels/s on a sample sized to about budget_s of work (a probe of
        2,000 channels per thread first)."""
        probe = min(self.n, 2000 * nthreads)
        dt = self.fit(max_iter, start, nthreads, probe)
        per = dt / max(self.channels(probe), 1)
        m = int(min(self.n, cap or self.n, max(probe, budget_s / max(per, 1e-12))))
        dt = self.fit(max_iter, start, nthreads, m)
        c = self.channels(m)
        return {"value": c / dt, "unit": UNIT, "threads": nthreads, "channels": c, "seconds": dt}


def cpu_baseline(args, wl: str, n: int, budget_s: float = 10.0) -> dict:
    """The reference's CPU path (oracle port) on the host cores over a bounded
    sample of the same workload: all threads and one thread (the reference
    driver's own setting, multifit_cpu/src/multifit.cpp:196-227), for the fit
    the timed form computes and for multifit_cpu's literal settings."""
    mi, st, fit = reference_fit_setting(args)
    ref = CpuReference(wl, min(n, 2_000_000), pulse_covariance() if args.form == "fp32-cov" else None)
    allt = ref.rate(mi, st, ref.nt, budget_s * 0.4)
    one = ref.rate(mi, st, 1, budget_s * 0.2)
    lit_all = ref.rate(10, 0, ref.nt, budget_s * 0.25)
    lit_one = ref.rate(10, 0, 1, budget_s * 0.15)
    return {"value": allt["value"], "unit": UNIT, "cores": ref.nt, "kind": "port",
            "sample": f"first {allt['channels']} channels of {wl}, {fit}, all {ref.nt} host threads, "
                      f"{allt['seconds']:.2f} s",
            "one_thread": one,
            "multifit_cpu_settings": {"fit": "reference start, max_iter 10", "all_threads": lit_all,
                                      "one_thread": lit_one}}


def run_reference(args, world, rank):
    """The reference arm: the reference's CPU implementation of the path (the
    oracle port; the reference itself needs Eigen, absent here) on all host
    threads, over the same workload, channel count and fit as the GPU arm,
    with inputs from the oracle's own generator. Nothing of the engine is
    loaded. Rank 0 alone runs it."""
    if rank != 0:
        return None
    wl = args.workload or default_workload(args.form)
    sys.path.insert(0, ROOT)
    import oracle

    n = int(getattr(args, "channels", 0) or oracle.WORKLOADS[wl]["n"])
    mi, st, fit = reference_fit_setting(args)
    ref = CpuReference(wl, n, pulse_covariance() if args.form == "fp32-cov" else None)
    # a step fits every channel unless that would take longer than the step cap:
    # then the first m channels of each set, stated in the line
    probe_dt = ref.fit(mi, st, ref.nt, min(n, 20_000))
    est = probe_dt / max(ref.channels(min(n, 20_000)), 1) * ref.channels(None)
    cap_s = getattr(args, "ref_step_cap_s", 8.0)
    m = None if est <= cap_s else max(1000, int(n * cap_s / est))
    for _ in range(args.warmup):
        ref.fit(mi, st, ref.nt, m)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ref.fit(mi, st, ref.nt, m)
    dt = (time.perf_counter() - t0) / args.steps
    c = ref.channels(m)
    value = c / dt
    sample = (f"all {c} channels of {wl} per step" if m is None else f"first {c} of {n} channels of {wl} per step")
    sample += f", {fit}, all {ref.nt} host threads"
    # multifit_cpu's literal settings on the same channels, and one thread
    lit_steps = max(1, min(3, args.steps))
    t0 = time.perf_counter()
    for _ in range(lit_steps):
        ref.fit(10, 0, ref.nt, m)
    lit = {"fit": "multifit_cpu literal (reference start, max_iter 10)", "value": c * lit_steps /
           (time.perf_counter() - t0), "unit": UNIT, "threads": ref.nt, "channels": c, "steps": lit_steps}
    budget = getattr(args, "cpu_seconds", 10.0)
    one = ref.rate(mi, st, 1, budget * 0.5, cap=n)
    lit_one = ref.rate(10, 0, 1, budget * 0.5, cap=n)
    out = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Philox generator; the workload's shapes and value distributions)",
        "config": workload_config(args, wl, n, world),
        "implementation": {"path": "the reference's multifit_cpu fit, restated in C++ (oracle/; the reference "
                                   "needs Eigen, absent here)",
                           "generator": "oracle/synth_oracle.cpp (the engine library is not loaded)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": ref.nt, "kind": "port", "sample": sample,
                         "one_thread": one,
                         "multifit_cpu_settings": {"all_threads": lit, "one_thread": lit_one}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=["warm", "fp32", "mixed", "fp64", "fp32-cov"], default="warm")
    ap.add_argument("--schedule", choices=["auto", "grid", "persistent"], default="auto",
                    help="auto: persistent work stealing for workloads of several condition sets "
                         "(mixed/warm forms), else grid")
    ap.add_argument("--autotune", action="store_true",
                    help="sweep the persistent schedule's launch shape on the workload first (untimed)")
    ap.add_argument("--workload", default="",
                    help="default: warm-eval-10m (warm/fp32/mixed), ecal-1m-pu2 (fp64, fp32-cov)")
    ap.add_argument("--train-channels", type=int, default=0)
    ap.add_argument("--train-epochs", type=int, default=3)
    ap.add_argument("--channels", type=int, default=0, help="override the workload's channel count")
    ap.add_argument("--max-iter", type=int, default=10)
    ap.add_argument("--start", type=int, default=0, choices=[0, 1])
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU work of the cpu_baseline sample and of the reference arm's one-thread legs")
    ap.add_argument("--ref-step-cap-s", type=float, default=8.0,
                    help="reference arm: a step fits every channel unless that takes longer than this")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
