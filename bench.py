"""Benchmark: outer ADMM iterations/s of CDLmotif's CDL hot path on one GB300.

Workload (the headline configuration): N = 20000 sequences of L = 200 bases,
one-hot float32 (4 channels), 5 planted motifs of widths 8..20 (Dirichlet(0.1)
columns, 10..40 % occupancy, random strand), K = M = 64 filters of 16 bases
(Lg = 4L + 8W = 928), lambda 0.1, rho 1, sigma 100.  One step = one outer ADMM
iteration of cdl_optimize (src/WRAPPER/wrap.jl:6-11): 15 X-steps, update_best!,
1 D-step.

  value  device-resident: state and data already in HBM.
  e2e    through the public C ABI with host buffers: every step is one training of
         cdl_optimize (src/WRAPPER/wrap.jl:1-32): it uploads the one-hot data from
         pinned host memory (cdlgb_load_data), initialises the state
         (cdlgb_init_state), runs E = iter_num = 10 outer iterations (the reference's
         default, src/SETUP/WRAPPER_setup.jl:10; cdlgb_run_outer) and reads the
         objectives and D_best back; the unit is the same (outer iterations/s).

``--impl reference`` times the CPU restatement of the reference (oracle/cdl_cpu.cpp:
src/CDL/train.jl's statements in float32 on host arrays with full complex FFTs,
OpenMP over the sequences on every host core; the reference has no host path of its
own and Julia is absent) on the first 2000 sequences, one outer iteration per step,
and reports the same metric scaled to the full N (the factor is in the line).

``--impl refstruct`` times the reference-structured CUDA baseline (baseline/refstruct.cu:
the reference's CUDA.jl statements restated one for one, full-spectrum cuFFT C2C,
a sync after every custom kernel), the stand-in for the reference GPU path, on the
same workload on the GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="plain_n20000_l200_k64", N=20000, L=200, M=64, filter_size=16,
                widths=[8, 11, 14, 17, 20], occ=[0.1, 0.175, 0.25, 0.325, 0.4],
                lam=0.1, rho=1.0, sigma=100.0, csc_iter=15, cdl_iter=1, seed=2024)
METRIC = "ADMM outer iterations/s at N=20k, L=200, K=64 (15 X-steps + update_best + 1 D-step)"
UNIT = "outer_iter/s"


def _pkg():
    import __graft_entry__ as ge
    return ge._pkg()


def dataset(wl=WORKLOAD, N=None):
    pkg = _pkg()
    n = wl["N"] if N is None else N
    bases, _, _ = pkg.synth.plant_dataset(wl["seed"], n, wl["L"], wl["widths"], wl["occ"])
    return bases[:n]


# DRAM bytes (read + write) of one launch on 1000 sequences of the L=200, K=64 workload,
# from the ncu captures summarised in profiles/
XITER_DRAM_BYTES_N1000 = 1394415360      # k_xiter, one launch = 15 X-steps
XWARP_DRAM_BYTES_N1000 = 1391571456      # k_xstep_warp, one launch = 1 X-step
# warp instructions issued per sequence and X-step by k_xiter<32, 29, 288, 1, 16>
# (smsp__inst_executed.sum of the same 1000-sequence capture / (1000 x 15))
XITER_WARP_INSTR_PER_SEQ_XSTEP = 126.6e3
N_SM, SCHEDULERS_PER_SM = 152, 4


def algorithmic_bytes(wl=WORKLOAD):
    """Minimum HBM traffic per outer iteration and per X-step / D-step (state read
    and written once per step, FP32): X-step 24 B per (l,m,n) + 28 B per (l,n);
    D-step 32 B per (l,m,n) + 24 B per (l,n); objective 4 B per (l,m,n) + 4 per (l,n)."""
    Lg = 4 * wl["L"] + 8 * wl["filter_size"]
    LMN = Lg * wl["M"] * wl["N"]
    LN = Lg * wl["N"]
    bx = 24 * LMN + 28 * LN
    bd = 32 * LMN + 24 * LN
    bo = 4 * LMN + 4 * LN
    return dict(Lg=Lg, LMN=LMN, LN=LN, xstep=bx, dstep=bd, obj=bo,
                outer=wl["csc_iter"] * bx + wl["cdl_iter"] * bd + bo)


# ------------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
              "utilization.gpu")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        util = [float(r[9]) for r in rows if len(r) > 9 and r[9].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows),
                "gpu_util_mean_pct": float(np.mean(util)) if util else None,
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
                if any(r[3].replace(".", "").isdigit() for r in rows) else None}


# ------------------------------------------------------------------------ CPU leg
def cpu_reference(steps: int, warmup: int, n_sample: int, threads: int = 0):
    """Times the float32 C++/OpenMP CPU restatement of the reference (oracle/cdl_cpu.cpp:
    src/CDL/train.jl's statements on host arrays, full complex FFTs) with `threads`
    OpenMP threads (0 = every host core) on the first n_sample sequences of the
    workload: W untimed and K timed outer iterations.  Returns (outer iterations/s
    scaled to the full N, mean ms per sample step, threads, sample text)."""
    from oracle.cdl_cpu import CPUADMM, threads as omp_threads
    pkg = _pkg()
    wl = WORKLOAD
    bases = dataset(wl, N=n_sample)
    S = pkg.synth.onehot(bases)
    Lg = 4 * wl["L"] + 8 * wl["filter_size"]
    X0 = pkg.synth.init_X0(1, n_sample, wl["M"], Lg)
    D0 = pkg.synth.init_D0_unit_norm(1, wl["M"], Lg, 4 * wl["filter_size"])
    c = CPUADMM(S, X0, D0, wl["M"], wl["filter_size"], wl["rho"], wl["sigma"], wl["lam"],
                threads=threads)
    nt = threads or omp_threads()
    t = []
    for s in range(warmup + steps):
        t0 = time.perf_counter()
        c.run_outer(1, wl["csc_iter"], wl["cdl_iter"])
        if s >= warmup:
            t.append(time.perf_counter() - t0)
    c.close()
    sec = float(np.mean(t))
    factor = wl["N"] / n_sample
    rate = 1.0 / (sec * factor)
    sample = (f"{n_sample} of {wl['N']} sequences, one outer iteration per step, float32 C++/OpenMP "
              f"restatement of the reference (full complex FFTs) on {nt} threads; rate = "
              f"1 / (seconds per step x {factor:g}) (extrapolation factor {factor:g})")
    return rate, sec * 1e3, nt, sample


# ------------------------------------------------------------------------ GPU leg
def max_over_ranks(x: float, world: int, device: str) -> float:
    """The largest of every rank's x (all-reduce MAX; the process group's backend
    decides where the tensor lives: NCCL on the GPU, gloo on the CPU)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, units_per_rank: int, seconds_max: float) -> float:
    """Whole-job rate of `world` independent replicas, each processing units_per_rank
    outer iterations, timed by the slowest rank."""
    return world * units_per_rank / seconds_max


def run_gpu(args, rank: int, world: int):
    import torch
    pkg = _pkg()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = WORKLOAD
    bases = dataset(wl)
    S = pkg.synth.onehot(bases)
    setup = pkg.CDLSetup(M=wl["M"], filter_size=wl["filter_size"], lambda_=wl["lam"], rho=wl["rho"],
                         sigma=wl["sigma"], csc_iter_num=wl["csc_iter"], cdl_iter_num=wl["cdl_iter"],
                         track_residuals=bool(args.residuals))
    stream = torch.cuda.current_stream(dev)
    c = pkg.CDL(setup, device=dev, fft_mode=args.fft_mode)
    c.set_stream(stream.cuda_stream)
    # pinned host copy of the inputs for the end-to-end leg
    S_pin_t = torch.empty(S.shape, dtype=torch.float32, pin_memory=True)
    S_pin = S_pin_t.numpy()
    S_pin[...] = S
    c.load_data(S_pin)
    c.init_state(seed=wl["seed"])

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- device-resident leg
    for _ in range(args.warmup):
        pkg.run_outer(c, 1)
    c.profile(True)
    c.profile_read(reset=True)
    sampler = ClockSampler(dev)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        pkg.run_outer(c, 1)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    prof = c.profile_read(reset=True)
    c.profile(False)
    ms_max = max_over_ranks(ms, world, f"cuda:{dev}")
    value = replica_rate(world, args.steps, ms_max / 1e3)

    # ---- end-to-end leg through the C ABI with host buffers
    E = args.e2e_outer
    if args.skip_e2e:
        c.close()
        return dict(value=value, ms=ms_max, clocks=clocks, prof=prof, e2e=None, h2d=0, d2h=0,
                    fused=prof["xfused"][1] > 0)
    for _ in range(max(1, args.warmup // 2)):
        c.load_data(S_pin)
        c.init_state(seed=wl["seed"])
        pkg.run_outer(c, E)
        c.get("D_best")
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_steps = max(2, args.steps // 5)      # one training (E outer iterations) each
    for _ in range(e_steps):
        c.load_data(S_pin)                   # H2D of the step's inputs
        c.init_state(seed=wl["seed"])
        pkg.run_outer(c, E)                  # objectives come back to the host
        Db = c.get("D_best")                 # D2H of the learned filters
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    t_max = max_over_ranks(t_e2e, world, f"cuda:{dev}")
    e2e_value = replica_rate(world, e_steps * E, t_max)
    h2d = S.nbytes
    d2h = Db.nbytes + 8 * E
    fused = bool(c._p.fft_mode != 1) and prof["xfused"][1] > 0
    c.close()
    return dict(value=value, ms=ms_max, clocks=clocks, prof=prof, e2e=e2e_value, h2d=h2d, d2h=d2h,
                fused=fused)


def run_refstruct(args, config):
    """The reference-structured CUDA baseline on the bench workload: wall time per outer
    iteration (the baseline synchronises after every custom kernel, as CUDA.@sync)."""
    sys.path.insert(0, os.path.join(ROOT, "baseline"))
    import refstruct
    pkg = _pkg()
    wl = WORKLOAD
    S = pkg.synth.onehot(dataset())
    Lg = algorithmic_bytes()["Lg"]
    X0 = pkg.synth.init_X0(wl["seed"], wl["N"], wl["M"], Lg)
    D0 = pkg.synth.init_D0_unit_norm(wl["seed"], wl["M"], Lg, 4 * wl["filter_size"])
    steps, warm = max(1, min(args.steps, 3)), 1
    try:
        rs = refstruct.RefStruct(S, X0, D0, wl["M"], wl["filter_size"], wl["rho"], wl["sigma"], wl["lam"])
    except RuntimeError as e:
        return {"impl": "refstruct", "unavailable": str(e)}
    del X0
    with rs:
        rs.run_outer(warm, wl["csc_iter"], wl["cdl_iter"])
        t0 = time.perf_counter()
        rs.run_outer(steps, wl["csc_iter"], wl["cdl_iter"])
        dt = time.perf_counter() - t0
    rate = steps / dt
    return {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": 1, "steps": steps,
            "warmup": warm, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded planted motifs, Dirichlet(0.1) PWMs)", "config": config,
            "impl": "refstruct",
            "note": "reference-structured CUDA baseline (baseline/refstruct.cu): stand-in for the "
                    "reference CUDA.jl path, which cannot run here"}


def measured_hbm_peak() -> float:
    """The measured HBM copy bandwidth (GB/s) of MEASURED_PEAKS.json, else the fallback."""
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except Exception:
        return 6800.0


def roofline(prof, steps, fused, sm_mhz=None):
    """Roofline of the dominant kernel, from the phase timers recorded (CUDA events on
    the launching stream) during the timed region.  For the multi-iteration X-step also
    its issue-rate bound: warp instructions per launch (from the ncu capture, per
    sequence) over the issue slots of the launch (SMs x 4 schedulers x median SM clock x
    launch time)."""
    ab = algorithmic_bytes()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    traffic = None
    note = None
    if fused and prof["xfused"][1] > 0:
        launches = prof["xfused"][1]
        steps_per_launch = max(1, round(prof["xstep"][1] / launches))
        ms_avg = prof["xfused"][0] / launches
        alg = ab["xstep"] * steps_per_launch
        if steps_per_launch > 1:
            kernel = (f"multi-iteration fused X-step k_xiter<32, 29, 288, 1, 16> "
                      f"({steps_per_launch} X-steps per launch, duals on chip)")
            if ab["Lg"] == 928 and WORKLOAD["M"] == 64:
                # dram__bytes_read.sum + dram__bytes_write.sum of one launch (15 X-steps)
                # captured by ncu on 1000 sequences, scaled per sequence
                traffic = int(XITER_DRAM_BYTES_N1000 / 1000 * WORKLOAD["N"])
            note = ("state stays on chip across the X-steps of a launch: DRAM traffic is one "
                    "pass over it, far below the per-X-step algorithmic bytes; the kernel is "
                    "bound by SM issue (FP32 FFT work), not HBM")
        else:
            kernel = "fused X-step kernel (k_xstep_warp<32, 29>, register-resident four-step FFTs)"
            if ab["Lg"] == 928 and WORKLOAD["M"] == 64:
                traffic = int(XWARP_DRAM_BYTES_N1000 / 1000 * WORKLOAD["N"])
    else:
        ms_avg = prof["xstep"][0] / max(prof["xstep"][1], 1)
        alg = ab["xstep"]
        kernel = "X-step (cuFFT path: k_xprep + R2C + k_xsolve + C2R + k_mask_update)"
    achieved = alg / (ms_avg / 1e3) / 1e9
    out = {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": peak,
           "peak_source": peak_src, "unit": "GB/s", "frac": round(achieved / peak, 4),
           "traffic": traffic, "algorithmic_bytes_per_launch": alg,
           "avg_launch_ms": round(ms_avg, 4)}
    if note:
        out["note"] = note
    if fused and prof["xfused"][1] > 0 and steps_per_launch > 1 and ab["Lg"] == 928 \
            and WORKLOAD["M"] == 64:
        mhz = sm_mhz or 2070.0
        instr = XITER_WARP_INSTR_PER_SEQ_XSTEP * WORKLOAD["N"] * steps_per_launch
        slots = N_SM * SCHEDULERS_PER_SM * mhz * 1e6 * (ms_avg / 1e3)
        out["issue"] = {"bound": "sm_issue", "warp_instructions_per_launch": instr,
                        "issue_slots_per_launch": slots, "sm_mhz": mhz,
                        "frac": round(instr / slots, 4),
                        "note": "the kernel's binding roof: one instruction per scheduler and "
                                "cycle; the HBM fraction above counts per-X-step bytes"}
    return out


def serve_requests(n_req: int, seed: int = 77, rate: float = 20.0):
    """The serving workload's request stream: Poisson arrivals (mean `rate`/s),
    N log-uniform in [200, 50000], L uniform in [50, 1000], 1-6 planted Dirichlet(0.1)
    motifs of width 8-20 at 10-40 % occupancy; each request is FASTA text (the server
    pads L to the next FFT-friendly length).  Returns (arrival s, FASTA bytes, N, L)."""
    pkg = _pkg()
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(n_req):
        t += rng.exponential(1.0 / rate)
        N = int(round(np.exp(rng.uniform(np.log(200), np.log(50000)))))
        L = int(rng.integers(50, 1001))
        k = int(rng.integers(1, 7))
        widths = [int(w) for w in rng.integers(8, 21, k)]
        occ = [float(o) for o in rng.uniform(0.1, 0.4, k)]
        bases, _, _ = pkg.synth.plant_dataset(seed * 1000 + i, N, L, widths, occ)
        out.append((t, pkg.synth.to_fasta(bases).encode(), N, L))
    return out


def run_serve(args):
    pkg = _pkg()
    from cdlmotif_gb300 import serve
    reqs = serve_requests(args.serve_requests)
    setup = pkg.CDLSetup(M=32, filter_size=16, lambda_=0.1, rho=1.0, sigma=100.0)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    res = serve.serve_stream(setup, [(t, d) for t, d, *_ in reqs], slots=args.serve_slots,
                             iter_num=args.serve_iters, seed=1, keep_results=False,
                             pad_friendly=True)
    clocks = sampler.stop()
    res.pop("results", None)
    return {"metric": "served datasets/hr (Poisson 20/s, N log-uniform 200-50000, L 50-1000, K=32, W=16)",
            "value": res["datasets_per_hr"], "unit": "datasets/hr", "higher_is_better": True,
            "p50_latency_s": res["p50_s"], "p99_latency_s": res["p99_s"],
            "mean_queue_s": res["mean_queue_s"], "makespan_s": res["makespan_s"],
            "requests": res["requests"], "completed": res["completed"],
            "rejected": res["rejected"], "slots": args.serve_slots,
            "outer_iterations_per_dataset": args.serve_iters, "dtype": "f32",
            "data": "synthetic (seeded planted motifs), FASTA text through cdlgb_server_submit_fasta",
            "clocks": clocks,
            "config": {"workload": "serving", "requests": args.serve_requests,
                       "N": [int(r[2]) for r in reqs], "L": [int(r[3]) for r in reqs]}}


def batched_requests(n: int = 64, seed: int = 91):
    """The batched workload: n datasets, N log-uniform in [500, 20000], L in {100, 200, 500},
    1-5 planted Dirichlet(0.1) motifs of width 8-20 at 10-40 % occupancy (K = 32, W = 16)."""
    pkg = _pkg()
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        N = int(round(np.exp(rng.uniform(np.log(500), np.log(20000)))))
        L = int(rng.choice([100, 200, 500]))
        k = int(rng.integers(1, 6))
        widths = [int(w) for w in rng.integers(8, 21, k)]
        occ = [float(o) for o in rng.uniform(0.1, 0.4, k)]
        bases, _, _ = pkg.synth.plant_dataset(seed * 1000 + i, N, L, widths, occ)
        out.append(pkg.synth.onehot(bases))
    return out


def run_batched(args):
    """The 64-dataset mix processed plainly (one training after another, each alone on
    the GPU) and batched (all submitted at once to the library's training server, up to
    `serve_slots` trainings in flight); datasets/hr of both, how busy the GPU was in the
    plain form (the sum of every training's device time -- data upload, initialisation,
    X-steps, D-steps, objectives, code threshold -- from the library's CUDA-event
    phase timers against the wall clock, and nvidia-smi's utilisation), and the largest
    difference between a dataset's D_best alone and in the mix (the kernels are
    deterministic and contexts share nothing, so it should be 0)."""
    pkg = _pkg()
    from cdlmotif_gb300 import serve
    data = batched_requests(args.batched_n)
    setup = pkg.CDLSetup(M=32, filter_size=16, lambda_=0.1, rho=1.0, sigma=100.0)
    iters = args.serve_iters
    serve.run_training(setup, data[0], iters, 1, 0)          # warm-up (plans, kernels)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    sampler = ClockSampler(dev)
    sampler.start()
    t0 = time.perf_counter()
    alone = [serve.run_training(setup, d, iters, 1, 0, profile=True) for d in data]
    t_plain = time.perf_counter() - t0
    clocks_plain = sampler.stop()
    busy_ms = sum(a["device_ms"] for a in alone)
    sampler = ClockSampler(dev)
    sampler.start()
    res = serve.serve_stream(setup, [(0.0, d) for d in data], slots=args.serve_slots,
                             iter_num=iters, seed=1)
    clocks = sampler.stop()
    mix = res.pop("results")
    diff = max(float(np.max(np.abs(mix[i]["D_best"] - alone[i]["D_best"]))) for i in mix)
    plain_rate = 3600.0 * len(data) / t_plain
    busy = busy_ms / 1e3 / t_plain
    return {"metric": "datasets/hr, 64-dataset mix (N log-uniform 500-20000, L in {100,200,500}, K=32, W=16)",
            "value": res["datasets_per_hr"], "unit": "datasets/hr", "higher_is_better": True,
            "plain_datasets_per_hr": plain_rate, "batched_over_plain": res["datasets_per_hr"] / plain_rate,
            "plain_seconds": t_plain, "batched_makespan_s": res["makespan_s"],
            "plain_kernel_seconds": busy_ms / 1e3, "plain_busy_fraction": busy,
            "plain_idle_fraction": 1.0 - busy,
            "batching_bound_if_idle_removed": 1.0 / busy if busy > 0 else None,
            "batched_fraction_of_bound": (res["datasets_per_hr"] / plain_rate) * busy,
            "completed": res["completed"], "rejected": res["rejected"], "slots": args.serve_slots,
            "outer_iterations_per_dataset": iters, "max_abs_diff_D_best_alone_vs_mix": diff,
            "dtype": "f32", "data": "synthetic (seeded planted motifs)",
            "clocks_plain": clocks_plain, "clocks": clocks,
            "config": {"workload": "batched64", "N": [int(d.shape[0]) for d in data],
                       "L": [int(d.shape[1] // 4) for d in data]}}


def run_interference(args, n_small: int = 5):
    """What one dataset's life (cdlgb_create, load, init, 3 outer iterations, code
    threshold, destroy) costs a training that runs beside it in the same process: an
    N = 20000 training (L = 200, K = 32, W = 16) loops outer iterations on one host
    thread while N = 1000 datasets (same L, K, W) are trained one after another on
    another.  Reported: the big training's ms per outer iteration alone and during,
    the GPU time it loses per small dataset (the outer iterations it would have done
    alone in that wall time, minus those it did, times its ms per iteration), and the
    small datasets' median call times alone and beside it.  A loss near the small
    dataset's own kernel time means its set-up and teardown stalled nothing."""
    import threading
    pkg = _pkg()
    setup = pkg.CDLSetup(M=32, filter_size=16, lambda_=0.1, rho=1.0, sigma=100.0)
    big = pkg.synth.onehot(pkg.synth.plant_dataset(71, 20000, 200, [10, 14], [0.3, 0.3])[0])
    small = pkg.synth.onehot(pkg.synth.plant_dataset(72, 1000, 200, [10, 14], [0.3, 0.3])[0])

    def one():
        t = {}
        t0 = time.perf_counter()
        c = pkg.CDL(setup)
        t["create"] = time.perf_counter() - t0
        t0 = time.perf_counter(); c.load_data(small); t["load"] = time.perf_counter() - t0
        t0 = time.perf_counter(); c.init_state(seed=3); t["init"] = time.perf_counter() - t0
        t0 = time.perf_counter(); pkg.run_outer(c, 3); t["outer3"] = time.perf_counter() - t0
        t0 = time.perf_counter(); pkg.code_threshold(c); t["threshold"] = time.perf_counter() - t0
        t0 = time.perf_counter(); c.close(); t["destroy"] = time.perf_counter() - t0
        return t

    def med(ts):
        return {k: 1e3 * float(np.median([t[k] for t in ts])) for k in ts[0]}

    one()                                             # warm-up (modules, tables)
    alone = med([one() for _ in range(n_small)])
    stop = threading.Event()
    done = [0]

    def background():
        with pkg.init_cdl(setup, big) as c:
            while not stop.is_set():
                pkg.run_outer(c, 1)
                done[0] += 1

    th = threading.Thread(target=background)
    th.start()
    try:
        time.sleep(3.0)
        d0, t0 = done[0], time.perf_counter()
        time.sleep(2.0)
        big_alone_ms = 1e3 * (time.perf_counter() - t0) / max(1, done[0] - d0)
        d0, t0 = done[0], time.perf_counter()
        beside = [one() for _ in range(n_small)]
        el = time.perf_counter() - t0
        got = done[0] - d0
    finally:
        stop.set()
        th.join()
    lost = (1e3 * el / big_alone_ms - got) * big_alone_ms / n_small
    return {"metric": "GPU time a running N=20000 training loses per N=1000 dataset trained beside it",
            "value": lost, "unit": "ms", "higher_is_better": False,
            "big_ms_per_outer_alone": big_alone_ms, "big_ms_per_outer_beside": 1e3 * el / max(1, got),
            "small_calls_ms_alone": alone, "small_calls_ms_beside": med(beside),
            "small_datasets": n_small, "dtype": "f32", "data": "synthetic (seeded planted motifs)",
            "config": {"workload": "interference", "big": {"N": 20000, "L": 200, "K": 32},
                       "small": {"N": 1000, "L": 200, "K": 32, "outer_iterations": 3}}}


def run_lengths(args, shapes=((100, 16), (200, 16), (500, 16), (200, 4)), N: int = 5000, K: int = 32,
                outer: int = 3):
    """Per transform length: the batched mix's lengths (L = 100, 200, 500 with W = 16:
    Lg = 528, 928, 2128) and L = 200 at the reference's default W = 4 (Lg = 832) on
    N = 5000 sequences with K = 32 filters, `outer` timed outer
    iterations after one untimed: outer iterations/s, the X-step and D-step device time
    per outer iteration from the library's phase timers, and the kernel path each length
    takes (register-FFT lengths run the multi-iteration X-step and the spectral D-step
    on the register-FFT transforms; the others the generic in-kernel FFT X-step).  The
    X-step's and D-step's algorithmic bytes over their time give each one's HBM rate."""
    import torch
    pkg = _pkg()
    peak = measured_hbm_peak()
    out = []
    for shape in shapes:
        L, W = shape[0], shape[1]
        Kx = shape[2] if len(shape) > 2 else K
        wl = dict(WORKLOAD, N=N, L=L, M=Kx, filter_size=W, name=f"len_n{N}_l{L}_w{W}_k{Kx}")
        S = pkg.synth.onehot(dataset(wl))
        setup = pkg.CDLSetup(M=Kx, filter_size=wl["filter_size"], lambda_=wl["lam"], rho=wl["rho"],
                             sigma=wl["sigma"])
        ab = algorithmic_bytes(wl)
        with pkg.init_cdl(setup, S, seed=wl["seed"]) as c:
            pkg.run_outer(c, 1)
            c.profile(True)
            c.profile_read(reset=True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pkg.run_outer(c, outer)
            torch.cuda.synchronize()
            sec = time.perf_counter() - t0
            pr = c.profile_read()
            xs, ds = pr["xstep"][0] / outer, pr["dstep"][0] / outer
            out.append({"L": L, "W": W, "Lg": ab["Lg"], "N": N, "K": Kx, "outer_iter_per_s": outer / sec,
                        "xstep_ms_per_outer": xs, "dstep_ms_per_outer": ds,
                        "objective_ms_per_outer": pr["objective"][0] / outer,
                        "xstep_frac_of_hbm_peak": (15 * ab["xstep"] / (xs / 1e3)) / (peak * 1e9) if xs else None,
                        "dstep_frac_of_hbm_peak": (ab["dstep"] / (ds / 1e3)) / (peak * 1e9) if ds else None,
                        "fused_xstep_launches_per_outer": pr["xfused"][1] / outer,
                        "cufft_exec_per_outer": pr["fft_calls"] / outer})
    return {"metric": "outer iterations/s per transform length (N=5000, K=32, W=16)",
            "value": None, "unit": "outer_iter/s", "lengths": out, "hbm_peak_gbs": peak,
            "dtype": "f32", "data": "synthetic (seeded planted motifs)",
            "config": {"workload": "lengths", "L_W": [list(x) for x in shapes], "N": N, "K": K}}


def search_inputs(wl=WORKLOAD, K=32, N=None):
    """The search-stage inputs on the bench dataset: the planted motifs' cores (two
    columns trimmed per side, so that extend! has columns to find) and random
    Dirichlet(1) PWMs of widths 8..16, K in all."""
    pkg = _pkg()
    n = wl["N"] if N is None else N
    bases, motifs, _ = pkg.synth.plant_dataset(wl["seed"], n, wl["L"], wl["widths"], wl["occ"])
    pwms = []
    for m in motifs:
        core = m[:, 2:-2]
        pwms.append(np.log2(((core + 0.05) / 1.2) / 0.25).astype(np.float32))
    rng = np.random.default_rng(17)
    while len(pwms) < K:
        w = int(rng.integers(8, 17))
        pfm = rng.dirichlet(np.ones(4), size=w).T
        pwms.append(np.log2(((pfm + 0.02) / 1.08) / 0.25).astype(np.float32))
    return bases, pwms


def search_round(pkg, c, pwms, thresh, filter_size=4, times=None):
    """One round of find_motif's refinement loop (src/WRAPPER/wrap.jl:88-98) through
    the package: overlapping_scan!, non_overlap_scan!, extend! (extension + PFMs),
    masked_trim! (trim + PWMs + Touzet thresholds)."""
    def tick(name, t0):
        if times is not None:
            times[name] = times.get(name, 0.0) + time.perf_counter() - t0
        return time.perf_counter()
    lens = np.array([p.shape[1] for p in pwms], np.int32)
    t = time.perf_counter()
    pos, sc, uc = pkg.overlapping_scan(c, pwms, thresh)
    t = tick("overlapping_scan", t)
    pos, sc, uc = pkg.non_overlap_scan(c, pos, sc, lens, uc)
    t = tick("non_overlap_scan", t)
    ext = pkg.extend(c, pos, lens, filter_size, use_comp=uc, smoothing=False)
    t = tick("extend", t)
    out = pkg.masked_trim(ext["pfms"], filter_size, ext["positions"], ext["use_comp"], c=c)
    tick("masked_trim", t)
    return out


def run_search(args):
    """Motif-search stage on the bench dataset (N = 20000, L = 200): search rounds/s
    through the package's public calls (host arrays in and out, as a caller sees them),
    per-call times, the one-off background shuffle and e-value filter, and the oracle
    on a sample of sequences as the CPU figure."""
    pkg = _pkg()
    wl = WORKLOAD
    K = args.search_k
    bases, pwms = search_inputs(wl, K)
    S = pkg.synth.onehot(bases)
    c = pkg.CDL(pkg.CDLSetup(M=2, filter_size=2))
    c.load_data(S)
    thresh = pkg.get_thresh(c, pwms)
    for _ in range(args.warmup):
        search_round(pkg, c, pwms, thresh)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    times = {}
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = search_round(pkg, c, pwms, thresh, times=times)
    dt = time.perf_counter() - t0
    clocks = sampler.stop()
    t1 = time.perf_counter()
    c.make_background(k=3, seed=1)
    t_bg = time.perf_counter() - t1
    lens = np.array([p.shape[1] for p in pwms], np.int32)
    pos, _, _ = pkg.overlapping_scan(c, pwms, thresh)
    t1 = time.perf_counter()
    ev = pkg.filter_using_evalue(c, pwms, thresh, pos, cpu=True, non_overlap=True)
    t_ev = time.perf_counter() - t1
    c.close()
    res = {"metric": f"motif search rounds/s at N={wl['N']}, L={wl['L']}, K={K} (overlapping_scan! + "
                     "non_overlap_scan! + extend! + masked_trim! with thresholds)",
           "value": args.steps / dt, "unit": "round/s", "higher_is_better": True,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
           "phases_ms_per_step": {k: 1e3 * v / args.steps for k, v in times.items()},
           "motifs_after_round": int(len(out["pfms"])),
           "background_k3_ms": 1e3 * t_bg, "evalue_filter_ms": 1e3 * t_ev,
           "evalue_filter_kept": int(ev["keep"].sum()),
           "dtype": "f32 scores / int32 counts", "data": "synthetic (seeded planted motifs)",
           "clocks": clocks,
           "config": {"workload": f"search_n{wl['N']}_l{wl['L']}_k{K}", "N": wl["N"], "L": wl["L"],
                      "K": K, "filter_size_for_length_filters": 4,
                      "timing": "wall clock around host-array calls (each call returns its results)"}}
    if not args.no_cpu:
        res["cpu_baseline"] = search_cpu_baseline(S, pwms, thresh, args.search_cpu_n)
    return res


def search_cpu_baseline(S, pwms, thresh, n_sample):
    """The oracle's scans, non-overlap selection, extension and counts on the first
    n_sample sequences, scaled to N (thresholds, trims and PFMs are per motif, left out)."""
    from oracle import search_oracle as SO
    lens = np.array([p.shape[1] for p in pwms], np.int32)
    Ss = S[:n_sample]
    t0 = time.perf_counter()
    rp, rs, rc = SO.overlapping_scan(Ss, pwms, lens, thresh)
    pos, sc, uc = SO.non_overlap_select(rp.T, rs.T, rc.T, lens)
    npos, nl, _, _ = SO.extend_positions(Ss, pos, uc, lens)
    SO.count_matrices(Ss, npos.T, uc.T, nl)
    dt = time.perf_counter() - t0
    return {"value": (n_sample / S.shape[0]) / dt, "unit": "round/s", "cores": 1, "kind": "port",
            "sample": f"{n_sample} of {S.shape[0]} sequences, one round, NumPy/Python oracle; "
                      "rate scaled by N"}


def run_precision(args):
    """Precision study on the N = 20000, L = 200, K = 64 workload: from one initial state,
    the float32 CUDA path, the reference's statement order evaluated in float32 (torch,
    full complex FFTs: the drift FP32 rounding alone causes in the reference) and an
    all-FP64 reference (torch, half-spectrum form) are run outer iteration by outer
    iteration; at each checkpoint the relative L2 distance of X, X_best, d, D_best, G1 and
    the objective from FP64 is reported for both float32 runs, with the float32 path's
    residual norms beside the FP64 ones."""
    import torch
    pkg = _pkg()
    from oracle.torch_admm import FP64Reference, LiteralADMM, relative_residuals
    wl = dict(WORKLOAD)
    if args.precision_reference_defaults:
        # the reference's own CDL_setup defaults (src/SETUP/WRAPPER_setup.jl:3-5)
        wl.update(lam=0.01, rho=100.0, sigma=100.0)
    bases = dataset(wl)
    S = pkg.synth.onehot(bases)
    setup = pkg.CDLSetup(M=wl["M"], filter_size=wl["filter_size"], lambda_=wl["lam"], rho=wl["rho"],
                         sigma=wl["sigma"], csc_iter_num=wl["csc_iter"], cdl_iter_num=wl["cdl_iter"])
    c = pkg.init_cdl(setup, S, seed=wl["seed"])
    dev = "cuda:0"
    chunk = 512

    def rel(a, b64):
        """relative L2 distance of a (numpy float32 or torch) from the float64 tensor b64,
        summed in float64 over chunks of the first axis"""
        num = den = 0.0
        for i0 in range(0, b64.shape[0], chunk):
            i1 = min(b64.shape[0], i0 + chunk)
            x = a[i0:i1]
            x = (torch.from_numpy(np.ascontiguousarray(x)) if isinstance(x, np.ndarray) else x)
            x = x.to(dev, torch.float64)
            num += float(((x - b64[i0:i1]) ** 2).sum())
            den += float((b64[i0:i1] ** 2).sum())
        return (num / den) ** 0.5

    X0, D0 = c.X, c.G1
    ref = FP64Reference(S, X0, D0, wl["M"], wl["filter_size"], wl["rho"], wl["sigma"], wl["lam"],
                        device=dev, chunk=chunk)
    lit = LiteralADMM(S, X0, D0, wl["M"], wl["filter_size"], wl["rho"], wl["sigma"], wl["lam"],
                      device=dev, chunk=chunk, dtype=torch.float32)
    del X0
    at = sorted({int(v) for v in args.precision_at.split(",") if v})
    rows = []
    secs = {"f32_cuda": 0.0, "f32_reference_order": 0.0, "f64": 0.0}
    first_nonfinite = {"f32_cuda": None, "f32_reference_order": None, "f64": None}
    objectives = {"f32_cuda": [], "f32_reference_order": [], "f64": []}
    for it in range(1, at[-1] + 1):
        t0 = time.perf_counter()
        o32 = float(pkg.run_outer(c, 1)[0])
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ol = lit.run_outer(1)[0]
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        o64 = ref.run_outer(1)[0]
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        secs["f32_cuda"] += t1 - t0
        secs["f32_reference_order"] += t2 - t1
        secs["f64"] += t3 - t2
        for k, o in (("f32_cuda", o32), ("f32_reference_order", ol), ("f64", o64)):
            objectives[k].append(o)
            if first_nonfinite[k] is None and not np.isfinite(o):
                first_nonfinite[k] = it
        if it not in at:
            continue
        row = {"outer_iteration": it, "objective_f64": o64,
               "cuda_f32": {"objective_rel_gap": abs(o32 - o64) / abs(o64),
                            "X": rel(c.X, ref.X), "X_best": rel(c.X_best, ref.X_best),
                            "d": rel(c.d, ref.d), "D_best": rel(c.D_best, ref.D_best),
                            "G1": rel(c.G1, ref.G1)},
               "reference_order_f32": {"objective_rel_gap": abs(ol - o64) / abs(o64),
                                       "X": rel(lit.X, ref.X), "X_best": rel(lit.X_best, ref.X_best),
                                       "d": rel(lit.d, ref.d), "D_best": rel(lit.D_best, ref.D_best),
                                       "G1": rel(lit.G1, ref.G1)},
               "relative_residuals_f64": relative_residuals(ref.resid)}
        if hasattr(c, "residuals"):
            row["relative_residuals_cuda_f32"] = relative_residuals(c.residuals())
        rows.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    c.close()
    return {"metric": "precision: float32 CUDA path and float32 reference order vs all-FP64",
            "workload": wl["name"], "N": wl["N"], "lambda": wl["lam"], "rho": wl["rho"],
            "sigma": wl["sigma"], "rows": rows, "seconds": secs,
            "first_nonfinite_objective": first_nonfinite, "objectives": objectives,
            "note": "same initial state for all three; float64 objective and residual sums; "
                    "FP64 = torch float64 cuFFT (half-spectrum form); reference order = "
                    "src/CDL/train.jl statement by statement in torch float32, c2c FFTs"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference", "refstruct"])
    ap.add_argument("--fft-mode", type=int, default=0, help="0 auto, 1 cuFFT, 2 fused")
    ap.add_argument("--e2e-outer", type=int, default=10,
                    help="outer iterations per end-to-end step (one training: iter_num)")
    ap.add_argument("--cpu-sample", type=int, default=1000,
                    help="sequences of the CPU baseline leg (one outer iteration)")
    ap.add_argument("--ref-sample", type=int, default=2000,
                    help="sequences per step of --impl reference")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=0, help="override N (small cases for profiling)")
    ap.add_argument("--residuals", action="store_true",
                    help="keep the FP64 residual record every outer iteration (track_residuals)")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--serve", action="store_true",
                    help="serving workload: Poisson request stream, datasets/hr and p50/p99")
    ap.add_argument("--serve-requests", type=int, default=500)
    ap.add_argument("--serve-iters", type=int, default=3)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--batched", action="store_true",
                    help="64-dataset mix: plain (one at a time) vs batched (served) datasets/hr")
    ap.add_argument("--batched-n", type=int, default=64)
    ap.add_argument("--lengths", action="store_true",
                    help="outer iterations/s and phase times at the batched mix's transform lengths")
    ap.add_argument("--length-shapes", default="100:16,200:16,500:16,200:4",
                    help="L:W (or L:W:K) for --lengths")
    ap.add_argument("--interference", action="store_true",
                    help="GPU time a running training loses per dataset trained beside it")
    ap.add_argument("--precision", action="store_true",
                    help="precision study: float32 GPU path vs an all-FP64 GPU reference")
    ap.add_argument("--precision-reference-defaults", action="store_true",
                    help="precision study with the reference's CDL_setup defaults (lambda 0.01, rho 100)")
    ap.add_argument("--precision-at", default="1,3,10,100",
                    help="outer iterations at which the precision study reports")
    ap.add_argument("--search", action="store_true",
                    help="motif-search stage: scans, non-overlap selection, extension, trim")
    ap.add_argument("--search-k", type=int, default=32)
    ap.add_argument("--search-cpu-n", type=int, default=2000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.n:
        WORKLOAD["N"] = args.n
        WORKLOAD["name"] = f"plain_n{args.n}_l{WORKLOAD['L']}_k{WORKLOAD['M']}"
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    wl = WORKLOAD
    config = {"workload": wl["name"], "N": wl["N"], "L": wl["L"], "K": wl["M"],
              "filter_size": wl["filter_size"], "Lg": algorithmic_bytes()["Lg"], "lambda": wl["lam"],
              "rho": wl["rho"], "sigma": wl["sigma"], "csc_iter_num": wl["csc_iter"],
              "cdl_iter_num": wl["cdl_iter"], "parallelism": f"replicas{world}",
              "l2": "inputs larger than L2 (ADMM state ~28 GB per replica)",
              "residual_record": bool(args.residuals)}

    if args.serve:
        if rank == 0:
            print(json.dumps(run_serve(args)))
        return
    if args.search:
        if rank == 0:
            print(json.dumps(run_search(args)))
        return
    if args.precision:
        if rank == 0:
            print(json.dumps(run_precision(args)))
        return
    if args.batched:
        if rank == 0:
            print(json.dumps(run_batched(args)))
        return
    if args.lengths:
        if rank == 0:
            shapes = tuple(tuple(int(v) for v in x.split(":")) for x in args.length_shapes.split(","))
            print(json.dumps(run_lengths(args, shapes=shapes)))
        return
    if args.interference:
        if rank == 0:
            print(json.dumps(run_interference(args)))
        return

    if args.impl == "reference":
        if world > 1 and rank != 0:
            return
        rate, ms, nt, sample = cpu_reference(args.steps, args.warmup, args.ref_sample)
        line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded planted motifs)", "config": config, "impl": "reference",
                "note": "ms_per_step is the measured time of one step on the sample; value is "
                        "scaled to the full N by the extrapolation factor in cpu_baseline.sample",
                "cpu_baseline": {"value": rate, "unit": UNIT, "cores": nt, "kind": "port",
                                 "sample": sample, "sample_ms_per_step": ms},
                "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.impl == "refstruct":
        if world > 1 and rank != 0:
            return
        print(json.dumps(run_refstruct(args, config)))
        return

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # the CPU baseline runs before any GPU call, single process, bounded sample
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, ms, nt, sample = cpu_reference(1, 0, args.cpu_sample)
        cpu = {"value": rate, "unit": UNIT, "cores": nt, "kind": "port", "sample": sample}
    r = run_gpu(args, rank, world)
    if rank != 0:
        return
    prof = r["prof"]
    launches = prof["launches"]
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded planted motifs, Dirichlet(0.1) PWMs)", "config": config,
            "clocks": r["clocks"],
            "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"], "outer_iterations_per_step": args.e2e_outer},
            "gpu_launches": launches,
            "library_calls": {"cufft_exec": prof["fft_calls"]},
            "roofline": roofline(prof, args.steps, r["fused"], (r["clocks"] or {}).get("sm_mhz")),
            "phases_ms_per_step": {k: round(v[0] / args.steps, 3) for k, v in prof.items()
                                   if isinstance(v, tuple) and v[1]},
            "path": "fused" if r["fused"] else "cufft",
            "cpu_baseline": cpu}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
