"""Benchmark of the projector-DQMC sweep on GB300.

Workload: 256 independent Markov chains of the spinless t-V model on the
6x6 honeycomb lattice (N = 72 sites, V/t = 1, dt = 0.05, 2Θ = 20 -> 400
slices, n_wrap = 10), FP64 throughout, energy and density structure factor
measured every sweep.  One step = one forward+backward sweep of every chain.

Metric: effective samples/s = (chain-sweeps/s) / τ_int(E_kin), summed over
all GPUs.  τ_int is estimated (Sokal window) from the measured energy series
of the timed sweeps, pooled over the chains.

  value   device-resident: fields and B chains live in HBM, one kdq_sweep
          per step, timed with CUDA events on the library's stream
  e2e     through the reference-shaped C-ABI call kdq_phy_update with host
          buffers: fields uploaded, chain rebuilt, one sweep, fields and
          measurement rows read back, every step

`--impl reference` times the CPU restatement of the reference algorithm (the
oracle) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "eff. samples/s (sweeps/s÷τ_int) vs plain FP64 DQMC, 1 GB300, obs within 1σ"
UNIT = "chain-sweeps/s / tau_int"
NCHAINS = 256
RECORD = 2   # measurements as the reference's estimator, wraps folded into two products (kdq_phy_update)
TAU_FILE = ROOT / "profiles" / "tau_int_tv_honeycomb_6x6.json"


def reference_tau_int():
    """τ_int of the plain local-update sweep on this workload, from a long
    committed GPU run (both arms run the same Markov chain algorithm)."""
    try:
        return float(json.loads(TAU_FILE.read_text())["tau_int"])
    except Exception:
        return None


def _tu_4x4():
    from kapdqmc_gb300 import tU_Hubbard_Para
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.1, Θrelax=5.0, Θquench=0.0,
                           Lattice="SQUARE45", site=[2, 4], BatchSize=10, Initial="H0")


def _tv_6x6():
    from kapdqmc_gb300 import tV_Hubbard_Para
    return tV_Hubbard_Para(Ht=1.0, Hv1=1.0, Hv2=1.0, Δt=0.05, Θrelax=10.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[6, 6], BatchSize=10, Initial="H0")


def _tu_12x12():
    from kapdqmc_gb300 import tU_Hubbard_Para
    return tU_Hubbard_Para(Ht=1.0, Hu1=8.0, Hu2=8.0, Δt=0.05, Θrelax=8.0, Θquench=0.0,
                           Lattice="SQUARE45", site=[6, 12], BatchSize=8, Initial="H0")


def _tuv_8x8():
    from kapdqmc_gb300 import tUV_Hubbard_Para
    return tUV_Hubbard_Para(Ht=1.0, Hu=4.0, Hv=0.5, Lattice="SQUARE45", site=[4, 8], Δt=0.1, Θ=10.0,
                            BatchSize=10, Initial="H0", allow_marginal=True)


def _tu_hc_9x9():
    from kapdqmc_gb300 import tU_Hubbard_Para
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.1, Θrelax=10.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[9, 9], BatchSize=10, Initial="H0")


# The bench line is c2 (the metric's configuration: batched plain FP64 sweep);
# the others are the remaining single-GPU configurations, for `--workload`.
WORKLOADS = {
    "c1": dict(make=_tu_4x4, chains=1, Ns=16, Nt=100, n_wrap=10,
               desc="t-U 4x4 square (N=16), 100 slices, n_wrap=10, U/t=4, dt=0.1, one chain, "
                    "energy + double occupancy per sweep",
               model="tU_Hubbard_Para(SQUARE45, site=[2,4])"),
    "c2": dict(make=_tv_6x6, chains=256, Ns=72, Nt=400, n_wrap=10,
               desc="t-V 6x6 honeycomb (N=72), 400 slices, n_wrap=10, V/t=1, dt=0.05, 256 independent "
                    "chains, energy + density structure factor per sweep",
               model="tV_Hubbard_Para(HoneyComb120, site=[6,6])"),
    "c3": dict(make=_tu_12x12, chains=128, Ns=144, Nt=320, n_wrap=8,
               desc="t-U 12x12 square (N=144), 320 slices, n_wrap=8, U/t=8, dt=0.05, 128 independent "
                    "chains, energy + double occupancy per sweep",
               model="tU_Hubbard_Para(SQUARE45, site=[6,12])"),
    "c4": dict(make=_tuv_8x8, chains=256, Ns=64, Nt=200, n_wrap=10,
               desc="t-UV 8x8 square (N=64), 200 slices, n_wrap=10, U/t=4, V/t=0.5, dt=0.1, 256 chains "
                    "(128 replica pairs), energies per sweep",
               model="tUV_Hubbard_Para(SQUARE45, site=[4,8], allow_marginal=True)"),
    "c5": dict(make=_tu_hc_9x9, chains=256, Ns=162, Nt=200, n_wrap=10,
               desc="t-U 9x9 honeycomb (N=162), 200 slices, n_wrap=10, U/t=4, dt=0.1, 256 chains, "
                    "energy, double occupancy and structure factors per sweep",
               model="tU_Hubbard_Para(HoneyComb120, site=[9,9])"),
}
WL = WORKLOADS["c2"]
PRECISION = "fp64"


def make_model():
    return WL["make"]()


def config():
    return {"workload": WL["desc"] + f", {PRECISION}", "model": WL["model"], "chains_per_gpu": NCHAINS,
            "Ns": WL["Ns"], "Nt": WL["Nt"], "n_wrap": WL["n_wrap"], "precision": PRECISION,
            "l2": "no flush: per-GPU chain state (B chains, fields, G) is larger than the 129 MB L2"}


def tau_int(series: np.ndarray, c: float = 5.0):
    """Integrated autocorrelation time of (chains, T) series, Sokal window."""
    x = np.asarray(series, dtype=np.float64)
    x = x - x.mean()
    T = x.shape[1]
    var = np.mean(x * x)
    if var <= 0 or T < 3:
        return 0.5
    tau = 0.5
    for t in range(1, T - 1):
        rho = np.mean(x[:, :-t] * x[:, t:]) / var
        tau += rho
        if t >= c * tau:
            break
    return max(tau, 0.5)


def clocks_start(path):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        return subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                 "-lms", "200"], stdout=f, stderr=subprocess.DEVNULL), f
    except OSError:
        return None, None


def clocks_stop(proc, f, path, device):
    if proc is None:
        return None
    proc.terminate()
    proc.wait()
    f.close()
    sm, mx, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        p = [v.strip() for v in line.split(",")]
        if len(p) < 9 or p[0] != str(device):
            continue
        try:
            sm.append(float(p[1]))
            mx = max(mx, float(p[2]))
        except ValueError:
            continue
        for n, v in zip(names, p[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
            "samples": len(sm)}


def fp64_peak_tflops(torch, dev):
    """Measured FP64 ceiling: cuBLAS DGEMM 4096^3, best of 5 (CUDA events)."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * 4096 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def traffic_per_launch():
    """DRAM bytes (read + write) per sweep-kernel launch from the committed ncu capture."""
    try:
        return float(json.loads((ROOT / "profiles" / "k_block_tv6x6_traffic.json").read_text())
                     ["dram_bytes_per_launch"])
    except Exception:
        return None


def hbm_peak_gbs():
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except Exception:
        return 6800.0


# ---------------------------------------------------------------- CPU arm
def _cpu_worker(args):
    """One chain of the workload through the C restatement of the reference sweep."""
    seed, chain, sweeps = args
    sys.path.insert(0, str(ROOT / "oracle"))
    import cport
    if sweeps == 0:                       # warm-up: load the library only
        cport.load()
        return 0.0
    import dqmc_oracle as O
    import philox
    from kapdqmc_gb300 import Initial_s
    model = make_model()
    s = Initial_s(model, 1000 + chain)
    n = O.proposals_per_sweep(model)
    ks, us = zip(*(philox.tape(seed, chain, w, n) for w in range(sweeps)))
    cport.load()
    t0 = time.perf_counter()
    cport.tv_phy_update(model, s, sweeps, np.concatenate(ks), np.concatenate(us), record=True)
    return time.perf_counter() - t0


CPU_KIND = "port"
CPU_SWEEPS = 10          # per chain in the GPU arm's cpu_baseline sample (about 10 s of CPU work)
CPU_SAMPLE = ("C restatement of the reference t-V sweep (dense bond-rotation GEMMs as the reference; "
              "OpenBLAS/LAPACK from numpy, 1 thread each), one chain per host core")


class CpuArm:
    """The reference algorithm on the host cores: one chain per core, all busy."""

    def __init__(self, cores: int):
        import multiprocessing as mp
        sys.path.insert(0, str(ROOT / "oracle"))
        import cport
        cport.build()
        self.cores = cores
        saved = {v: os.environ.get(v) for v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
        for v in saved:                     # inherited by the workers before numpy loads
            os.environ[v] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(cores)
        finally:
            for v, x in saved.items():
                if x is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = x
        self.pool.map(_cpu_worker, [(7, c, 0) for c in range(cores)])      # load in every worker
        self.calls = 0

    def step(self, sweeps_per_chain: int = 1) -> float:
        """Wall time of sweeps_per_chain sweeps of `cores` chains run concurrently."""
        self.calls += 1
        t0 = time.perf_counter()
        self.pool.map(_cpu_worker, [(7 + self.calls, c, sweeps_per_chain) for c in range(self.cores)])
        return time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_chain_sweeps_per_s(cores: int, sweeps_per_chain: int = 1):
    arm = CpuArm(cores)
    try:
        wall = arm.step(sweeps_per_chain)
    finally:
        arm.close()
    return cores * sweeps_per_chain / wall, wall


def run_tau(args):
    """Long run of the plain sweep: τ_int(E_kin) with a binning cross-check.

    Prints the JSON that is committed as the workload's τ_int (both bench arms
    run the same Markov chain algorithm, so they share it)."""
    from kapdqmc_gb300 import Initial_s
    from kapdqmc_gb300.sweep import Sweeper
    model = make_model()
    sw = Sweeper(model, NCHAINS)
    sw.set_precision(PRECISION)
    sw.set_fields(np.stack([Initial_s(model, 5000 + c) for c in range(NCHAINS)]))
    sw.set_rng(424242)
    sw.init()
    burn = 20
    sw.sweep(burn + args.tau_run, record=RECORD)
    sw.synchronize()
    ek = sw.get_obs(burn + args.tau_run)[:, burn:, 0]
    tau = tau_int(ek)
    # binning: τ_int ≈ var(bin means) * B / (2 var)
    var = ek.var()
    bins = {}
    for B in (1, 2, 4, 8, 16):
        T = ek.shape[1] // B
        m = ek[:, :T * B].reshape(ek.shape[0], T, B).mean(axis=2)
        bins[B] = float(m.var() * B / (2 * var))
    out = {"workload": config()["workload"], "chains": NCHAINS, "sweeps": args.tau_run, "burn_in": burn,
           "observable": "kinetic energy (first measurement column)", "estimator": "Sokal window c=5",
           "tau_int": tau, "tau_int_binning": bins, "energy_mean": float(ek.mean()),
           "energy_err": float(ek.mean(axis=1).std() / math.sqrt(NCHAINS))}
    print(json.dumps(out))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    arm = CpuArm(cores)
    try:
        for _ in range(args.warmup):
            arm.step(1)
        walls = [arm.step(1) for _ in range(max(args.steps, 1))]
    finally:
        arm.close()
    cs = cores * len(walls) / sum(walls)
    tau = args.tau_int or reference_tau_int() or 1.0
    value = cs / tau
    sample = (f"{CPU_SAMPLE}; {cores} chains x 1 sweep per step; tau_int={tau:.3g} "
              f"(the workload's committed long-run value)")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": float(np.mean(walls)) * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded HS fields and Philox proposal stream)", "config": config(),
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": CPU_KIND, "sample": sample,
                            "chain_sweeps_per_s": cs},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ---------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch
    from kapdqmc_gb300 import Initial_s
    from kapdqmc_gb300.flops import sweep_flops
    from kapdqmc_gb300.sweep import Sweeper

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    model = make_model()
    sw = Sweeper(model, NCHAINS, device=local)
    sw.set_precision(PRECISION)
    fields = np.stack([Initial_s(model, 1000 + NCHAINS * rank + c) for c in range(NCHAINS)])
    seed = 20261203 + rank
    stream = torch.cuda.ExternalStream(sw.stream, device=dev)

    # ---- device-resident throughput
    sw.set_fields(fields)
    sw.set_rng(seed)
    # tile class: one timed sweep per class that covers the lattice (fields
    # and random-stream positions restored; leaves the handle initialised)
    tiles, tile_ms = sw.autotune() if not args.no_autotune else (sw.tiles, {})
    sw.init()
    sw.sweep(args.warmup, record=RECORD)
    sw.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk_dir = os.environ.get("KDQ_CLOCKS_DIR")   # keep the raw clock samples there when set
    clk_path = os.path.join(clk_dir, f"clocks_rank{rank}.csv") if clk_dir else \
        os.path.join(tempfile.gettempdir(), f"kdq_clocks_{os.getpid()}.csv")
    cproc, cfile = clocks_start(clk_path)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sw.sweep(args.steps, record=RECORD)
    e1.record(stream)
    e1.synchronize()
    clocks = clocks_stop(cproc, cfile, clk_path, local)
    sw.synchronize()
    ms = e0.elapsed_time(e1)
    st = sw.stats()
    obs = sw.get_obs(args.warmup + args.steps)
    ek = obs[:, args.warmup:, 0]
    tau_live = tau_int(ek)
    tau = args.tau_int or (reference_tau_int() if WL is WORKLOADS["c2"] and PRECISION == "fp64" else None) \
        or tau_live
    cs_per_s, t_max = replica_throughput(dist, ms, NCHAINS * args.steps, dev)
    value = cs_per_s / tau

    # ---- roofline of the sweep kernel (the only kernel of the timed region)
    acc_per_chain_sweep = st["accepted"] / (NCHAINS * args.steps)
    launches_per_sweep = 2 * (len(model.nodes) - 1) + 1     # block launches + one control reset per call
    block_launches = args.steps * 2 * (len(model.nodes) - 1)
    per_launch = NCHAINS / (2 * (len(model.nodes) - 1))
    avg_launch_s = ms * 1e-3 / block_launches
    peak = fp64_peak_tflops(torch, dev)
    kc = bool(np.any(np.imag(np.asarray(model.eK)) != 0))
    fl = sweep_flops(model, acc_per_chain_sweep, record=RECORD, k_complex=kc)
    if PRECISION == "fp64":
        flops_per_launch = fl["total"] * per_launch
        pipe = "FP64 DFMA (CUDA cores)"
    else:   # the FP64 part (QR, LU, G recompute) is what the mixed sweep is bound by
        flops_per_launch = fl["stabilise_qr_lu"] * per_launch
        pipe = "FP64 DFMA for QR, LU and the G recompute (the FP32 bulk products are reported apart)"
    achieved = flops_per_launch / avg_launch_s / 1e12
    roof = {"bound": "fp64", "pipe": pipe, "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (no FP64 figure in MEASURED_PEAKS.json)",
            "traffic": traffic_per_launch() if WL is WORKLOADS["c2"] and PRECISION == "fp64" else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, mean over the sweep's "
                              "k_block launches of the same workload (profiles/k_block_tv6x6_launches.md)",
            "flops_per_launch": flops_per_launch,
            "flops_per_chain_sweep": fl}
    if PRECISION == "mixed":
        roof["fp32_achieved_tflops"] = (fl["total"] - fl["stabilise_qr_lu"]) * per_launch / avg_launch_s / 1e12

    if args.phases:
        sw.enable_phase_timing(True)
        sw.sweep(1, record=RECORD)
        sw.synchronize()
        ph = sw.phase_cycles()
        tot = sum(ph.values())
        print(json.dumps({"phase_shares": {k: round(v / tot, 4) for k, v in ph.items()},
                          "ms_per_chain_sweep_at_sm_clock": {k: v / NCHAINS / 2.07e6 for k, v in ph.items()}}),
              file=sys.stderr, flush=True)
        sw.enable_phase_timing(False)

    # ---- Rényi-2 entropy of the left half (t-UV 8x8): chain pairs (2c, 2c+1)
    # are the replicas; e^{-S2} = <|det g_A|^2> with g_A the Grover matrix of
    # the pair's G at tau = Nt/2 (untimed sweeps after the timed region)
    renyi = None
    if WL is WORKLOADS["c4"]:
        from kapdqmc_gb300.geometry import area_index
        index = area_index("SQUARE45", list(model.site), ((1, 1), (model.site[0], model.site[1])))
        sw.keep_middle_green(True)
        vals = []
        for _ in range(args.renyi_sweeps):
            sw.sweep(1, record=RECORD)
            sw.synchronize()
            vals.append(np.abs(sw.grover_det_middle(index)) ** 2)
        sw.keep_middle_green(False)
        v = np.array(vals)                       # (sweeps, pairs)
        pair_means = v.mean(axis=0)
        mean, err = float(pair_means.mean()), float(pair_means.std(ddof=1) / math.sqrt(len(pair_means)))
        renyi = {"S2": -math.log(mean), "S2_err": err / mean, "region": f"left half, {len(index)} sites",
                 "pairs": len(pair_means), "sweeps": args.renyi_sweeps,
                 "estimator": "e^-S2 = <|det(2 G1 G2 - G1 - G2 + I)_A|^2>, pair means over sweeps"}

    # ---- end to end through kdq_phy_update with host buffers
    e2e_steps = max(2, min(args.steps, 5))
    cur = sw.get_fields()
    h2d = cur.nbytes
    d2h = cur.nbytes + NCHAINS * model_nobs(sw) * 8
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_rows = []
    for _ in range(e2e_steps):
        sw.set_fields(cur)
        o = sw.phy_update(1, record=RECORD)
        cur = sw.get_fields()
        e2e_rows.append(o[:, 0, 0])
    wall = time.perf_counter() - t0
    e2e_cs, _ = replica_throughput(dist, wall * 1e3, NCHAINS * e2e_steps, dev)
    wall = dist_max(dist, wall, dev)
    e2e_value = e2e_cs / tau

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None,
               "dtype": "f64" if PRECISION == "fp64" else "f32 bulk products and updates, f64 ratios/QR/recompute",
               "data": "synthetic (seeded HS fields and Philox proposal stream)",
               "config": dict(config(), parallelism=f"replicas x{world}"),
               "chain_sweeps_per_s": cs_per_s, "tau_int": tau, "tau_int_live": tau_live,
               "tau_int_source": "committed long run" if tau != tau_live else "this run",
               "acceptance": st["accepted"] / max(st["proposals"], 1),
               "max_drift": st["max_drift"],
               "energy_mean": float(ek.mean()), "energy_err": float(ek.mean(axis=1).std() / math.sqrt(NCHAINS)),
               "gpu_launches": args.steps * launches_per_sweep,
               "tiles": {"class": tiles, "autotune_sweep_ms": tile_ms},
               **({"renyi2": renyi} if renyi else {}),
               "roofline": roof, "clocks": clocks,
               "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                       "ms_per_step": wall / e2e_steps * 1e3}}
        print(json.dumps(out), file=sys.stderr, flush=True)
        if not args.no_cpu and world == 1 and WL is WORKLOADS["c2"]:
            cores = os.cpu_count() or 1
            cs_cpu, wall_cpu = cpu_chain_sweeps_per_s(cores, sweeps_per_chain=CPU_SWEEPS)
            out["cpu_baseline"] = {"value": cs_cpu / tau, "unit": UNIT, "cores": cores, "kind": CPU_KIND,
                                   "chain_sweeps_per_s": cs_cpu,
                                   "sample": f"{CPU_SAMPLE}; {cores} chains x {CPU_SWEEPS} sweeps of the same workload, "
                                             f"{wall_cpu:.1f} s"}
        print(json.dumps(out))
    sw.close()
    if dist:
        dist.destroy_process_group()


def run_slmc(args):
    """Self-learning proposals against the plain local-update sweep (t-U).

    1. Equilibrate the chains, then collect `--slmc-train-sweeps` sweeps of
       configurations (chains x sweeps of them) with their log|det|.
    2. Fit the effective model with the library's CUDA training kernels.
    3. From the same equilibrated fields run two arms of `--steps` timed
       sweeps each, measuring every sweep: local updates only, and local
       updates plus the cluster moves.  τ_int of the energy and of the AF
       structure factor (SDW0 column) come from each arm's own series.
    4. The plain FP64 sweep's chain-sweeps/s is timed on the same fields, so
       the gain is against the plain FP64 GPU method.
    One JSON line; value = the cluster-move arm's effective samples/s (the
    slower of the two observables)."""
    import torch
    from kapdqmc_gb300 import Initial_s, slmc
    from kapdqmc_gb300.sweep import Sweeper

    model = make_model()
    if model.kind != 0:
        print(json.dumps({"slmc": "unavailable", "why": "cluster moves are implemented for t-U only"}))
        return
    dev = torch.device("cuda", 0)
    seed = 777
    fields = np.stack([Initial_s(model, 3000 + c) for c in range(NCHAINS)])

    def sweeper(prec, s0, rng):
        sw = Sweeper(model, NCHAINS)
        sw.set_precision(prec)
        sw.set_fields(s0)
        sw.set_rng(rng)
        return sw

    def timed(sw, n):
        stream = torch.cuda.ExternalStream(sw.stream, device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sw.sweep(n, record=RECORD)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3

    # 1. equilibrate and collect training data
    sw = sweeper(PRECISION, fields, seed)
    sw.init()
    sw.sweep(args.slmc_burn, record=0)
    t0 = time.perf_counter()
    X, Y = [], []
    for _ in range(args.slmc_train_sweeps):
        sw.sweep(1, record=0)
        X.append(slmc.cnn_fields(sw.get_fields()))
        Y.append(sw.log_det()[0])
    t_collect = time.perf_counter() - t0
    s_eq = sw.get_fields()
    sw.close()
    X = np.concatenate(X)
    Y = np.concatenate(Y)
    # 2. fit
    t0 = time.perf_counter()
    params, loss, (mu, sd) = slmc.fit_effective_model(X, Y, epochs=args.slmc_epochs, batch=64, lr=2e-3, seed=1)
    t_train = time.perf_counter() - t0
    F = slmc.cnn_forward(X[:512], params)
    resid = float(np.std(F - 2 * Y[:512]))

    # 3. the two arms
    arms = {}
    for name, on in (("local", False), ("slmc", True)):
        sw = sweeper(PRECISION, s_eq, seed + 1)
        if on:
            sw.slmc_enable(params, args.slmc_moves, args.slmc_len, args.slmc_steps)
        sw.init()
        sw.sweep(args.warmup, record=RECORD)
        sw.synchronize()
        secs = timed(sw, args.steps)
        obs = sw.get_obs(args.warmup + args.steps)[:, args.warmup:, :]
        st = sw.slmc_stats() if on else None
        sw.close()
        cs = NCHAINS * args.steps / secs
        te, ta = tau_int(obs[:, :, 0]), tau_int(obs[:, :, 4])
        arm = {"chain_sweeps_per_s": cs, "tau_int_energy": te, "tau_int_af_sf": ta,
               "eff_samples_per_s": cs / max(te, ta),
               "energy": [float(obs[:, :, 0].mean()), float(obs[:, :, 0].mean(axis=1).std() / math.sqrt(NCHAINS))],
               "double_occupancy": [float(obs[:, :, 1].mean() / model.Ns),
                                    float(obs[:, :, 1].mean(axis=1).std() / math.sqrt(NCHAINS) / model.Ns)],
               "af_sf": [float(obs[:, :, 4].mean()), float(obs[:, :, 4].mean(axis=1).std() / math.sqrt(NCHAINS))]}
        if st:
            arm["cluster_moves"] = dict(st, acceptance=st["accepted"] / max(1, st["proposed"] - st["unchanged"]))
        arms[name] = arm
    # 4. the plain FP64 sweep's throughput on the same fields
    sw = sweeper("fp64", s_eq, seed + 2)
    sw.init()
    sw.sweep(1, record=RECORD)
    sw.synchronize()
    n64 = max(2, args.steps // 10)
    cs64 = NCHAINS * n64 / timed(sw, n64)
    sw.close()
    base = cs64 / max(arms["local"]["tau_int_energy"], arms["local"]["tau_int_af_sf"])

    def within(a, b, k):
        return abs(a[k][0] - b[k][0]) <= math.hypot(a[k][1], b[k][1]) * 2.0

    out = {"metric": METRIC, "value": arms["slmc"]["eff_samples_per_s"], "unit": UNIT, "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "c128" if PRECISION == "fp64" else "c64+c128",
           "data": "synthetic (seeded HS fields and Philox proposal and cluster-move streams)",
           "config": dict(config(), slmc={"moves_per_slice": args.slmc_moves, "cluster_len": args.slmc_len,
                                          "eff_steps": args.slmc_steps}),
           "plain_fp64_eff_samples_per_s": base, "gain_vs_plain_fp64": arms["slmc"]["eff_samples_per_s"] / base,
           "plain_fp64_chain_sweeps_per_s": cs64, "arms": arms,
           "obs_agree_2sigma": {k: within(arms["slmc"], arms["local"], k)
                                for k in ("energy", "double_occupancy", "af_sf")},
           "training": {"configs": int(X.shape[0]), "collect_s": t_collect, "train_s": t_train,
                        "epochs": args.slmc_epochs, "loss_first_last": [float(loss[0]), float(loss[-1])],
                        "target_sd": sd, "residual_sd": resid}}
    print(json.dumps(out))


# Members of the group line: (workload, chains, precision); every configuration
# with a quarter of its batch, so that no member fills the GPU alone.
GROUP = [("c1", 64, "fp64"), ("c2", 64, "fp64"), ("c4", 64, "mixed"), ("c5", 64, "mixed")]


def run_group(args):
    """Chains of four lattices and three models swept as one CUDA graph per
    sweep (kdq_group_sweep) against the same handles swept one after another."""
    from kapdqmc_gb300 import Initial_s
    from kapdqmc_gb300.sweep import Sweeper, SweeperGroup

    sws = []
    for i, (wl, n, prec) in enumerate(GROUP):
        model = WORKLOADS[wl]["make"]()
        sw = Sweeper(model, n)
        sw.set_precision(prec)
        sw.set_fields(np.stack([Initial_s(model, 4000 + 100 * i + c) for c in range(n)]))
        sw.set_rng(777 + i)
        sw.autotune()
        sws.append(sw)
    total = sum(n for _, n, _ in GROUP)

    def separate(sweeps):
        t = time.perf_counter()
        for sw in sws:
            sw.sweep(sweeps, record=RECORD)
            sw.synchronize()
        return time.perf_counter() - t

    separate(1)                                   # graphs captured, caches warm
    t_sep = separate(args.steps)
    with SweeperGroup(sws) as grp:
        grp.sweep(1, record=RECORD)
        grp.synchronize()
        t0 = time.perf_counter()
        grp.sweep(args.steps, record=RECORD)
        grp.synchronize()
        t_grp = time.perf_counter() - t0
    member_s = {}
    for (wl, n, prec), sw in zip(GROUP, sws):
        t = time.perf_counter()
        sw.sweep(args.steps, record=RECORD)
        sw.synchronize()
        member_s[f"{wl}/{n}/{prec}"] = (time.perf_counter() - t) / args.steps
        sw.close()
    out = {"metric": "chain-sweeps/s of a group of lattices and models swept as one CUDA graph",
           "value": total * args.steps / t_grp, "unit": "chain-sweeps/s", "n_gpus": 1,
           "steps": args.steps, "warmup": 1, "higher_is_better": True, "dtype": "f64 / f32 bulk (mixed members)",
           "data": "synthetic (seeded HS fields and Philox proposal stream)",
           "config": {"workload": "group: " + ", ".join(f"{wl} x{n} {p}" for wl, n, p in GROUP)},
           "separate_value": total * args.steps / t_sep,
           "speedup_vs_separate": t_sep / t_grp,
           "seconds_per_sweep_alone": member_s}
    print(json.dumps(out))


def run_scee(args):
    """Coupled SCEE sweep (ctrl_SCEEicr) on a t-U workload: replica pairs of
    the workload's chains, regions A = the first third of the lattice's
    columns (all rows), B = its first two thirds of rows (the reference's
    test regions, test/tU/HCtU_runtests.jl:21-24), lambda = 0.5, Nlambda = 2.
    Prints pair-sweeps/s on the GPU and, as the CPU baseline, the numpy
    restatement of the same sweep timed on one host core for one pair."""
    import torch
    from kapdqmc_gb300 import Initial_s, area_index
    from kapdqmc_gb300.sweep import Sweeper

    model = make_model()
    if model.kind != 0:
        print(json.dumps({"scee": "unavailable", "why": "the SCEE sweep is implemented for t-U only"}))
        return
    L = model.site[1]
    A = area_index(model.Lattice, model.site, ([1, 1], [L // 3, L]))
    B = area_index(model.Lattice, model.site, ([1, 1], [L // 3, 2 * L // 3]))
    pairs = NCHAINS // 2
    fields = np.stack([Initial_s(model, 9000 + c) for c in range(2 * pairs)])
    dev = torch.device("cuda", 0)
    sw = Sweeper(model, 2 * pairs)
    sw.set_fields(fields)
    sw.set_rng(4242)
    sw.scee_enable(A, B, 0.5, 2)
    sw.scee_run(args.warmup)            # untimed: includes building every block product
    sw.set_fields(sw.get_fields())
    stream = torch.cuda.ExternalStream(sw.stream, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    O = sw.scee_run(args.steps)
    e1.record(stream)
    e1.synchronize()
    secs = e0.elapsed_time(e1) * 1e-3
    sw.close()
    est = O[:, 1:]
    # algorithmic FP64 work of the slice wraps alone (a lower bound of the
    # sweep's work): per slice and replica Gt two N^3 products, Gt0 and G0t one
    # each, complex (8 flops per multiply-add), both directions
    wrap_flops = 2 * model.Nt * 2 * 4 * model.Ns ** 3 * 8
    peak = fp64_peak_tflops(torch, dev)
    achieved = wrap_flops * pairs * args.steps / secs / 1e12
    out = {"metric": "SCEE pair-sweeps/s (ctrl_SCEEicr)", "value": pairs * args.steps / secs,
           "unit": "pair-sweeps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": secs * 1e3 / args.steps, "higher_is_better": True, "dtype": "c128",
           "data": "synthetic (seeded HS fields and Philox stream)",
           "config": dict(config(), pairs=pairs, nA=len(A), nB=len(B), lam=0.5, nlam=2,
                          timed="one kdq_scee_run call: block products and chains rebuilt, then the sweeps"),
           "estimator_mean": float(est.mean()), "estimator_err": float(est.mean(axis=1).std() / math.sqrt(pairs)),
           "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                        "counted": "slice wraps only (8 N^3 complex multiply-adds per slice and pair)",
                        "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"}}
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import dqmc_oracle as O_
        import philox
        import scee_oracle
        n_rep = 2 * model.Ns * model.Nt
        k0, u0 = philox.tape(1, 0, 0, n_rep)
        k1, u1 = philox.tape(1, 1, 0, n_rep)
        tape = O_.Tape(np.stack([k0, k1], axis=1).ravel(), np.stack([u0, u1], axis=1).ravel())
        sc = scee_oracle.SCEE(model, fields[0], fields[1], A, B, 0.5, 2, tape).init()
        n_sl = min(model.Nt, int(model.nodes[3]))     # the first three blocks of the forward sweep
        t0 = time.perf_counter()
        for lt in range(1, n_sl + 1):
            sc.forward_slice(lt)
        wall = (time.perf_counter() - t0) * (2 * model.Nt) / n_sl
        cores = os.cpu_count() or 1
        out["cpu_baseline"] = {"value": cores / wall, "unit": "pair-sweeps/s", "cores": cores, "kind": "port",
                               "sample": f"numpy restatement of ctrl_SCEEicr, one pair, the first {n_sl} forward "
                                         f"slices on one core scaled to a sweep ({wall:.1f} s per pair-sweep), "
                                         f"times the core count"}
    print(json.dumps(out))


def dist_max(dist, value: float, device=None) -> float:
    """Max of a per-rank value over all ranks (identity without a process group)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(dist, ms_local: float, units_local: int, device=None):
    """Whole-job units/s of independent replicas: units of all ranks over the slowest rank's time."""
    world = dist.get_world_size() if dist is not None else 1
    ms = dist_max(dist, ms_local, device)
    return units_local * world / (ms * 1e-3), ms


def model_nobs(sw):
    return sw.n_obs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--group", action="store_true",
                    help="lattices of several configurations swept as one CUDA graph vs one after another")
    ap.add_argument("--renyi-sweeps", type=int, default=10,
                    help="t-UV 8x8 (c4): untimed sweeps whose replica pairs estimate S2 of the left half")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default tile class instead of timing each class first")
    ap.add_argument("--tau-int", type=float, default=None,
                    help="τ_int used to convert chain-sweeps/s (default: the committed long-run value)")
    ap.add_argument("--phases", action="store_true",
                    help="print the per-stage clock shares of one untimed sweep to stderr")
    ap.add_argument("--tau-run", type=int, default=0,
                    help="long run of this many sweeps; prints the workload's τ_int JSON and exits")
    ap.add_argument("--chains", type=int, default=None,
                    help="chains per GPU (profiling of small cases only; bench lines use the workload's)")
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS),
                    help="configuration (default c2, the metric's; the CPU arm exists for c2 only)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="arithmetic of the sweep (mixed: complex sweeps only)")
    ap.add_argument("--slmc", action="store_true",
                    help="self-learning cluster moves against local updates (t-U workloads; prints its own line)")
    ap.add_argument("--scee", action="store_true",
                    help="coupled SCEE sweep of replica pairs (t-U workloads; prints its own line)")
    ap.add_argument("--slmc-burn", type=int, default=10)
    ap.add_argument("--slmc-train-sweeps", type=int, default=80,
                    help="sweeps of configurations collected for training (x chains configurations)")
    ap.add_argument("--slmc-epochs", type=int, default=10)
    ap.add_argument("--slmc-moves", type=int, default=1)
    ap.add_argument("--slmc-len", type=int, default=32)
    ap.add_argument("--slmc-steps", type=int, default=64)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    global WL, NCHAINS, PRECISION
    WL = WORKLOADS[args.workload]
    NCHAINS = args.chains or WL["chains"]
    PRECISION = args.precision
    if args.impl == "reference" and args.workload != "c2":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU restatement covers the t-V workload only"}))
        return
    if args.group:
        run_group(args)
    elif args.scee:
        if args.workload == "c2":
            WL = WORKLOADS["c5"]
            NCHAINS = args.chains or WL["chains"]
        run_scee(args)
    elif args.slmc:
        if args.workload == "c2":
            WL = WORKLOADS["c5"]
            NCHAINS = args.chains or WL["chains"]
        run_slmc(args)
    elif args.tau_run:
        run_tau(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
