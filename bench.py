"""Benchmark of the projector-DQMC sweep on GB300.

Workload (the metric's own configuration): 256 independent Markov chains of
the t-U Hubbard model on the 12x12 square lattice (N = 144, U/t = 8,
dt = 0.05, 2Θ = 16 -> 320 slices, n_wrap = 8), energy and double occupancy
measured every sweep.  One step = one forward+backward sweep of every chain.

Metric: effective samples/s = chain-sweeps/s / (2 τ_int(E_kin)) of the
mixed-precision sweep (FP32 bulk products and updates, FP64 ratios,
stabilisation and recompute), summed over all GPUs; `vs_baseline` is its
ratio to the plain FP64 GPU sweep measured in the same run on the same
fields (the metric's "vs plain FP64 DQMC").  τ_int (Sokal window, τ_int >= 1/2
for uncorrelated samples, so N sweeps are worth N / (2 τ_int) independent
samples) comes from a committed long run of each arm (`--tau-run`) and is
also estimated live from the timed sweeps.

  value   device-resident: fields and B chains live in HBM, one kdq_sweep
          per step, timed with CUDA events on the library's stream
  e2e     through the reference-shaped C-ABI call kdq_phy_update with host
          buffers: fields uploaded, chain rebuilt, one sweep, fields and
          measurement rows read back, every step

`--impl reference` times the C restatement of the reference algorithm
(t-U, t-V or t-UV, whichever the workload is) on the host cores instead;
`--workload c1|c2|c4|c5` selects the other configurations.
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
UNIT = "chain-sweeps/s / (2 tau_int)"
NCHAINS = 256
RECORD = 2   # measurements as the reference's estimator, wraps folded into two products (kdq_phy_update)


def tau_file():
    return ROOT / "profiles" / f"tau_int_{WL['tag']}.json"


def committed_tau(precision):
    """τ_int(E_kin) of `precision` on this workload from its committed long run."""
    try:
        return float(json.loads(tau_file().read_text())[precision]["tau_int"])
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


# The bench line is c3 at the spec batch (256 chains at N = 144, the
# metric's configuration); the others are the remaining single-GPU
# configurations, for `--workload`.
WORKLOADS = {
    "c1": dict(make=_tu_4x4, chains=1, Ns=16, Nt=100, n_wrap=10, tag="tu_square_4x4",
               desc="t-U 4x4 square (N=16), 100 slices, n_wrap=10, U/t=4, dt=0.1, one chain, "
                    "energy + double occupancy per sweep",
               model="tU_Hubbard_Para(SQUARE45, site=[2,4])"),
    "c2": dict(make=_tv_6x6, chains=256, Ns=72, Nt=400, n_wrap=10, tag="tv_honeycomb_6x6",
               desc="t-V 6x6 honeycomb (N=72), 400 slices, n_wrap=10, V/t=1, dt=0.05, 256 independent "
                    "chains, energy + density structure factor per sweep",
               model="tV_Hubbard_Para(HoneyComb120, site=[6,6])"),
    "c3": dict(make=_tu_12x12, chains=256, Ns=144, Nt=320, n_wrap=8, tag="tu_square_12x12",
               desc="t-U 12x12 square (N=144), 320 slices, n_wrap=8, U/t=8, dt=0.05, 256 independent "
                    "chains, energy + double occupancy per sweep",
               model="tU_Hubbard_Para(SQUARE45, site=[6,12])"),
    "c4": dict(make=_tuv_8x8, chains=256, Ns=64, Nt=200, n_wrap=10, tag="tuv_square_8x8",
               desc="t-UV 8x8 square (N=64), 200 slices, n_wrap=10, U/t=4, V/t=0.5, dt=0.1, 256 chains "
                    "(128 replica pairs), energies per sweep",
               model="tUV_Hubbard_Para(SQUARE45, site=[4,8], allow_marginal=True)"),
    "c5": dict(make=_tu_hc_9x9, chains=256, Ns=162, Nt=200, n_wrap=10, tag="tu_honeycomb_9x9",
               desc="t-U 9x9 honeycomb (N=162), 200 slices, n_wrap=10, U/t=4, dt=0.1, 256 chains, "
                    "energy, double occupancy and structure factors per sweep",
               model="tU_Hubbard_Para(HoneyComb120, site=[9,9])"),
}
WL = WORKLOADS["c3"]
PRECISION = "mixed"


def make_model():
    return WL["make"]()


def config():
    return {"workload": WL["desc"] + f", {PRECISION}", "model": WL["model"], "chains_per_gpu": NCHAINS,
            "Ns": WL["Ns"], "Nt": WL["Nt"], "n_wrap": WL["n_wrap"], "precision": PRECISION,
            "parallelism": f"replicas x{int(os.environ.get('WORLD_SIZE', '1'))}",
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


def gemm_peak_tflops(torch, dev, dtype, tf32=False):
    """Measured pipe ceiling: a cuBLAS GEMM 4096^3 of `dtype`, best of 5
    (CUDA events); FP32 with TF32 disabled is the CUDA-core FP32 pipe, with
    TF32 enabled the TF32 tensor pipe."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = tf32
    try:
        a = torch.randn(4096, 4096, dtype=dtype, device=dev)
        b = torch.randn(4096, 4096, dtype=dtype, device=dev)
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
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return best


def fp64_peak_tflops(torch, dev):
    return gemm_peak_tflops(torch, dev, torch.float64)


def traffic_per_launch():
    """DRAM bytes (read + write) per sweep-kernel launch from the committed ncu
    capture of this workload and precision, scaled to the bench's chains."""
    try:
        d = json.loads((ROOT / "profiles" / f"k_block_{WL['tag']}_{PRECISION}_traffic.json").read_text())
        return float(d["dram_bytes_per_launch_per_chain"]) * NCHAINS
    except Exception:
        return None


def hbm_peak_gbs():
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except Exception:
        return 6800.0


# ---------------------------------------------------------------- CPU arm
_CPU = {}   # per worker process: model, this worker's chain field, tapes


def _cpu_init(wl, counter):
    """Pool initializer: each worker owns one chain (numbered by the shared
    counter) of workload `wl`; model, field and library are built here,
    outside any timed call."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import cport
    from kapdqmc_gb300 import Initial_s
    global WL
    WL = WORKLOADS[wl]
    with counter.get_lock():
        chain = counter.value
        counter.value += 1
    model = make_model()
    cport.load()
    _CPU.update(model=model, chain=chain, s=Initial_s(model, 1000 + chain))


def _cpu_worker(args):
    """Sweep this worker's chain `sweeps` times through the C restatement of
    the reference sweep, with a tape drawn before the clock starts; returns
    the seconds of the C call."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import cport
    import dqmc_oracle as O
    import philox
    seed, sweeps = args
    model, chain = _CPU["model"], _CPU["chain"]
    n = O.proposals_per_sweep(model)
    ks, us = zip(*(philox.tape(seed, chain, w, n) for w in range(sweeps)))
    k, u = np.concatenate(ks), np.concatenate(us)
    run = (cport.tu_phy_update, cport.tv_phy_update, cport.tuv_phy_update)[model.kind]
    t0 = time.perf_counter()
    s, _, _ = run(model, _CPU["s"], sweeps, k, u, record=True)
    dt = time.perf_counter() - t0
    _CPU["s"] = s
    return dt


CPU_KIND = "port"


def cpu_sample_desc():
    what = ("C restatement of the reference t-U sweep (complex eK and complex GEMMs as the reference)",
            "C restatement of the reference t-V sweep (dense bond-rotation GEMMs as the reference)",
            "C restatement of the reference t-UV sweep (complex eK, complex GEMMs and rank-2 bond updates as "
            "the reference)")[make_model().kind]
    return what + "; OpenBLAS/LAPACK from numpy, 1 thread each; one chain per host core"


class CpuArm:
    """The reference algorithm on the host cores: one chain per core, all busy.
    Model, fields and proposal tapes are built outside the timed calls."""

    def __init__(self, cores: int):
        import multiprocessing as mp
        sys.path.insert(0, str(ROOT / "oracle"))
        import cport
        cport.build()
        self.cores = cores
        saved = {v: os.environ.get(v) for v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
        for v in saved:                     # inherited by the workers before numpy loads
            os.environ[v] = "1"
        ctx = mp.get_context("spawn")
        wl = next(k for k, v in WORKLOADS.items() if v is WL)
        try:
            self.pool = ctx.Pool(cores, initializer=_cpu_init, initargs=(wl, ctx.Value("i", 0)))
        finally:
            for v, x in saved.items():
                if x is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = x
        self.calls = 0

    def step(self, sweeps_per_chain: int = 1) -> float:
        """Seconds for `cores` chains to run sweeps_per_chain sweeps concurrently:
        the slowest worker's C-call time (all workers start together)."""
        self.calls += 1
        times = self.pool.map(_cpu_worker, [(7 + self.calls, sweeps_per_chain)] * self.cores, chunksize=1)
        return max(times)

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


OBS_NAMES = {0: ("Ek", "Eu", "CDW0", "CDW1", "SDW0", "SDW1", "S_charge_full", "S_charge_full_q1",
                 "S_spin_full", "S_spin_full_q1"),
             1: ("Ek", "Ev", "R0_AA", "R0_BB", "R0_BA", "R0_AB", "R1_AA", "R1_BB", "R1_BA", "R1_AB"),
             2: ("Ek", "Eu", "Ev", "CDW0", "CDW1", "SDW0", "SDW1", "S_charge_full", "S_charge_full_q1",
                 "S_spin_full", "S_spin_full_q1")}
SPIN_COL = {0: 8, 2: 9}     # corrected AF spin structure factor (staggered, full measurement)


def full_measurement(model) -> bool:
    return model.kind == 0 or (model.kind == 2 and model.is_complex)


def new_sweeper(model, prec, fields, seed, device=0):
    from kapdqmc_gb300.sweep import Sweeper
    sw = Sweeper(model, len(fields), device=device)
    sw.set_precision(prec)
    if full_measurement(model):
        sw.set_measure_full(True)
    sw.set_fields(fields)
    sw.set_rng(seed)
    return sw


def obs_summary(model, obs):
    """Mean and standard error (over independent chains) of every column;
    obs is (chains, sweeps, n_obs) of equilibrated sweeps."""
    names = OBS_NAMES[model.kind]
    cm = obs.mean(axis=1)
    out = {}
    for q in range(obs.shape[2]):
        if not np.any(obs[:, :, q]):
            continue
        out[names[q]] = [float(cm[:, q].mean()), float(cm[:, q].std(ddof=1) / math.sqrt(cm.shape[0]))]
    if "Eu" in out and model.kind == 0:     # double occupancy per site
        out["double_occupancy"] = [out["Eu"][0] / model.Ns, out["Eu"][1] / model.Ns]
    return out


def binned_tau(x):
    """τ_int from binning: var(bin means) * B / (2 var), B = 1 .. 16."""
    var = x.var()
    bins = {}
    for B in (1, 2, 4, 8, 16):
        T = x.shape[1] // B
        if T < 2:
            break
        m = x[:, :T * B].reshape(x.shape[0], T, B).mean(axis=2)
        bins[B] = float(m.var() * B / (2 * var)) if var > 0 else 0.5
    return bins


def run_tau(args):
    """Long runs of the bench's two arms: τ_int of the energy (and of the AF
    spin structure factor where it is measured), binning cross-checks, and
    every observable's mean and error per arm with the mixed-vs-FP64
    difference in units of its combined error.  The mixed arm equilibrates
    from random fields; the FP64 arm starts from its final fields.  Prints
    the JSON that is committed as profiles/tau_int_<workload>.json."""
    from kapdqmc_gb300 import Initial_s
    model = make_model()
    fields = np.stack([Initial_s(model, 5000 + c) for c in range(NCHAINS)])
    arms = [("mixed", args.tau_burn, args.tau_run)] if model.is_complex else []
    arms.append(("fp64", args.tau_burn if not arms else max(5, args.tau_burn // 3),
                 args.tau_run_fp64 or max(20, args.tau_run // 3)))
    out = {"workload": config()["workload"], "chains": NCHAINS, "record": RECORD,
           "estimator": "Sokal window c=5 on the chain-pooled autocovariance; binning as a check",
           "errors": "standard error over independent chains of the per-chain means"}
    for prec, burn, sweeps in arms:
        sw = new_sweeper(model, prec, fields, 424242 + len(out))
        sw.init()
        t0 = time.perf_counter()
        sw.sweep(burn + sweeps, record=RECORD)
        sw.synchronize()
        wall = time.perf_counter() - t0
        obs = sw.get_obs(burn + sweeps)[:, burn:, :]
        fields = sw.get_fields()
        st = sw.stats()
        sw.close()
        arm = {"burn_in": burn, "sweeps": sweeps, "wall_s": wall,
               "chain_sweeps_per_s": NCHAINS * (burn + sweeps) / wall,
               "tau_int": tau_int(obs[:, :, 0]), "tau_int_binning": binned_tau(obs[:, :, 0]),
               "acceptance": st["accepted"] / max(st["proposals"], 1), "max_drift": st["max_drift"],
               "obs": obs_summary(model, obs)}
        if model.kind in SPIN_COL and obs.shape[2] > SPIN_COL[model.kind] and np.any(obs[:, :, SPIN_COL[model.kind]]):
            x = obs[:, :, SPIN_COL[model.kind]]
            arm["tau_int_af_spin_sf"] = tau_int(x)
            arm["tau_int_af_spin_sf_binning"] = binned_tau(x)
        out[prec] = arm
        print(json.dumps({prec: {k: v for k, v in arm.items() if k != "obs"}}), file=sys.stderr, flush=True)
    if "mixed" in out and "fp64" in out:
        a, b = out["mixed"]["obs"], out["fp64"]["obs"]
        out["z_mixed_vs_fp64"] = {k: (a[k][0] - b[k][0]) / math.hypot(a[k][1], b[k][1])
                                  for k in a if k in b and math.hypot(a[k][1], b[k][1]) > 0}
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
    tau = args.tau_int or committed_tau("fp64")
    tau_src = "given" if args.tau_int else "the plain FP64 sweep's committed long-run value"
    if tau is None:
        tau, tau_src = 0.5, "the lower bound 0.5: no committed long run for this workload"
    value = cs / (2 * tau)
    sample = (f"{cpu_sample_desc()}; {cores} chains x 1 sweep per step (model, fields and proposal tapes "
              f"built outside the timed calls); tau_int={tau:.3g} ({tau_src})")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": float(np.mean(walls)) * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "c128" if make_model().is_complex else "f64",
           "data": "synthetic (seeded HS fields and Philox proposal stream)", "config": config(),
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": CPU_KIND, "sample": sample,
                            "chain_sweeps_per_s": cs},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ---------------------------------------------------------------- GPU arm
def timed_arm(torch, dist, dev, model, prec, fields, seed, warmup, steps, autotune=True, clocks=False, rank=0):
    """One arm of the bench: `warmup` untimed sweeps, then `steps` sweeps timed
    with CUDA events on the library's stream between barriers."""
    sw = new_sweeper(model, prec, fields, seed, device=dev.index)
    stream = torch.cuda.ExternalStream(sw.stream, device=dev)
    tiles, tile_ms = sw.autotune() if autotune else (sw.tiles, {})
    sw.init()
    sw.sweep(warmup, record=RECORD)
    sw.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    cproc = cfile = clk_path = None
    if clocks:
        clk_dir = os.environ.get("KDQ_CLOCKS_DIR")   # keep the raw clock samples there when set
        clk_path = os.path.join(clk_dir, f"clocks_rank{rank}.csv") if clk_dir else \
            os.path.join(tempfile.gettempdir(), f"kdq_clocks_{os.getpid()}.csv")
        cproc, cfile = clocks_start(clk_path)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sw.sweep(steps, record=RECORD)
    e1.record(stream)
    e1.synchronize()
    clk = clocks_stop(cproc, cfile, clk_path, dev.index) if clocks else None
    sw.synchronize()
    ms = e0.elapsed_time(e1)
    st = sw.stats()
    obs = sw.get_obs(warmup + steps)[:, warmup:, :]
    return dict(sw=sw, ms=ms, stats=st, obs=obs, tiles=tiles, tile_ms=tile_ms, clocks=clk)


def run_gpu(args):
    import torch
    from kapdqmc_gb300 import Initial_s
    from kapdqmc_gb300.flops import mixed_roofline, sweep_flops

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
    fields = np.stack([Initial_s(model, 1000 + NCHAINS * rank + c) for c in range(NCHAINS)])
    seed = 20261203 + rank
    prec = PRECISION if model.is_complex else "fp64"

    # ---- the headline arm, device-resident
    A = timed_arm(torch, dist, dev, model, prec, fields, seed, args.warmup, args.steps,
                  autotune=not args.no_autotune, clocks=True, rank=rank)
    sw, ms, st = A["sw"], A["ms"], A["stats"]
    ek = A["obs"][:, :, 0]
    tau_live = tau_int(ek)
    tau = args.tau_int or committed_tau(prec) or tau_live
    cs_per_s, t_max = replica_throughput(dist, ms, NCHAINS * args.steps, dev)
    value = cs_per_s / (2 * tau)

    # ---- roofline of the sweep kernel (the only kernel of the timed region)
    acc_per_chain_sweep = st["accepted"] / (NCHAINS * args.steps)
    launches_per_sweep = 2 * (len(model.nodes) - 1) + 1     # block launches + one control reset per call
    block_launches = args.steps * 2 * (len(model.nodes) - 1)
    per_launch = NCHAINS / (2 * (len(model.nodes) - 1))
    avg_launch_s = ms * 1e-3 / block_launches
    kc = bool(np.any(np.imag(np.asarray(model.eK)) != 0))
    fl = sweep_flops(model, acc_per_chain_sweep, record=RECORD, k_complex=kc)
    traffic = {"traffic": traffic_per_launch(),
               "traffic_source": f"ncu dram__bytes_read.sum + dram__bytes_write.sum per k_block launch, per chain, "
                                 f"times the chains of a launch (profiles/k_block_{WL['tag']}_{prec}_traffic.json)"}
    if prec == "fp64":
        peak = fp64_peak_tflops(torch, dev)
        flops_per_launch = fl["total"] * per_launch
        achieved = flops_per_launch / avg_launch_s / 1e12
        roof = {"bound": "fp64", "pipe": "FP64 DFMA (CUDA cores)", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (no FP64 figure in MEASURED_PEAKS.json)",
                **traffic, "flops_per_launch": flops_per_launch, "flops_per_chain_sweep": fl}
    else:
        # time roofline over the pipes the mixed sweep's stages run on
        p_tf32 = gemm_peak_tflops(torch, dev, torch.float32, tf32=True)
        p_fp32 = gemm_peak_tflops(torch, dev, torch.float32, tf32=False)
        work = mixed_roofline(fl)                                  # pipe flops per chain-sweep
        t_pipe = {"tensor": work["tensor"] * per_launch / (p_tf32 * 1e12),
                  "fp32": work["fp32"] * per_launch / (p_fp32 * 1e12)}
        t_roof = sum(t_pipe.values())
        flops_per_launch = fl["total"] * per_launch                # algorithmic flops
        achieved = flops_per_launch / avg_launch_s / 1e12
        peak = flops_per_launch / t_roof / 1e12
        roof = {"bound": max(t_pipe, key=t_pipe.get), "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak,
                "what": "algorithmic flops of a launch over its measured time (achieved) and over its roofline "
                        "time (peak): sum over pipes of the pipe work at the pipe's measured rate, with the "
                        "3xTF32 products (kinetic, recompute X and BR X, delayed flushes) as 3 TF32 products "
                        "each and the double-float stabilisation at 12 FP32 operations per real multiply-add",
                "pipe_roofline_s_per_launch": t_pipe, "launch_s": avg_launch_s,
                "peaks_tflops": {"tf32_tensor": p_tf32, "fp32_cuda_core": p_fp32},
                "peak_source": "cuBLAS TF32 and FP32 (TF32 off) GEMM 4096^3 measured in this run",
                **traffic, "flops_per_launch": flops_per_launch, "flops_per_chain_sweep": fl,
                "pipe_work_per_chain_sweep": work}

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
    e2e_steps = max(2, min(args.steps, 3))
    cur = sw.get_fields()
    h2d = cur.nbytes
    d2h = cur.nbytes + NCHAINS * model_nobs(sw) * 8
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sw.set_fields(cur)
        sw.phy_update(1, record=RECORD)
        cur = sw.get_fields()
    wall = time.perf_counter() - t0
    e2e_cs, _ = replica_throughput(dist, wall * 1e3, NCHAINS * e2e_steps, dev)
    wall = dist_max(dist, wall, dev)
    e2e_value = e2e_cs / (2 * tau)
    eq_fields = cur
    sw.close()

    # ---- the plain FP64 GPU sweep on the same fields: the metric's baseline
    base = None
    if prec == "mixed" and not args.no_fp64_arm:
        n64 = max(2, args.steps // 5)
        B = timed_arm(torch, dist, dev, model, "fp64", eq_fields, seed + 7, args.warmup, n64, autotune=False)
        B["sw"].close()
        cs64, _ = replica_throughput(dist, B["ms"], NCHAINS * n64, dev)
        tau64 = args.tau_int or committed_tau("fp64") or tau_int(B["obs"][:, :, 0])
        base = {"chain_sweeps_per_s": cs64, "tau_int": tau64, "eff_samples_per_s": cs64 / (2 * tau64),
                "steps": n64, "warmup": args.warmup, "ms_per_step": B["ms"] / n64,
                "max_drift": B["stats"]["max_drift"]}

    if rank == 0:
        committed = {}
        try:
            committed = json.loads(tau_file().read_text())
        except Exception:
            pass
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
               "scaling": "weak",
               "vs_baseline": value / base["eff_samples_per_s"] if base else None,
               "vs_baseline_what": "mixed arm's effective samples/s over the plain FP64 GPU sweep's, same run, "
                                   "same fields (no published number exists for this metric)",
               "dtype": "c128" if prec == "fp64" and model.is_complex else (
                   "f64" if prec == "fp64" else "c64 bulk products and updates, c128 ratios/QR/recompute"),
               "data": "synthetic (seeded HS fields and Philox proposal stream)",
               "config": config(),
               "chain_sweeps_per_s": cs_per_s, "tau_int": tau, "tau_int_live": tau_live,
               "tau_int_source": "committed long run" if tau != tau_live else "this run",
               "acceptance": st["accepted"] / max(st["proposals"], 1),
               "max_drift": st["max_drift"],
               "obs_this_run": obs_summary(model, A["obs"]),
               "obs_long_run_z_mixed_vs_fp64": committed.get("z_mixed_vs_fp64"),
               "fp64_arm": base,
               "gpu_launches": args.steps * launches_per_sweep,
               "tiles": {"class": A["tiles"], "autotune_sweep_ms": A["tile_ms"]},
               **({"renyi2": renyi} if renyi else {}),
               "roofline": roof, "clocks": A["clocks"],
               "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                       "ms_per_step": wall / e2e_steps * 1e3,
                       "what": "kdq_phy_update per step: fields host->device, chain rebuilt, one sweep, "
                               "fields and rows device->host"}}
        print(json.dumps(out), file=sys.stderr, flush=True)
        if not args.no_cpu and world == 1 and WL is not WORKLOADS["c1"]:
            cores = os.cpu_count() or 1
            cs_cpu, wall_cpu = cpu_chain_sweeps_per_s(cores, sweeps_per_chain=args.cpu_sweeps)
            tau_cpu = committed_tau("fp64") or tau
            out["cpu_baseline"] = {"value": cs_cpu / (2 * tau_cpu), "unit": UNIT, "cores": cores, "kind": CPU_KIND,
                                   "chain_sweeps_per_s": cs_cpu,
                                   "sample": f"{cpu_sample_desc()}; {cores} chains x {args.cpu_sweeps} sweeps of the "
                                             f"same workload, {wall_cpu:.1f} s; tau_int {tau_cpu:.3g}"}
        print(json.dumps(out))
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


def run_slmc_scan(args):
    """Local updates against learned cluster moves on a small t-U lattice
    over a range of couplings: per U, the local sweep's acceptance and
    tau_int of the energy and of the AF spin structure factor, an effective
    model trained on the chains' configurations (held-out residual), and
    the same chains with one cluster move per slice of the largest and of
    half that cluster length.  One JSON line per U."""
    from kapdqmc_gb300 import Initial_s, slmc, tU_Hubbard_Para
    site = [int(v) for v in args.scan_site.split(",")]
    nch = args.chains or 256

    def arm(model, fields, seed, burn, sweeps, slmc_args=None):
        sw = new_sweeper(model, "mixed", fields, seed)
        if slmc_args is not None:
            sw.slmc_enable(*slmc_args)
        sw.init()
        sw.sweep(burn, record=0)
        sw.synchronize()
        t0 = time.perf_counter()
        sw.sweep(sweeps, record=RECORD)
        sw.synchronize()
        wall = time.perf_counter() - t0
        obs = sw.get_obs(sweeps)
        st, stats, s = (sw.slmc_stats() if slmc_args is not None else None), sw.stats(), sw.get_fields()
        sw.close()
        return {"chain_sweeps_per_s": len(fields) * sweeps / wall, "acceptance": stats["accepted"] / max(1, stats["proposals"]),
                "tau_int_energy": tau_int(obs[:, :, 0]), "tau_int_af_sf": tau_int(obs[:, :, 8]),
                "tau_int_binning_energy": binned_tau(obs[:, :, 0]), "tau_int_binning_af_sf": binned_tau(obs[:, :, 8]),
                "obs": obs_summary(model, obs), "cluster_moves": st}, s

    for U in (float(u) for u in args.scan_u.split(",")):
        model = tU_Hubbard_Para(Ht=1.0, Hu1=U, Hu2=U, Δt=0.1, Θrelax=5.0, Θquench=0.0, Lattice="SQUARE45",
                                site=site, BatchSize=10, Initial="H0")
        fields = np.stack([Initial_s(model, 100 + c) for c in range(nch)])
        local, s_eq = arm(model, fields, 1, 100, args.steps)
        sw = new_sweeper(model, "mixed", s_eq, 5)
        sw.init()
        X, Y = [], []
        for _ in range(40):
            sw.sweep(1, record=0)
            X.append(slmc.cnn_fields(sw.get_fields()))
            Y.append(sw.log_det()[0])
        sw.close()
        X, Y = np.concatenate(X), np.concatenate(Y)
        ntr = int(0.9 * len(X))
        params, loss, _ = slmc.fit_effective_model(X[:ntr], Y[:ntr], epochs=10, batch=64, lr=2e-3, seed=1)
        held = float(np.std(slmc.cnn_forward(X[ntr:], params) - 2 * Y[ntr:]) / np.std(2 * Y[ntr:]))
        out = {"U": U, "Ns": model.Ns, "Nt": model.Nt, "chains": nch, "sweeps": args.steps, "local": local,
               "heldout_residual_over_sd": held, "loss_first_last": [float(loss[0]), float(loss[-1])]}
        lmax = min(32, model.Ns // 2, model.Ns - 8)
        for L, steps in ((lmax, 64), (max(1, lmax // 2), 32)):
            out[f"cluster_L{L}_steps{steps}"], _ = arm(model, s_eq, 2, 20, args.steps, (params, 1, L, steps))
        print(json.dumps(out), flush=True)


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
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-sweeps", type=int, default=2,
                    help="sweeps per chain of the CPU baseline leg (one chain per host core)")
    ap.add_argument("--no-fp64-arm", action="store_true",
                    help="skip the plain FP64 GPU sweep timed beside the mixed arm")
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
    ap.add_argument("--tau-burn", type=int, default=30, help="burn-in sweeps of --tau-run")
    ap.add_argument("--tau-run-fp64", type=int, default=0, help="FP64 sweeps of --tau-run (default a third)")
    ap.add_argument("--tau-run", type=int, default=0,
                    help="long run of this many sweeps; prints the workload's τ_int JSON and exits")
    ap.add_argument("--chains", type=int, default=None,
                    help="chains per GPU (profiling of small cases only; bench lines use the workload's)")
    ap.add_argument("--workload", default=None, choices=sorted(WORKLOADS),
                    help="configuration (default: c3 at 256 chains, the metric's; c5 for --scee and --slmc)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="arithmetic of the headline arm (mixed: complex sweeps only; t-V runs fp64)")
    ap.add_argument("--slmc", action="store_true",
                    help="self-learning cluster moves against local updates (t-U workloads; prints its own line)")
    ap.add_argument("--scee", action="store_true",
                    help="coupled SCEE sweep of replica pairs (t-U workloads; prints its own line)")
    ap.add_argument("--slmc-scan", action="store_true",
                    help="local updates vs learned cluster moves on a small t-U lattice over --scan-u")
    ap.add_argument("--scan-site", default="2,4", help="SQUARE45 site of --slmc-scan (2,4: the 4x4 torus)")
    ap.add_argument("--scan-u", default="4,8,12,16", help="couplings U/t of --slmc-scan")
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
    if args.workload is None:
        args.workload = "c5" if (args.scee or args.slmc) else "c3"
    WL = WORKLOADS[args.workload]
    NCHAINS = args.chains or WL["chains"]
    PRECISION = args.precision if make_model().is_complex else "fp64"
    if args.group:
        run_group(args)
    elif args.scee:
        run_scee(args)
    elif args.slmc:
        run_slmc(args)
    elif args.slmc_scan:
        run_slmc_scan(args)
    elif args.tau_run:
        run_tau(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
