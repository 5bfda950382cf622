"""Benchmark of the GB300 adaptive embedded-RK N-body integrator.

Workload (one GPU): one N = 16384 Plummer sphere (scale radius 1, velocities
from the distribution function, seed 101), softening 0.005, the 13-stage
Fehlberg 7(8) pair, atol = rtol = 1e-8, t in [0, 2], FP32 pair forces on
hi/lo positions (hi/lo differences for close pairs) with Kahan-compensated
accumulation, FP64 state / stage combination / norm.
A step is one whole integration t = 0 -> 2 from the seeded state (about 150
adaptive attempts): the initial-step estimate on the device, then attempts of
13 fused stage kernels (force + next-stage combination) and one controller
kernel, replayed 16 attempts per CUDA graph with the state resident in HBM.
value = accepted steps per second of device time (the host's polls between
graph replays included).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU implementation of the path (the
thread-pool executor restated in oracle/, all host threads) on the same
workload, one reference attempt per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {
    "workload": "plummer16384_rkf78_mixed",
    "n_particles": 16384,
    "model": "Plummer sphere a=1, G=1, equal masses 1/N",
    "seed": 101,
    "softening": 0.005,
    "tableau": "RKF78",
    "atol": 1e-8,
    "rtol": 1e-8,
    "t0": 0.0,
    "tf": 2.0,
    "precision": "mixed",
}
METRIC = "accepted steps/s and pair-interactions/s at equal energy error: learned+mixed vs FP64"
FP32_LANES_PER_SM = 128
FLOPS_PER_INTERACTION = 20  # Nyland, Harris & Prins (GPU Gems 3, ch. 31) convention
# FP32-pipe operations per interaction of the pair term: 3 for the hi-only
# differences, 3 FMA for r^2 + eps^2, 2 multiplies for r^-3, 3 FMA
# accumulations (rsqrt runs on the SFU), plus the hi/lo revisit of close
# pairs (a few per cent of them, ~20 operations each): ~11.5.  The 20-FLOP
# convention counts 10 FMA-equivalents, so the FP32 pipe caps the fraction
# near 10/11.5.
HILO_FP32_OPS = 11.5
# DRAM bytes (read + write) of one headline stage launch from an ncu capture
# of the same kernel and geometry (python bench.py --workload stage).
STAGE_DRAM_BYTES_16384 = 2542592
FP64_TFLOPS_NOMINAL = 1.25  # GB300 FP64 (non-tensor), one FMA = 2 FLOP


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_gpu{gpu_index}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "samples": len(sm), "reasons": sorted(reasons)}


def load_mlp(args):
    if args.controller != "learned":
        return None
    import ode_prototyping_gb300 as gb
    path = args.mlp or os.path.join(ROOT, "ode_prototyping_gb300", "weights",
                                   "proposer_plummer16384_rkf78.bin")
    return gb.GbMlp.from_buffer_copy(open(path, "rb").read())


def drift(e0: dict, e1: dict) -> dict:
    """Conservation diagnostics between two states (FP64 device kernel):
    relative energy error, and the change of total momentum and angular
    momentum (absolute; both start near zero in the centre-of-mass frame)."""
    return {"energy_rel_err": abs(e1["e"] - e0["e"]) / abs(e0["e"]),
            "momentum_drift": float(np.linalg.norm(e1["p"] - e0["p"])),
            "angular_momentum_drift": float(np.linalg.norm(e1["l"] - e0["l"]))}


def stage_kernel_name(precision: str, geo: dict) -> str:
    """The integrator's stage kernel for a geometry: one-lane packed mixed
    stages run as independent partner chunks, everything else as clusters."""
    if precision == "mixed" and geo["lanes"] == 1 and geo["j_split"] > 1 \
            and geo["mixed_variant"] != 1:
        return f"fused_split_kernel (mixed, one stage, {geo['j_split']} partner chunks per tile)"
    return f"fused_stage_kernel ({precision}, one stage)"


def c1_cpu_baseline(x0: np.ndarray, n: int, eps: float, tol: float) -> dict:
    """The reference's thread-pool loop (restated in oracle/) over the whole
    C1 integration t = 0 -> 1 on all host threads, host clock."""
    import oracle
    threads = os.cpu_count() or 1
    ode, _ = oracle.nbody_ode(n, eps, 1.0 / n)
    sess = oracle.Session("DOPRI5", ode, x0, 0.0, 1.0, tol, tol, threads)
    t0 = time.perf_counter()
    accepted = attempts = 0
    while True:
        done, a = sess.attempt()
        if done:
            break
        attempts += 1
        accepted += int(a)
    wall = time.perf_counter() - t0
    sess.close()
    return {"value": accepted / wall, "unit": "accepted steps/s", "cores": threads,
            "kind": "port", "seconds": wall, "accepted": accepted, "attempts": attempts,
            "sample": f"the whole C1 integration (N={n}, DOPRI5, tol {tol:g}, t in [0, 1]) by "
                      f"the reference thread-pool loop restated in oracle/gbode_oracle.c on "
                      f"{threads} host threads"}


def aggregate_over_ranks(accepted: float, rhs: float, ms: float, device: str = "cuda"):
    """Whole-job totals over replicas (one independent system per GPU):
    accepted steps and RHS evaluations summed, device time = max over ranks."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return accepted, rhs, ms
    tt = torch.tensor([accepted, rhs], dtype=torch.float64, device=device)
    dist.all_reduce(tt)
    tm = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(tm, op=dist.ReduceOp.MAX)
    return float(tt[0]), float(tt[1]), float(tm[0])


def replica_seed(rank: int) -> int:
    """Seed of the system rank `rank` integrates (replicas are independent)."""
    return WORKLOAD["seed"] + rank


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args, world, rank):
    """The reference's CPU implementation (thread-pool executor, restated in
    oracle/), one adaptive attempt per step, all host threads."""
    if rank != 0:
        return
    import oracle
    import ode_prototyping_gb300 as gb
    W = WORKLOAD
    n = W["n_particles"]
    x0 = gb.ic_plummer(n, W["seed"], 1.0)
    threads = os.cpu_count() or 1
    ode, _ = oracle.nbody_ode(n, W["softening"], 1.0 / n)
    sess = oracle.Session(W["tableau"], ode, x0, W["t0"], W["tf"], W["atol"], W["rtol"],
                          threads)
    budget_s = float(os.environ.get("GBODE_REF_BUDGET_S", "200"))
    t_start = time.perf_counter()
    # at least three untimed attempts: the loop's first attempts from the
    # initial-step estimate are rejections (start-up, not the steady rate)
    for _ in range(max(args.warmup, 3)):
        sess.attempt()
        if time.perf_counter() - t_start > budget_s / 3:
            break
    s0 = sess.stats()
    done_steps, acc, t_tot = 0, 0, 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        done, a = sess.attempt()
        t_tot += time.perf_counter() - t0
        if done:
            break
        done_steps += 1
        acc += int(a)
        if time.perf_counter() - t_start > budget_s:
            break
    s1 = sess.stats()
    rhs = s1["n_rhs"] - s0["n_rhs"]
    value = acc / t_tot if t_tot > 0 else 0.0
    sample = (f"{done_steps} attempts of the thread-pool reference loop restated in "
              f"oracle/gbode_oracle.c on {threads} host threads, N={n}, {W['tableau']}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "accepted steps/s",
        "n_gpus": args.gpus, "steps": done_steps, "steps_requested": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_tot / max(done_steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": dict(W, precision="f64 (reference CPU path)"),
        "pair_interactions_per_s": rhs * n * (n - 1) / t_tot if t_tot > 0 else 0.0,
        "cpu_baseline": {"value": value, "unit": "accepted steps/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "accepted steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    sess.close()
    print(json.dumps(line), flush=True)


def cpu_baseline(attempts_per_accepted: float) -> dict:
    """Bounded sample of the same workload on the host cores: one attempt of
    the reference's thread-pool loop (restated in oracle/, all host threads)
    from the seeded state, after its initial-step estimate, timed with the
    host clock.  Scaled to accepted steps/s with the trajectory's attempts per
    accepted step (the same algorithm, measured on the whole integration)."""
    import oracle
    import ode_prototyping_gb300 as gb
    W = WORKLOAD
    n = W["n_particles"]
    threads = os.cpu_count() or 1
    x0 = gb.ic_plummer(n, W["seed"], 1.0)
    ode, _ = oracle.nbody_ode(n, W["softening"], 1.0 / n)
    sess = oracle.Session(W["tableau"], ode, x0, W["t0"], W["tf"], W["atol"], W["rtol"],
                          threads)
    s0 = sess.stats()
    t0 = time.perf_counter()
    sess.attempt()
    t_att = time.perf_counter() - t0
    s1 = sess.stats()
    sess.close()
    rhs = s1["n_rhs"] - s0["n_rhs"]
    return {"value": 1.0 / (t_att * attempts_per_accepted), "unit": "accepted steps/s",
            "cores": threads, "kind": "port",
            "sample": f"1 attempt ({rhs} RHS, {t_att:.2f} s) of the reference thread-pool loop "
                      f"restated in oracle/, N={n} {W['tableau']}, on {threads} host threads; "
                      f"accepted steps/s = 1 / (seconds per attempt x "
                      f"{attempts_per_accepted:.4f} attempts per accepted step over the whole "
                      f"t0..tf trajectory of the same algorithm)",
            "seconds_per_attempt": t_att,
            "pair_interactions_per_s": rhs * n * (n - 1) / t_att}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--controller", default="reference", choices=["reference", "pi", "learned"])
    ap.add_argument("--mlp", default=None, help="trained proposer weights (learned controller)")
    ap.add_argument("--n-bodies", type=int, default=16384, help="stage: bodies")
    ap.add_argument("--stage-precision", default="mixed", choices=["mixed", "f64"],
                    help="stage: precision of the integrator")
    ap.add_argument("--tol", type=float, default=1e-9, help="c2_tol: atol = rtol")
    ap.add_argument("--learned-config", default="plummer4096_rkf78",
                    help="c4: proposer training/evaluation configuration")
    ap.add_argument("--workload", default="c2",
                    choices=["c2", "c2_f64", "c2_tol", "c1", "c3", "c4", "c5a", "c5b", "rk_hbm",
                             "stage"],
                    help="c2 (default, the headline), or another configuration")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload != "c2":
        run_other_workload(args)
        return

    import torch
    import ode_prototyping_gb300 as gb
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    W = WORKLOAD
    n = W["n_particles"]
    eps = W["softening"]
    seed = replica_seed(rank)  # replicas: an independent system per GPU
    x0 = gb.ic_plummer(n, seed, 1.0)
    stream = torch.cuda.Stream()
    ode = gb.NBodyODE(n, eps, 1.0 / n)
    A = 16
    exe = gb.Gb300Executor(precision=W["precision"], controller=args.controller,
                           attempts_per_sync=A, mlp=load_mlp(args))
    S = gb.tableau(W["tableau"]).n_stages
    it = gb.Integrator(W["tableau"], ode, exe, stream=stream)
    x0_dev = gb.to_device(x0)
    e0 = gb.energy(x0_dev, n, eps, 1.0 / n)

    def one_job():
        """One step: the whole integration t0 -> tf from the seeded state."""
        it.start(x0_dev, W["t0"], W["tf"], W["atol"], W["rtol"])
        rc = it.advance(0)
        if rc != 0:
            raise RuntimeError(f"integration failed with status {rc}")
        return it.stats()

    for _ in range(max(args.warmup, 0)):
        one_job()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    accepted = attempts = rhs = 0
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(k & 0xFF)  # L2 flushed between timed steps
            ev0[k].record(stream)
            st = one_job()
            ev1[k].record(stream)
            accepted += st["n_accepted"]
            attempts += st["n_attempts"]
            rhs += st["n_rhs"]
    stream.synchronize()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = sum(a.elapsed_time(b) for a, b in zip(ev0, ev1))
    xs, t_now = it.state()
    e1 = gb.energy(xs, n, eps, 1.0 / n)
    cons = drift(e0, e1)
    energy_err = cons["energy_rel_err"]
    per_job = {"accepted": accepted // max(args.steps, 1), "attempts": attempts // max(args.steps, 1),
               "rhs_evals": rhs // max(args.steps, 1)}
    # launches per job: start-up kernels + graph replays of A attempts x (S + 1)
    replays = -(-per_job["attempts"] // A)
    launches_per_job = 12 + replays * A * (S + 1)
    # whole-job aggregate over ranks: accepted steps summed, time = max
    acc_all, rhs_all, ms_max = aggregate_over_ranks(float(accepted), float(rhs), ms)
    value = acc_all / (ms_max / 1e3)
    pair_rate = rhs_all * n * (n - 1) / (ms_max / 1e3)

    # dominant kernel: the fused stage kernel, timed alone on its stream on a
    # live integrator (restarted, so no launch finds the integration finished)
    it.start(x0_dev, W["t0"], W["tf"], W["atol"], W["rtol"])
    geo = it.geometry()
    reps = 20
    ks0 = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    ks1 = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    with torch.cuda.stream(stream):
        for r in range(reps):
            flush.fill_(r & 0xFF)
            ks0[r].record(stream)
            it.launch_stage(1 + r % (S - 2))
            ks1[r].record(stream)
    stream.synchronize()
    k_ms = statistics.mean(a.elapsed_time(b) for a, b in zip(ks0, ks1))
    achieved = FLOPS_PER_INTERACTION * n * (n - 1) / (k_ms / 1e3) / 1e12
    pk, pk_kind = peaks()
    sm_mhz_max = float(pk.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = n_sm * FP32_LANES_PER_SM * 2 * sm_mhz_max * 1e6 / 1e12
    it.close()

    line = {
        "metric": METRIC, "value": value, "unit": "accepted steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": {**W, "controller": args.controller, "parallelism": f"replicas{world}",
                   "l2": "flushed between timed steps (256 MiB write)",
                   "step": "one whole integration t0 -> tf from the seeded state: initial "
                           "step on the device, then attempts of 13 fused stage kernels + "
                           "1 controller kernel replayed 16 per CUDA graph"},
        "pair_interactions_per_s": pair_rate,
        "per_step": per_job, "rejected_fraction": 1 - accepted / max(attempts, 1),
        "t_reached": t_now, "energy_rel_err": energy_err,
        "momentum_drift": cons["momentum_drift"],
        "angular_momentum_drift": cons["angular_momentum_drift"],
        "clocks": clocks,
        "gpu_launches": args.steps * launches_per_job,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": STAGE_DRAM_BYTES_16384 if n == 16384 else None,
                     "traffic_note": "DRAM bytes per launch from one ncu capture of this "
                                     "kernel (compute-bound: positions + stage rows mostly "
                                     "served from L2)",
                     "kernel": stage_kernel_name(W["precision"], geo),
                     "kernel_ms": k_ms, "geometry": geo,
                     "peak_note": f"nominal FP32 pipe: {n_sm} SMs x {FP32_LANES_PER_SM} lanes x 2"
                                  f" x {sm_mhz_max:.0f} MHz ({pk_kind} peaks file has no FP32)",
                     "flops_per_interaction": FLOPS_PER_INTERACTION,
                     "fp32_ops_per_interaction": HILO_FP32_OPS,
                     "fp32_pipe_cap_frac": FLOPS_PER_INTERACTION / 2 / HILO_FP32_OPS},
    }
    if rank == 0:
        line["e2e"] = e2e(gb, torch, x0)
        if not args.no_fp64:
            line["fp64_comparison"] = fp64_compare(gb, torch, x0, line)
            line["equal_energy_le_1e-8"] = energy_target_compare(gb, torch, x0)
        if not args.no_cpu_baseline:
            try:
                line["cpu_baseline"] = cpu_baseline(attempts / max(accepted, 1))
            except Exception as ex:  # reported, not fatal
                line["cpu_baseline"] = {"value": None, "error": repr(ex)}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def _timed(torch, stream, fn, steps, flush):
    """Device time of `steps` calls of fn on `stream`, L2 flushed before each."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    out = []
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.fill_(k & 0xFF)
            ev[k][0].record(stream)
            out.append(fn())
            ev[k][1].record(stream)
    stream.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev), out


def _batch_ics(gb, torch, sizes, seeds, kind, eps):
    xs = []
    for n, seed, e in zip(sizes, seeds, eps):
        if kind == "virial":
            x = gb.ic_plummer(int(n), int(seed))
            q = 0.5 + np.random.default_rng(int(seed)).uniform()  # virial ratio in [0.5, 1.5)
            en = gb.energy(x, int(n), e, 1.0 / n)
            x[3 * int(n):] *= np.sqrt(q * abs(en["pe"]) / (2.0 * en["ke"]))
        else:
            x = gb.ic_binary_plummer(int(n), int(seed), 0.1, 1e-3, 1e-2)
        xs.append(x)
    return np.concatenate(xs)


def run_other_workload(args):
    """The other configurations: c1 (the plain FP64 method, N = 1024), c3
    (512-system batch), c5a (N = 262144 cold collapse), c5b (64 binary-rich
    N = 8192 systems).  One JSON line each, same keys as the headline."""
    import torch
    import ode_prototyping_gb300 as gb
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    line = {"metric": METRIC, "unit": "accepted steps/s", "n_gpus": 1, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "data": "synthetic", "warmup": args.warmup}
    if args.workload == "c2_f64":
        # the plain FP64 GB300 path over the whole headline trajectory
        W = WORKLOAD
        n, eps = W["n_particles"], W["softening"]
        x0 = gb.to_device(gb.ic_plummer(n, W["seed"], 1.0))
        it = gb.Integrator(W["tableau"], gb.NBodyODE(n, eps, 1.0 / n),
                           gb.Gb300Executor(precision="f64", attempts_per_sync=16), stream=stream)

        def job():
            it.start(x0, W["t0"], W["tf"], W["atol"], W["rtol"])
            assert it.advance(0) == 0
            return it.stats()
        ms, st = _timed(torch, stream, job, 1, flush)
        e0 = gb.energy(x0, n, eps, 1.0 / n)
        e1 = gb.energy(it.state()[0], n, eps, 1.0 / n)
        line.update(value=st[0]["n_accepted"] / (ms / 1e3), dtype="f64", steps=1,
                    ms_per_step=ms, warmup=0,
                    pair_interactions_per_s=st[0]["n_rhs"] * n * (n - 1) / (ms / 1e3),
                    per_step={"accepted": st[0]["n_accepted"], "attempts": st[0]["n_attempts"],
                              "rhs": st[0]["n_rhs"]},
                    **drift(e0, e1),
                    config={**W, "precision": "f64", "step": "whole integration"})
        it.close()
    elif args.workload == "c2_tol":
        # The headline system integrated t = 0 -> 2 by the mixed path and by the
        # plain FP64 path at a tighter tolerance (--tol), each once: accepted
        # steps/s and the conservation diagnostics of both, so the two are
        # compared at an energy error below 1e-8.
        W = WORKLOAD
        n, eps = W["n_particles"], W["softening"]
        x0 = gb.to_device(gb.ic_plummer(n, W["seed"], 1.0))
        e0 = gb.energy(x0, n, eps, 1.0 / n)
        res = {}
        for prec in ("mixed", "f64"):
            it = gb.Integrator(W["tableau"], gb.NBodyODE(n, eps, 1.0 / n),
                               gb.Gb300Executor(precision=prec, attempts_per_sync=16),
                               stream=stream)

            def job():
                it.start(x0, W["t0"], W["tf"], args.tol, args.tol)
                assert it.advance(0) == 0
                return it.stats()
            if prec == "mixed":
                job()  # warm-up
            ms, st = _timed(torch, stream, job, 1, flush)
            e1 = gb.energy(it.state()[0], n, eps, 1.0 / n)
            res[prec] = {"accepted_steps_per_s": st[0]["n_accepted"] / (ms / 1e3),
                         "accepted": st[0]["n_accepted"], "attempts": st[0]["n_attempts"],
                         "ms": ms, **drift(e0, e1)}
            it.close()
        line.update(value=res["mixed"]["accepted_steps_per_s"], dtype="f32+f64", steps=1,
                    ms_per_step=res["mixed"]["ms"], warmup=1, paths=res,
                    speedup_mixed_vs_f64=res["mixed"]["accepted_steps_per_s"]
                    / res["f64"]["accepted_steps_per_s"],
                    config={**W, "atol": args.tol, "rtol": args.tol,
                            "workload": "plummer16384_rkf78_tight_tolerance",
                            "step": "one whole integration per path"})
    elif args.workload == "c1":
        n, eps, tol = 1024, 0.01, 1e-10
        x0 = gb.to_device(gb.ic_uniform_ball(n, 1, 0.1))
        it = gb.Integrator("DOPRI5", gb.NBodyODE(n, eps, 1.0 / n),
                           gb.Gb300Executor(precision="f64", attempts_per_sync=16), stream=stream)

        def job():
            it.start(x0, 0.0, 1.0, tol, tol)
            assert it.advance(0) == 0
            return it.stats()
        for _ in range(args.warmup):
            job()
        ms, st = _timed(torch, stream, job, args.steps, flush)
        acc = sum(s["n_accepted"] for s in st)
        rhs = sum(s["n_rhs"] for s in st)
        e0 = gb.energy(x0, n, eps, 1.0 / n)
        e1 = gb.energy(it.state()[0], n, eps, 1.0 / n)
        line.update(value=acc / (ms / 1e3), dtype="f64", steps=args.steps,
                    ms_per_step=ms / args.steps, pair_interactions_per_s=rhs * n * (n - 1) / (ms / 1e3),
                    per_step={"accepted": st[0]["n_accepted"], "attempts": st[0]["n_attempts"],
                              "rhs": st[0]["n_rhs"]},
                    **drift(e0, e1),
                    cpu_baseline=c1_cpu_baseline(gb.ic_uniform_ball(n, 1, 0.1), n, eps, tol),
                    config={"workload": "ball1024_dopri5_f64", "n_particles": n, "softening": eps,
                            "tableau": "DOPRI5", "atol": tol, "rtol": tol, "t": [0, 1],
                            "step": "whole integration"})
        it.close()
    elif args.workload in ("c3", "c5b"):
        if args.workload == "c3":
            rng = np.random.default_rng(303)
            sizes = np.round(np.exp(rng.uniform(np.log(64), np.log(4096), 512))).astype(np.int64)
            eps = 0.01 * 4.0 / np.cbrt(sizes)
            x0 = _batch_ics(gb, torch, sizes, 3000 + np.arange(512), "virial", eps)
            tab, tol, tf = "DOPRI5", 1e-9, 1.0
        else:
            sizes = np.full(64, 8192, dtype=np.int64)
            eps = np.full(64, 1e-4)
            x0 = _batch_ics(gb, torch, sizes, 6000 + np.arange(64), "binary", eps)
            tab, tol, tf = "DOPRI5", 1e-8, 0.002
        x0d = gb.to_device(x0)
        res = {}
        for prec in ("mixed", "f64"):
            b = gb.Batch(tab, sizes, eps, precision=prec, attempts_per_sync=8, stream=stream)
            b.start(x0d, 0.0, tf, tol, tol)
            tune = b.autotune(2)
            limit = 0 if prec == "mixed" else 3  # FP64: a bounded window of graph replays

            def job():
                b.start(x0d, 0.0, tf, tol, tol)
                b.advance(limit)
                return b.stats()
            if prec == "mixed":
                for _ in range(args.warmup):
                    job()
            ms, st = _timed(torch, stream, job, args.steps if prec == "mixed" else 1, flush)
            acc = sum(s["n_accepted"] for s in st)
            inter = sum(s["interactions"] for s in st)
            res[prec] = {"accepted_steps_per_s": acc / (ms / 1e3),
                         "pair_interactions_per_s": inter / (ms / 1e3),
                         "ms_per_step": ms / len(st), "geometry": tune,
                         "accepted": st[0]["n_accepted"], "attempts": st[0]["n_attempts"],
                         "t_min": st[0]["t"], "done": st[0]["done"]}
            b.close()
        line.update(value=res["mixed"]["accepted_steps_per_s"], dtype="f32+f64",
                    steps=args.steps, ms_per_step=res["mixed"]["ms_per_step"],
                    pair_interactions_per_s=res["mixed"]["pair_interactions_per_s"],
                    fp64_comparison=res,
                    config={"workload": args.workload, "systems": int(len(sizes)),
                            "n_min": int(sizes.min()), "n_max": int(sizes.max()),
                            "bodies": int(sizes.sum()), "tableau": tab, "atol": tol,
                            "rtol": tol, "t": [0, tf], "step": "whole batch integration"})
    elif args.workload == "stage":
        # Four stage launches of the headline integrator on an N-body Plummer
        # sphere (a small case for profiling the fused stage kernel).
        n = args.n_bodies
        x0 = gb.to_device(gb.ic_plummer(n, WORKLOAD["seed"], 1.0))
        it = gb.Integrator(WORKLOAD["tableau"], gb.NBodyODE(n, WORKLOAD["softening"], 1.0 / n),
                           gb.Gb300Executor(precision=args.stage_precision, attempts_per_sync=1),
                           stream=stream)
        it.start(x0, WORKLOAD["t0"], WORKLOAD["tf"], WORKLOAD["atol"], WORKLOAD["rtol"])
        ms, _ = _timed(torch, stream, lambda: it.launch_stage(1), 1, flush)
        with torch.cuda.stream(stream):
            for r in range(3):
                it.launch_stage(2 + r)
        stream.synchronize()
        line.update(metric="fused stage kernel, one launch", unit="ms", value=ms,
                    higher_is_better=False, steps=1, ms_per_step=ms,
                    dtype="f32+f64" if args.stage_precision == "mixed" else "f64",
                    geometry=it.geometry(),
                    config={"workload": f"plummer{n}_rkf78_{args.stage_precision}_stage",
                            "n_particles": n,
                            "step": "one fused stage launch (four launched)"})
        it.close()
    elif args.workload == "c4":
        # Learned step-size proposer: trained on seed set A (weights shipped in
        # ode_prototyping_gb300/weights/, retrained here if absent), evaluated
        # on held-out seed set B against the reference and PI controllers.
        from ode_prototyping_gb300 import learned
        cfg = args.learned_config
        path = os.path.join(ROOT, "ode_prototyping_gb300", "weights", f"proposer_{cfg}.bin")
        trained_here = not os.path.exists(path)
        if trained_here:
            m, _ = learned.train_config(cfg)
        else:
            m = gb.GbMlp.from_buffer_copy(open(path, "rb").read())
        ev = learned.evaluate_config(cfg, m)
        c = learned.CONFIGS[cfg]
        lrn = ev["learned"]
        line.update(value=lrn["accepted"] / lrn["wall_s"], dtype="f32+f64", steps=1,
                    ms_per_step=1e3 * lrn["wall_s"], controllers=ev,
                    config={"workload": f"learned_proposer_{cfg}", **c,
                            "train_seeds": "A = 1..8", "eval_seeds": "B = 101..104",
                            "weights": "trained in this run" if trained_here else path[len(ROOT) + 1:],
                            "step": "whole integrations of the held-out systems"})
    elif args.workload == "rk_hbm":
        # The standalone element-wise kernels of one RKF78 attempt on vectors of
        # 2^24 doubles (128 MiB each, beyond L2): stage combinations, update and
        # error, error target, scaled norm.  Two ceilings per kernel: HBM
        # (algorithmic bytes = every vector element read or written once,
        # against the measured copy bandwidth) and the FP64 pipe (the IEEE
        # multiply and add per coefficient that bit-for-bit parity needs; a
        # division counted as ~9 FP64 instructions of a Newton-Raphson
        # sequence; GB300: 1.25 TFLOP/s = 0.625e12 FP64 instructions/s).
        import ctypes as C
        pk, src = peaks()
        fp64_ips = FP64_TFLOPS_NOMINAL * 1e12 / 2
        nv = 1 << 24
        t = gb.tableau("RKF78")
        S = t.n_stages
        g = torch.Generator(device="cuda").manual_seed(7)
        ks = torch.randn(S * nv, dtype=torch.float64, device="cuda", generator=g)
        x0 = torch.randn(nv, dtype=torch.float64, device="cuda", generator=g)
        out, x, err, tg = (torch.empty_like(x0) for _ in range(4))
        atol = torch.full_like(x0, 1e-8)
        rtol = torch.full_like(x0, 1e-8)
        nb = gb.lib().gb_rk_norm_workspace_bytes(nv)
        work = torch.empty(nb, dtype=torch.uint8, device="cuda")
        res_d = torch.zeros(1, dtype=torch.float64, device="cuda")
        sp = gb._stream(stream)
        nb_b = sum(1 for j in range(S) if t.b[j] != 0.0)
        nb_d = sum(1 for j in range(S) if t.b[j] != t.bt[j])
        nb_u = sum(1 for j in range(S) if t.b[j] != 0.0 or t.b[j] != t.bt[j])
        cases = []
        for s in range(1, S):
            nnz = sum(1 for j in range(s) if t.a[s - 1][j] != 0.0)
            cases.append((f"rk_stage_{s}", 8 * nv * (nnz + 2), nv * (2 * nnz + 2),
                          lambda s=s: gb.rk_stage(t, s, 1e-3, x0, ks, out, nv, stream)))
        cases.append(("rk_update_state_and_error", 8 * nv * (nb_u + 3),
                      nv * (2 * nb_b + 2 * nb_d + 3),
                      lambda: gb.rk_update(t, 1e-3, x0, ks, x, err, nv, stream)))
        cases.append(("rk_error_target", 8 * nv * 5, nv * 2,
                      lambda: gb.rk_error_target(atol, rtol, x, x0, tg, nv, stream)))
        cases.append(("rk_norm", 8 * nv * 2, nv * (9 + 2),
                      lambda: gb.check(gb.lib().gb_rk_norm_f64(
                          C.c_void_p(err.data_ptr()), C.c_void_p(tg.data_ptr()), nv,
                          C.c_void_p(work.data_ptr()), nb, C.c_void_p(res_d.data_ptr()), sp),
                          "gb_rk_norm_f64")))
        rows = {}
        for name, nbytes, nops, fn in cases:
            for _ in range(max(args.warmup, 3)):
                fn()
            ms, _ = _timed(torch, stream, fn, args.steps, flush)
            sec = ms / args.steps / 1e3
            hbm = nbytes / sec / 1e9 / pk["hbm_gbs"]
            f64 = nops / sec / fp64_ips
            rows[name] = {"bytes": nbytes, "fp64_instr": nops, "us": 1e6 * sec,
                          "GB/s": nbytes / sec / 1e9, "hbm_frac": hbm, "fp64_frac": f64,
                          "bound": "fp64" if nops / fp64_ips > nbytes / (pk["hbm_gbs"] * 1e9)
                          else "hbm"}
        tot_us = sum(r["us"] for r in rows.values())
        tot_b = sum(r["bytes"] for r in rows.values())
        tot_o = sum(r["fp64_instr"] for r in rows.values())
        floor_us = sum(1e6 * max(r["fp64_instr"] / fp64_ips, r["bytes"] / (pk["hbm_gbs"] * 1e9))
                       for r in rows.values())
        line.update(metric="element-wise RK kernels of one RKF78 attempt, n_var = 2^24",
                    unit="GB/s", value=tot_b / (tot_us / 1e6) / 1e9, dtype="f64",
                    steps=args.steps, ms_per_step=tot_us / 1e3, kernels=rows,
                    roofline={"bound": "fp64 (stage sums, update, norm) / hbm (target)",
                              "achieved_us": tot_us, "floor_us": floor_us,
                              "frac": floor_us / tot_us, "hbm_peak_gbs": pk["hbm_gbs"],
                              "fp64_peak_instr_per_s": fp64_ips, "peak_source": src,
                              "fp64_instr": tot_o},
                    config={"workload": "rkf78_elementwise_nvar16777216", "n_var": nv,
                            "tableau": "RKF78", "l2": "flushed (256 MiB write) before each call"})
    else:  # c5a
        n, eps, tol = 262144, 0.002, 1e-8
        x0 = gb.to_device(gb.ic_cold_sphere(n, 505, 0.01))
        it = gb.Integrator("DOPRI5", gb.NBodyODE(n, eps, 1.0 / n),
                           gb.Gb300Executor(precision="mixed", attempts_per_sync=1),
                           stream=stream)
        it.start(x0, 0.0, 1.0, tol, tol)
        it.enqueue(max(args.warmup, 1))
        it.sync()
        s0 = it.stats()
        ms, _ = _timed(torch, stream, lambda: it.enqueue(1), args.steps, flush)
        it.sync()
        s1 = it.stats()
        acc = s1["n_accepted"] - s0["n_accepted"]
        rhs = s1["n_rhs"] - s0["n_rhs"]
        xs, t = it.state()
        it.close()
        # accelerations of the mixed path against FP64 on the current state
        f64 = gb.nbody_rhs_f64(xs, n, eps, 1.0 / n)
        mx = gb.nbody_rhs_mixed(xs, n, eps, 1.0 / n)
        a64, amx = f64[3 * n:].view(-1, 3), mx[3 * n:].view(-1, 3)
        rel = ((amx - a64).norm() / a64.norm()).item()
        per = ((amx - a64).norm(dim=1) / a64.norm(dim=1)).median().item()
        line.update(value=acc / (ms / 1e3), dtype="f32+f64", steps=args.steps,
                    ms_per_step=ms / args.steps,
                    pair_interactions_per_s=rhs * n * (n - 1) / (ms / 1e3),
                    accepted=acc, t_reached=t, acc_rel_err_normwise=rel,
                    acc_rel_err_median=per,
                    config={"workload": "cold_collapse262144_dopri5_mixed", "n_particles": n,
                            "softening": eps, "tableau": "DOPRI5", "atol": tol, "rtol": tol,
                            "step": "one adaptive attempt"})
    print(json.dumps(line), flush=True)


def e2e(gb, torch, x0: np.ndarray, reps: int = 3) -> dict:
    """Same metric through the public API from host memory: pinned host state
    -> device, integrator creation + initial step + the whole integration,
    final state -> host; host clock around everything.  Each of `reps` runs
    is one such call; value = the median run."""
    W = WORKLOAD
    n = W["n_particles"]
    host = torch.from_numpy(x0).pin_memory()
    out = torch.empty(6 * n, dtype=torch.float64).pin_memory()
    runs = []
    for _ in range(max(reps, 1)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev = host.to("cuda", non_blocking=True)
        exe = gb.Gb300Executor(precision=W["precision"], attempts_per_sync=16)
        it = gb.Integrator(W["tableau"], gb.NBodyODE(n, W["softening"], 1.0 / n), exe)
        it.start(dev, W["t0"], W["tf"], W["atol"], W["rtol"])
        it.advance(0)
        xs, _ = it.state()
        out.copy_(xs)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        st = it.stats()
        it.close()
        runs.append(st["n_accepted"] / wall)
    return {"value": statistics.median(runs), "unit": "accepted steps/s",
            "h2d_bytes_per_step": 6 * n * 8, "d2h_bytes_per_step": 6 * n * 8,
            "attempts": st["n_attempts"], "runs": runs,
            "note": "per run: one whole integration through the public API; creation, "
                    "initial-step estimate and graph build inside the timed region; "
                    "value = median of the runs"}


def fp64_compare(gb, torch, x0, line, k: int = 6) -> dict:
    """The plain FP64 GB300 path on the same workload, same tolerance, for k
    attempts (its throughput), and the mixed path over the same k attempts
    (energy error over the same interval)."""
    W = WORKLOAD
    n = W["n_particles"]
    res = {}
    for prec in ("f64", "mixed"):
        stream = torch.cuda.Stream()
        exe = gb.Gb300Executor(precision=prec, attempts_per_sync=1)
        it = gb.Integrator(W["tableau"], gb.NBodyODE(n, W["softening"], 1.0 / n), exe,
                           stream=stream)
        it.start(x0, W["t0"], W["tf"], W["atol"], W["rtol"])
        it.sync()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        s0 = it.stats()
        a.record(stream)
        it.enqueue(k)
        b.record(stream)
        stream.synchronize()
        it.sync()
        s1 = it.stats()
        xs, t = it.state()
        e0 = gb.energy(x0, n, W["softening"], 1.0 / n)
        e1 = gb.energy(xs, n, W["softening"], 1.0 / n)
        ms = a.elapsed_time(b)
        res[prec] = {"accepted_steps_per_s": (s1["n_accepted"] - s0["n_accepted"]) / (ms / 1e3),
                     "attempts": k, "t_reached": t,
                     **drift(e0, e1), "ms": ms}
        res[prec + "_state"] = xs
        it.close()
    diff = (res["mixed_state"] - res["f64_state"]).abs().max().item()
    del res["mixed_state"], res["f64_state"]
    res["max_state_diff_mixed_vs_f64"] = diff
    res["speedup_mixed_vs_f64"] = (res["mixed"]["accepted_steps_per_s"] /
                                   max(res["f64"]["accepted_steps_per_s"], 1e-30))
    return res


def energy_target_compare(gb, torch, x0, tol: float = 1e-11, skip: int = 4,
                          k: int = 8) -> dict:
    """The same system at a tolerance where the relative energy error over
    t0 -> tf is at most 1e-8: the mixed path's whole trajectory with the
    reference controller and with the learned proposer trained at this
    tolerance (energy errors measured), and the plain FP64 path's throughput
    over k attempts at the same tolerance after `skip` untimed start-up
    attempts (the FP64 whole trajectory takes minutes: python bench.py
    --workload c2_tol --tol 1e-11)."""
    W = WORKLOAD
    n = W["n_particles"]
    stream = torch.cuda.Stream()
    out = {"tol": tol}
    # the proposer trained at this tolerance (ode_prototyping_gb300/learned.py)
    mlp = gb.GbMlp.from_buffer_copy(open(os.path.join(
        ROOT, "ode_prototyping_gb300", "weights", "proposer_plummer16384_rkf78_tol1e-11.bin"),
        "rb").read())
    for key in ("mixed", "mixed_learned", "f64"):
        prec = "f64" if key == "f64" else "mixed"
        learned = key == "mixed_learned"
        exe = gb.Gb300Executor(precision=prec, attempts_per_sync=16 if prec == "mixed" else 1,
                               controller="learned" if learned else "reference",
                               mlp=mlp if learned else None)
        it = gb.Integrator(W["tableau"], gb.NBodyODE(n, W["softening"], 1.0 / n), exe,
                           stream=stream)
        it.start(x0, W["t0"], W["tf"], tol, tol)
        it.sync()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        if prec == "f64":
            it.enqueue(skip)
            it.sync()
        s0 = it.stats()
        a.record(stream)
        if prec == "mixed":
            it.advance(0)
        else:
            it.enqueue(k)
        b.record(stream)
        stream.synchronize()
        it.sync()
        s1 = it.stats()
        xs, t = it.state()
        ms = a.elapsed_time(b)
        r = {"accepted_steps_per_s": (s1["n_accepted"] - s0["n_accepted"]) / (ms / 1e3),
             "accepted": s1["n_accepted"] - s0["n_accepted"],
             "attempts": s1["n_attempts"] - s0["n_attempts"],
             "rhs_evals": s1["n_rhs"] - s0["n_rhs"], "t_reached": t, "ms": ms}
        if prec == "mixed":
            e0 = gb.energy(x0, n, W["softening"], 1.0 / n)
            r.update(drift(e0, gb.energy(xs, n, W["softening"], 1.0 / n)))
        else:
            r["window"] = f"{k} attempts after {skip} start-up attempts"
        out[key] = r
        it.close()
    f64 = max(out["f64"]["accepted_steps_per_s"], 1e-30)
    out["speedup_mixed_vs_f64"] = out["mixed"]["accepted_steps_per_s"] / f64
    out["speedup_mixed_learned_vs_f64"] = out["mixed_learned"]["accepted_steps_per_s"] / f64
    out["rhs_saved_learned_vs_reference"] = (1.0 - out["mixed_learned"]["rhs_evals"] /
                                            max(out["mixed"]["rhs_evals"], 1))
    return out


if __name__ == "__main__":
    main()
