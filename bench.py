"""Benchmark of the GB300 adaptive embedded-RK N-body integrator.

Workload (one GPU): the configuration-2 system -- one N = 16384 Plummer
sphere (scale radius 1, velocities from the distribution function, seed 101),
softening 0.005, the 13-stage Fehlberg 7(8) pair, t in [0, 2], FP32 pair
forces on hi/lo positions with Kahan-compensated accumulation, FP64 state /
stage combination / norm -- integrated at atol = rtol = 1e-11, the loosest
tolerance measured at which its relative energy error over t = 0 -> 2 is at
most 1e-8 (the metric's operating point; configuration 2's own 1e-8 gives
~1e-7, reported beside it), with the learned step-size proposer trained at
that tolerance (ode_prototyping_gb300/weights/).
A step is one whole integration t = 0 -> 2 from the seeded state: the
initial-step estimate on the device, then attempts of 13 fused stage kernels
and one controller kernel, replayed 16 attempts per CUDA graph (each replay
re-sorts the bodies along a Morton curve) with the state resident in HBM.
value = accepted steps per second of device time (the host's polls between
graph replays included); time_to_tf_s beside it.  The same line carries the
plain FP64 GB300 path, the mixed path with the reference and PI controllers
and the learned + mixed path, each over the whole trajectory at the same
tolerance with its measured energy error.

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

# configuration 2: the system, its tableau and time span (its tolerance 1e-8
# is CONFIG2_TOL; the headline runs at METRIC_TOL)
CONFIG2_TOL = 1e-8
METRIC_TOL = 1e-11
PROPOSER = "proposer_plummer16384_rkf78_tol1e-11.bin"
WORKLOAD = {
    "workload": "plummer16384_rkf78_learned_mixed_tol1e-11",
    "n_particles": 16384,
    "model": "Plummer sphere a=1, G=1, equal masses 1/N",
    "seed": 101,
    "softening": 0.005,
    "tableau": "RKF78",
    "atol": METRIC_TOL,
    "rtol": METRIC_TOL,
    "t0": 0.0,
    "tf": 2.0,
    "precision": "mixed",
    "controller": "learned",
    "proposer": PROPOSER,
    "energy_target": "relative energy error over t0 -> tf <= 1e-8 (atol = rtol = 1e-11; "
                     "configuration 2's tolerance 1e-8 gives ~1e-7)",
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
STAGE_DRAM_BYTES_16384 = 2652160
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
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix=f"gbode_clocks_gpu{self.gpu}_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
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
        try:
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "samples": len(sm), "reasons": sorted(reasons)}


def load_mlp(path=None):
    """Proposer weights (default: the one trained at the headline tolerance)."""
    import ode_prototyping_gb300 as gb
    path = path or os.path.join(ROOT, "ode_prototyping_gb300", "weights", PROPOSER)
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
    W = WORKLOAD
    n = W["n_particles"]
    x0 = oracle.ic_plummer(n, W["seed"], 1.0)
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
    W = WORKLOAD
    n = W["n_particles"]
    threads = os.cpu_count() or 1
    x0 = oracle.ic_plummer(n, W["seed"], 1.0)
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


def integrate_once(gb, torch, x0_dev, stream, precision: str, controller: str, tol: float,
                   mlp=None):
    """One whole integration t0 -> tf from x0 on `stream`: (device ms, stats,
    final state).  The integrator is created outside the timed region."""
    W = WORKLOAD
    n = W["n_particles"]
    exe = gb.Gb300Executor(precision=precision, controller=controller, attempts_per_sync=16,
                           mlp=mlp if controller == "learned" else None)
    it = gb.Integrator(W["tableau"], gb.NBodyODE(n, W["softening"], 1.0 / n), exe,
                       stream=stream)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a.record(stream)
        it.start(x0_dev, W["t0"], W["tf"], tol, tol)
        rc = it.advance(0)
        b.record(stream)
    stream.synchronize()
    if rc != 0:
        raise RuntimeError(f"{precision}/{controller} integration failed with status {rc}")
    st = it.stats()
    xs, _ = it.state()
    xs = xs.clone()
    it.close()
    return a.elapsed_time(b), st, xs


def arm_record(gb, x0_dev, e0, ms, st, xs) -> dict:
    W = WORKLOAD
    n = W["n_particles"]
    e1 = gb.energy(xs, n, W["softening"], 1.0 / n)
    return {"time_to_tf_s": ms / 1e3, "accepted_steps_per_s": st["n_accepted"] / (ms / 1e3),
            "accepted": st["n_accepted"], "attempts": st["n_attempts"],
            "rejected_fraction": 1 - st["n_accepted"] / max(st["n_attempts"], 1),
            "rhs_evals": st["n_rhs"], "t_reached": st["t"],
            "pair_interactions_per_s": st["n_rhs"] * n * (n - 1) / (ms / 1e3), **drift(e0, e1)}


def metric_arms(gb, torch, x0_dev, e0, headline: dict, mlp) -> dict:
    """The metric: learned + mixed against the plain FP64 GB300 path at equal
    relative energy error <= 1e-8, every arm over the whole trajectory t0 ->
    tf at the same tolerance (the headline's): FP64 with the reference
    controller, mixed with the reference and PI controllers, learned + mixed
    (the headline's own last step).  Speed-ups are ratios of time to tf; the
    accepted-steps/s ratios sit beside them."""
    stream = torch.cuda.Stream()
    out = {"tol": METRIC_TOL, "learned_mixed": headline}
    for key, prec, ctl in (("mixed_reference", "mixed", "reference"), ("mixed_pi", "mixed", "pi"),
                           ("f64_reference", "f64", "reference")):
        ms, st, xs = integrate_once(gb, torch, x0_dev, stream, prec, ctl, METRIC_TOL)
        out[key] = arm_record(gb, x0_dev, e0, ms, st, xs)
    f64 = out["f64_reference"]
    for key in ("learned_mixed", "mixed_reference", "mixed_pi"):
        out[f"speedup_time_to_tf_{key}_vs_f64"] = f64["time_to_tf_s"] / out[key]["time_to_tf_s"]
        out[f"speedup_accepted_steps_per_s_{key}_vs_f64"] = (
            out[key]["accepted_steps_per_s"] / f64["accepted_steps_per_s"])
    out["energy_errors_le_1e-8"] = all(out[k]["energy_rel_err"] <= 1e-8 for k in
                                       ("learned_mixed", "mixed_reference", "mixed_pi",
                                        "f64_reference"))
    out["rhs_saved_learned_vs_reference"] = 1 - headline["rhs_evals"] / max(
        out["mixed_reference"]["rhs_evals"], 1)
    out["rhs_saved_learned_vs_pi"] = 1 - headline["rhs_evals"] / max(
        out["mixed_pi"]["rhs_evals"], 1)
    return out


def config2_tolerance(gb, torch, x0_dev, e0) -> dict:
    """Configuration 2 at its own tolerance (1e-8): the mixed path with the
    reference controller, whole trajectory (energy error ~1e-7)."""
    stream = torch.cuda.Stream()
    integrate_once(gb, torch, x0_dev, stream, "mixed", "reference", CONFIG2_TOL)  # warm-up
    ms, st, xs = integrate_once(gb, torch, x0_dev, stream, "mixed", "reference", CONFIG2_TOL)
    return {"tol": CONFIG2_TOL, "controller": "reference", "precision": "mixed",
            **arm_record(gb, x0_dev, e0, ms, st, xs)}


def pair_force_scale(x0, n: int, eps: float, rows: int = 512) -> np.ndarray:
    """Per body, the sum of the magnitudes of its pair terms (FP64, torch on
    the GPU): m sum_j |x_j - x_i| / (r^2 + eps^2)^(3/2)."""
    import torch
    p = x0[: 3 * n].view(-1, 3).to(torch.float64)
    out = torch.empty(n, dtype=torch.float64, device=p.device)
    for i0 in range(0, n, rows):
        d = p[None, :, :] - p[i0:i0 + rows, None, :]
        r = d.norm(dim=2)
        out[i0:i0 + rows] = (r / (r * r + eps * eps) ** 1.5).sum(dim=1)
    return out.cpu().numpy() / n


def mixed_accuracy(gb, x0, n: int, eps: float) -> dict:
    """Accelerations of the mixed path against FP64 on the initial state:
    normwise and per-body relative error (median, 99.9th percentile, max),
    and the per-body error against the sum of the body's pair-term
    magnitudes (the scale the pair differences' error bound refers to)."""
    ref = gb.nbody_rhs_f64(x0, n, eps, 1.0 / n).cpu().numpy()[3 * n:].reshape(-1, 3)
    got = gb.nbody_rhs_mixed(x0, n, eps, 1.0 / n).cpu().numpy()[3 * n:].reshape(-1, 3)
    err = np.linalg.norm(got - ref, axis=1)
    per = err / np.linalg.norm(ref, axis=1)
    cond = err / pair_force_scale(x0, n, eps)
    return {"normwise": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            "per_body_median": float(np.median(per)),
            "per_body_p999": float(np.quantile(per, 0.999)), "per_body_max": float(per.max()),
            "bodies_above_1e-6": int((per > 1e-6).sum()), "bodies": n,
            "per_body_max_over_pair_term_sum": float(cond.max())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the comparison arms (FP64, mixed reference / PI)")
    ap.add_argument("--mlp", default=None, help="proposer weights for the learned controller")
    ap.add_argument("--n-bodies", type=int, default=16384, help="stage: bodies")
    ap.add_argument("--stage-precision", default="mixed", choices=["mixed", "f64"],
                    help="stage: precision of the integrator")
    ap.add_argument("--tol", type=float, default=1e-9, help="c2_tol: atol = rtol")
    ap.add_argument("--sweep-tols", default="3e-12,1e-11,3e-11",
                    help="c2_sweep: tolerances of each controller's sweep (comma-separated)")
    ap.add_argument("--tol-override", type=float, default=None,
                    help="c3 / c5b: atol = rtol instead of the configuration's")
    ap.add_argument("--learned-config", default="plummer4096_rkf78",
                    help="c4: proposer training/evaluation configuration")
    ap.add_argument("--workload", default="c2",
                    choices=["c2", "c2_f64", "c2_tol", "c2_sweep", "c1", "c3", "c4", "c5a", "c5b", "pipes",
                             "rk_hbm", "stage"],
                    help="c2 (default, the headline), or another configuration")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "pipes":
        run_pipe_probe()
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
    mlp = load_mlp(args.mlp)
    exe = gb.Gb300Executor(precision=W["precision"], controller=W["controller"],
                           attempts_per_sync=A, mlp=mlp)
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
    per_job = {"accepted": accepted // max(args.steps, 1), "attempts": attempts // max(args.steps, 1),
               "rhs_evals": rhs // max(args.steps, 1)}
    # launches per job: start-up kernels (initial step, packing, first sort)
    # + per graph replay the re-sort (3 kernels of this library, the radix
    # sort's own kernels not counted) and A x (S stage kernels + 1 controller)
    replays = -(-per_job["attempts"] // A)
    launches_per_job = 15 + replays * (3 + A * (S + 1))
    # whole-job aggregate over ranks: accepted steps summed, time = max
    acc_all, rhs_all, ms_max = aggregate_over_ranks(float(accepted), float(rhs), ms)
    value = acc_all / (ms_max / 1e3)
    pair_rate = rhs_all * n * (n - 1) / (ms_max / 1e3)
    headline = {"time_to_tf_s": ms / 1e3 / max(args.steps, 1),
                "accepted_steps_per_s": accepted / (ms / 1e3), "accepted": per_job["accepted"],
                "attempts": per_job["attempts"],
                "rejected_fraction": 1 - accepted / max(attempts, 1),
                "rhs_evals": per_job["rhs_evals"], "t_reached": t_now,
                "pair_interactions_per_s": rhs * n * (n - 1) / (ms / 1e3), **cons}

    # dominant kernel: the fused stage kernel on a live integrator
    # (restarted, so no launch finds the integration finished), timed as
    # launched inside an attempt: 11 stage launches back to back after an
    # L2 flush, CUDA events around the run (on the integrator's stream),
    # repeated 10 times; kernel_ms = the mean per launch
    it.start(x0_dev, W["t0"], W["tf"], W["atol"], W["rtol"])
    geo = it.geometry()
    reps = 10
    ks0 = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    ks1 = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    with torch.cuda.stream(stream):
        for r in range(reps):
            flush.fill_(r & 0xFF)
            ks0[r].record(stream)
            for s in range(1, S - 1):
                it.launch_stage(s)
            ks1[r].record(stream)
    stream.synchronize()
    k_ms = statistics.mean(a.elapsed_time(b) for a, b in zip(ks0, ks1)) / (S - 2)
    achieved = FLOPS_PER_INTERACTION * n * (n - 1) / (k_ms / 1e3) / 1e12
    pk, pk_kind = peaks()
    sm_mhz_max = float(pk.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = n_sm * FP32_LANES_PER_SM * 2 * sm_mhz_max * 1e6 / 1e12
    it.close()
    stage_launches = per_job["rhs_evals"] - 2  # minus the initial step's two RHS

    line = {
        "metric": METRIC, "value": value, "unit": "accepted steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": {**W, "parallelism": f"replicas{world}",
                   "l2": "flushed between timed steps (256 MiB write)",
                   "step": "one whole integration t0 -> tf from the seeded state: initial "
                           "step on the device, then attempts of 13 fused stage kernels + "
                           "1 controller kernel replayed 16 per CUDA graph, bodies re-sorted "
                           "along a Morton curve at every replay"},
        "time_to_tf_s": headline["time_to_tf_s"],
        "pair_interactions_per_s": pair_rate,
        "per_step": per_job, "rejected_fraction": headline["rejected_fraction"],
        "t_reached": t_now, "energy_rel_err": cons["energy_rel_err"],
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
                     "kernel_timing": "mean per launch over 10 runs of 11 back-to-back stage "
                                      "launches (L2 flushed before each run), CUDA events on "
                                      "the launching stream",
                     "stage_launches_per_step_x_kernel_ms": stage_launches * k_ms,
                     "peak_note": f"nominal FP32 pipe: {n_sm} SMs x {FP32_LANES_PER_SM} lanes x 2"
                                  f" x {sm_mhz_max:.0f} MHz ({pk_kind} peaks file has no FP32)",
                     "flops_per_interaction": FLOPS_PER_INTERACTION,
                     "fp32_ops_per_interaction": HILO_FP32_OPS,
                     "fp32_pipe_cap_frac": FLOPS_PER_INTERACTION / 2 / HILO_FP32_OPS},
    }
    if rank == 0:
        # the measured ceilings the roofline fraction is read against
        try:
            pp = pipe_probe()
            line["roofline"]["measured_ceilings"] = {
                "f32x2_fma_frac_of_nominal": pp["ffma2_frac"],
                "scalar_fma_frac_of_nominal": pp["ffma_frac"],
                "sfu_rsqrt_per_sm_per_clock": pp["rsqrt_per_sm_per_clock"],
                "pair_loop_alone_frac_20flop": pp["pair_loop_frac_20flop"],
                "kernel_frac_of_pair_loop_ceiling": line["roofline"]["frac"]
                / pp["pair_loop_frac_20flop"],
                "note": "ode_prototyping_gb300/csrc/probe/pipes.cu: independent FMA chains, "
                        "and the stage kernel's pair loop without the close-pair test, "
                        "barriers, tails or epilogue (records in shared memory)"}
        except Exception as ex:  # reported, not fatal
            line["roofline"]["measured_ceilings"] = {"error": repr(ex)}
        line["e2e"] = e2e(gb, torch, x0, mlp)
        line["mixed_accuracy"] = mixed_accuracy(gb, x0_dev, n, eps)
        line["config2_tol_1e-8"] = config2_tolerance(gb, torch, x0_dev, e0)
        if not args.no_fp64:
            line["equal_energy_le_1e-8"] = metric_arms(gb, torch, x0_dev, e0, headline, mlp)
        if not args.no_cpu_baseline:
            try:
                apa = line.get("equal_energy_le_1e-8", {}).get("mixed_reference", {})
                ratio = apa.get("attempts", 552) / max(apa.get("accepted", 463), 1)
                line["cpu_baseline"] = cpu_baseline(ratio)
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


def pipe_probe() -> dict:
    """Throughput ceilings for the force kernel's roofline: runs
    ode_prototyping_gb300/csrc/probe/pipes.cu (built by the library build;
    compiled here if missing) -- scalar and f32x2 FMA, SFU rsqrt, and the
    pair loop alone -- and returns its measurements."""
    src = os.path.join(ROOT, "ode_prototyping_gb300", "csrc", "probe", "pipes.cu")
    exe = os.path.join(ROOT, "ode_prototyping_gb300", "_build", "probe_pipes")
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(exe), exist_ok=True)
        nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        src, "-o", exe], check=True)
    r = subprocess.run([exe], check=True, capture_output=True, text=True)
    return json.loads(r.stdout)


def run_pipe_probe():
    print(json.dumps({"workload": "pipes", **pipe_probe()}), flush=True)


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
    elif args.workload == "c2_sweep":
        # The controllers compared at equal energy error: the headline system
        # integrated t = 0 -> 2 (mixed precision) by the reference, PI and
        # learned controllers, each at the tolerances 3e-12, 1e-11, 3e-11; for
        # each controller the time to tf at a common relative energy error
        # (the geometric mean of the three controllers' errors at the middle
        # tolerance) is read off its own sweep by log-log interpolation.
        W = WORKLOAD
        n, eps = W["n_particles"], W["softening"]
        x0 = gb.to_device(gb.ic_plummer(n, W["seed"], 1.0))
        e0 = gb.energy(x0, n, eps, 1.0 / n)
        mlp = load_mlp(args.mlp)
        tols = [float(t) for t in args.sweep_tols.split(",")]
        sweep = {}
        for ctl in ("reference", "pi", "learned"):
            integrate_once(gb, torch, x0, stream, "mixed", ctl, 1e-11, mlp)  # warm-up
            rows = []
            for tol in tols:
                ms, st, xs = integrate_once(gb, torch, x0, stream, "mixed", ctl, tol, mlp)
                rows.append({"tol": tol, **arm_record(gb, x0, e0, ms, st, xs)})
            sweep[ctl] = rows
        mid = len(tols) // 2
        target = float(np.exp(np.mean([np.log(sweep[c][mid]["energy_rel_err"]) for c in sweep])))

        def at_target(rows):
            le = np.log([r["energy_rel_err"] for r in rows])
            lt = np.log([r["time_to_tf_s"] for r in rows])
            lr = np.log([r["rhs_evals"] for r in rows])
            order = np.argsort(le)
            le, lt, lr = le[order], lt[order], lr[order]
            x = np.log(target)
            return {"time_to_tf_s": float(np.exp(np.interp(x, le, lt))),
                    "rhs_evals": float(np.exp(np.interp(x, le, lr))),
                    "inside_sweep": bool(le[0] <= x <= le[-1])}
        eq = {c: at_target(sweep[c]) for c in sweep}
        for c in ("reference", "pi"):
            eq[f"learned_time_gain_vs_{c}"] = 1 - eq["learned"]["time_to_tf_s"] / eq[c]["time_to_tf_s"]
            eq[f"learned_rhs_saved_vs_{c}"] = 1 - eq["learned"]["rhs_evals"] / eq[c]["rhs_evals"]
        line.update(value=eq["learned"]["time_to_tf_s"], unit="s", higher_is_better=False,
                    metric="time to tf at equal relative energy error (learned / PI / reference)",
                    dtype="f32+f64", steps=1, ms_per_step=1e3 * eq["learned"]["time_to_tf_s"],
                    energy_target=target, sweep=sweep, at_equal_energy=eq,
                    config={**W, "tols": tols,
                            "proposer": os.path.basename(args.mlp) if args.mlp else PROPOSER,
                            "step": "whole integrations, three tolerances per controller"})
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
        # Batched ensembles, every arm over the whole span [0, tf] at the same
        # tolerance: mixed precision with the reference, PI and learned
        # controllers, and the plain FP64 batch; per-system relative energy
        # errors (median, 90th percentile, max) beside time to tf and
        # accepted steps/s.  --tol overrides the configuration's tolerance.
        if args.workload == "c3":
            # configuration 3: 512 Plummer spheres, N log-uniform in [64, 4096],
            # virial ratio U(0.5, 1.5), eps = 0.01 * 4 / N^(1/3), DOPRI5, tol 1e-9
            rng = np.random.default_rng(303)
            sizes = np.round(np.exp(rng.uniform(np.log(64), np.log(4096), 512))).astype(np.int64)
            eps = 0.01 * 4.0 / np.cbrt(sizes)
            x0 = _batch_ics(gb, torch, sizes, 3000 + np.arange(512), "virial", eps)
            tab, tol, tf = "DOPRI5", 1e-9, 1.0
            prop = "proposer_batch3_dopri5_tol1e-9.bin"
        else:
            # configuration 5, batched part: 64 binary-rich Plummer spheres of
            # N = 8192 (10 % of the bodies in bound pairs, semimajor axes
            # log-uniform in [1e-3, 1e-2]); the configuration gives no
            # softening, the pairs need one well below their separations:
            # eps = 1e-4; DOPRI5, tol 1e-8, t in [0, 0.02] (about one and a
            # half periods of the tightest pairs; the FP64 arm takes under a
            # minute over it)
            sizes = np.full(64, 8192, dtype=np.int64)
            eps = np.full(64, 1e-4)
            x0 = _batch_ics(gb, torch, sizes, 6000 + np.arange(64), "binary", eps)
            tab, tol, tf = "DOPRI5", 1e-8, 0.02
            prop = "proposer_binary2048_dopri5.bin"
        if args.tol_override is not None:
            tol = args.tol_override
        x0d = gb.to_device(x0)
        offs = np.concatenate([[0], np.cumsum(sizes)]) * 6
        e0 = [gb.energy(x0d[offs[k]:offs[k + 1]], int(sizes[k]), float(eps[k]), 1.0 / sizes[k])
              for k in range(len(sizes))]
        ppath = os.path.join(ROOT, "ode_prototyping_gb300", "weights", prop)
        mlp = (gb.GbMlp.from_buffer_copy(open(ppath, "rb").read())
               if os.path.exists(ppath) else None)

        def run_arm(prec, ctl, reps):
            b = gb.Batch(tab, sizes, eps, precision=prec, controller=ctl, attempts_per_sync=8,
                         stream=stream, mlp=mlp if ctl == "learned" else None,
                         max_attempts=200000)
            b.start(x0d, 0.0, tf, tol, tol)
            tune = b.autotune(2)

            def job():
                b.start(x0d, 0.0, tf, tol, tol)
                rc = b.advance(0)
                assert rc == 0, rc
                return b.stats()
            if reps > 1:
                job()  # warm-up
            ms, st = _timed(torch, stream, job, reps, flush)
            xs, ts = b.state()
            errs = []
            for k in range(len(sizes)):
                e1 = gb.energy(xs[offs[k]:offs[k + 1]], int(sizes[k]), float(eps[k]),
                               1.0 / sizes[k])
                errs.append(abs(e1["e"] - e0[k]["e"]) / abs(e0[k]["e"]))
            acc = sum(s["n_accepted"] for s in st)
            inter = sum(s["interactions"] for s in st)
            b.close()
            r = {"accepted_steps_per_s": acc / (ms / 1e3),
                 "pair_interactions_per_s": inter / (ms / 1e3),
                 "time_to_tf_s": ms / len(st) / 1e3, "geometry": tune,
                 "accepted": st[0]["n_accepted"], "attempts": st[0]["n_attempts"],
                 "rhs_evals": st[0]["n_rhs"], "t_min": float(ts.min()),
                 "energy_rel_err_median": float(np.median(errs)),
                 "energy_rel_err_p90": float(np.quantile(errs, 0.9)),
                 "energy_rel_err_max": float(np.max(errs))}
            print(json.dumps({"arm": [prec, ctl], **r}), flush=True)
            return r
        # --no-fp64: the mixed arm with the reference controller only (a short
        # run, e.g. for profiling the stage kernel)
        ctls = ["reference"] + ([] if args.no_fp64 else
                                ["pi"] + (["learned"] if mlp is not None else []))
        arms = {f"mixed_{c}": run_arm("mixed", c, args.steps) for c in ctls}
        if not args.no_fp64:
            arms["f64_reference"] = run_arm("f64", "reference", 1)
            f64 = arms["f64_reference"]
            for key in [k for k in arms if k != "f64_reference"]:
                arms[f"speedup_time_to_tf_{key}_vs_f64"] = (f64["time_to_tf_s"]
                                                            / arms[key]["time_to_tf_s"])
                arms[f"speedup_accepted_steps_per_s_{key}_vs_f64"] = (
                    arms[key]["accepted_steps_per_s"] / f64["accepted_steps_per_s"])
        head = arms.get("mixed_learned", arms["mixed_reference"])
        line.update(value=head["accepted_steps_per_s"], dtype="f32+f64",
                    steps=args.steps, ms_per_step=1e3 * head["time_to_tf_s"],
                    pair_interactions_per_s=head["pair_interactions_per_s"], arms=arms,
                    config={"workload": args.workload, "systems": int(len(sizes)),
                            "n_min": int(sizes.min()), "n_max": int(sizes.max()),
                            "bodies": int(sizes.sum()), "tableau": tab, "atol": tol,
                            "rtol": tol, "t": [0, tf],
                            "softening": "0.01 * 4 / N^(1/3)" if args.workload == "c3"
                            else float(eps[0]),
                            "proposer": prop if mlp is not None else None,
                            "step": "whole batch integration, every system to tf"})
    elif args.workload == "stage":
        # Four stage launches of the headline integrator on an N-body Plummer
        # sphere (a small case for profiling the fused stage kernel).
        n = args.n_bodies
        x0 = gb.to_device(gb.ic_plummer(n, WORKLOAD["seed"], 1.0))
        it = gb.Integrator(WORKLOAD["tableau"], gb.NBodyODE(n, WORKLOAD["softening"], 1.0 / n),
                           gb.Gb300Executor(precision=args.stage_precision, attempts_per_sync=1),
                           stream=stream)
        it.start(x0, WORKLOAD["t0"], WORKLOAD["tf"], WORKLOAD["atol"], WORKLOAD["rtol"])
        # one whole attempt first (13 launches), so every stage buffer and
        # tile box holds the integration's own data
        with torch.cuda.stream(stream):
            for r in range(gb.tableau(WORKLOAD["tableau"]).n_stages):
                it.launch_stage(r)
        stream.synchronize()
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
                            "step": "one fused stage launch (a whole attempt of 13, then "
                                    "four more launched)"})
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
        # Configuration 5, single system: N = 262144 cold collapse (uniform
        # sphere, velocities 1 % Gaussian noise, eps = 0.002), DOPRI5, tol
        # 1e-8.  The mixed path runs `steps` timed attempts after the warm-up
        # ones; then every arm integrates the same window [0, t_w] (t_w =
        # where those attempts ended) from the initial state: mixed with the
        # reference controller, mixed with the learned proposer, and the plain
        # FP64 path, each with its time and relative energy error at t_w.
        n, eps, tol = 262144, 0.002, 1e-8
        x0 = gb.to_device(gb.ic_cold_sphere(n, 505, 0.01))
        e0 = gb.energy(x0, n, eps, 1.0 / n)
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
        xs, t_w = it.state()
        it.close()
        # accelerations of the mixed path against FP64 on the current state
        f64 = gb.nbody_rhs_f64(xs, n, eps, 1.0 / n, tile=gb.tiling(f64_pair=1))
        mx = gb.nbody_rhs_mixed(xs, n, eps, 1.0 / n)
        a64, amx = f64[3 * n:].view(-1, 3), mx[3 * n:].view(-1, 3)
        rel = ((amx - a64).norm() / a64.norm()).item()
        per_b = ((amx - a64).norm(dim=1) / a64.norm(dim=1))
        window = {"t_w": t_w}
        ppath = os.path.join(ROOT, "ode_prototyping_gb300", "weights",
                             "proposer_binary2048_dopri5.bin")
        mlp = gb.GbMlp.from_buffer_copy(open(ppath, "rb").read())
        for key, prec, ctl in (("mixed", "mixed", "reference"),
                               ("learned_mixed", "mixed", "learned"),
                               ("f64", "f64", "reference")):
            itw = gb.Integrator("DOPRI5", gb.NBodyODE(n, eps, 1.0 / n),
                                gb.Gb300Executor(precision=prec, controller=ctl,
                                                 attempts_per_sync=4,
                                                 mlp=mlp if ctl == "learned" else None),
                                stream=stream)

            def job():
                itw.start(x0, 0.0, t_w, tol, tol)
                assert itw.advance(0) == 0
                return itw.stats()
            wms, wst = _timed(torch, stream, job, 1, flush)
            e1 = gb.energy(itw.state()[0], n, eps, 1.0 / n)
            window[key] = {"time_to_t_w_s": wms / 1e3, "accepted": wst[0]["n_accepted"],
                           "attempts": wst[0]["n_attempts"], "rhs_evals": wst[0]["n_rhs"],
                           "accepted_steps_per_s": wst[0]["n_accepted"] / (wms / 1e3),
                           **drift(e0, e1)}
            itw.close()
        for key in ("mixed", "learned_mixed"):
            window[f"speedup_time_{key}_vs_f64"] = (window["f64"]["time_to_t_w_s"]
                                                    / window[key]["time_to_t_w_s"])
        line.update(value=acc / (ms / 1e3), dtype="f32+f64", steps=args.steps,
                    ms_per_step=ms / args.steps,
                    pair_interactions_per_s=rhs * n * (n - 1) / (ms / 1e3),
                    accepted=acc, t_reached=t_w, acc_rel_err_normwise=rel,
                    acc_rel_err_median=per_b.median().item(),
                    acc_rel_err_p999=per_b.quantile(0.999).item(),
                    acc_rel_err_max=per_b.max().item(), window=window,
                    config={"workload": "cold_collapse262144_dopri5_mixed", "n_particles": n,
                            "softening": eps, "tableau": "DOPRI5", "atol": tol, "rtol": tol,
                            "proposer": "proposer_binary2048_dopri5.bin (DOPRI5, trained on "
                                        "binary-rich N = 2048 systems, not on this one)",
                            "step": "one adaptive attempt"})
    print(json.dumps(line), flush=True)


def e2e(gb, torch, x0: np.ndarray, mlp, reps: int = 3) -> dict:
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
        exe = gb.Gb300Executor(precision=W["precision"], controller=W["controller"],
                               attempts_per_sync=16, mlp=mlp)
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


if __name__ == "__main__":
    main()
