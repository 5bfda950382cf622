"""Learned step-size proposer: data, training and evaluation.

1. ``collect_logs`` runs the plain integrator with the device-side controller
   log on (``log_steps``): per attempt, the 16 features the controller sees
   after the attempt, the attempted step, the scaled error and the decision.
2. ``build_dataset`` pairs every accepted attempt k with the next attempt
   k+1 and sets the target to the step change that would have put attempt
   k+1 at the error ratio rho under the local error model err ~ dt^(q+1):
   r_k = log(dt_{k+1} (rho / err_{k+1})^(1/(q+1))) - log(dt_k), minus the
   elementary controller's own proposal log(safety) - log(err_k)/(q+1): the
   network learns a correction to the reference's step-size formula, so
   features outside the training range fall back towards that formula.
3. ``train`` fits the 16 -> 64 -> 64 -> 1 SiLU network with the library's
   own forward / backward / Adam kernels (``gb_mlp_train``), asymmetric loss
   (over-long steps cost a rejected attempt, so over-prediction weighs more).
4. ``evaluate`` integrates held-out systems with the reference, PI and
   learned controllers and reports RHS evaluations, rejected fraction,
   accepted steps per second and the relative energy error.

The embedded error estimate still accepts or rejects every attempt, and
every rejection hands the step back to the PI controller.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import (GbMlp, GbIntegrateStats, Gb300Executor, Integrator, NBodyODE, check, energy,
               ic_binary_plummer, ic_plummer, lib, tableau)

FEAT, LOG_DT, LOG_ERR, ACCEPTED = slice(0, 16), 16, 17, 18


def initial_state(kind: str, n: int, seed: int) -> np.ndarray:
    """'plummer': Plummer sphere; 'binary': Plummer sphere with 10% of the
    bodies in bound pairs, semimajor axes log-uniform in [1e-3, 1e-2];
    'virial': Plummer sphere with its velocities scaled by sqrt(Q), Q drawn
    uniform in [0.5, 1.5) from the seed (configuration 3's members)."""
    if kind == "plummer":
        return ic_plummer(n, seed)
    if kind == "binary":
        return ic_binary_plummer(n, seed, 0.1, 1e-3, 1e-2)
    if kind == "virial":
        x = ic_plummer(n, seed)
        x[3 * n:] *= np.sqrt(0.5 + np.random.default_rng(seed).uniform())
        return x
    raise ValueError(f"unknown initial state {kind!r}")


def member(n, softening, i: int):
    """(bodies, softening) of the i-th training or evaluation run: a config's
    n may be a list (runs cycle through it) and its softening the rule
    'c3' (0.01 * 4 / N^(1/3), configuration 3's)."""
    nn = n[i % len(n)] if isinstance(n, (list, tuple)) else n
    soft = 0.04 / nn ** (1.0 / 3.0) if softening == "c3" else softening
    return int(nn), float(soft)


def tolerances(tol) -> list:
    """A config's tolerance: one value, or a list (every seed is run at each)."""
    return list(tol) if isinstance(tol, (list, tuple)) else [tol]


def collect_logs(seeds, n: int, softening: float, tab: str, tol, tf: float,
                 attempts: int, precision: str = "mixed", controller: str = "reference",
                 mlp: GbMlp | None = None, ic: str = "plummer"):
    logs = []
    runs = [(seed, t) for t in tolerances(tol) for seed in seeds]
    for i, (seed, tol) in enumerate(runs):
        nn, soft = member(n, softening, i)
        x0 = initial_state(ic, nn, seed)
        exe = Gb300Executor(precision=precision, controller=controller, attempts_per_sync=16,
                            log_steps=attempts, mlp=mlp)
        it = Integrator(tab, NBodyODE(nn, soft, 1.0 / nn), exe)
        it.start(x0, 0.0, tf, tol, tol)
        it.advance(attempts)
        logs.append(it.log())
        it.close()
    return logs


PI_BETA = 0.04  # the integrator's default PI memory exponent


def build_dataset(logs, q: int, rho: float = 0.6, pi_beta: float = PI_BETA):
    """Targets are residuals over the PI controller's log step ratio
    log(safety) - alpha log(err_k) + beta log(err_prev) (feature 13 holds
    log(err_prev)), the base the device adds the network output to."""
    xs, ys = [], []
    log_safety = np.log(0.38) / (1.0 + q)
    alpha = 1.0 / (1.0 + q) - 0.75 * pi_beta
    for rec in logs:
        for k in range(len(rec) - 1):
            if rec[k, ACCEPTED] < 0.5:
                continue
            base = log_safety - alpha * rec[k, LOG_ERR] + pi_beta * rec[k, 13]
            target = (rec[k + 1, LOG_DT] + (np.log(rho) - rec[k + 1, LOG_ERR]) / (q + 1)
                      - rec[k, LOG_DT] - base)
            if not np.isfinite(target):
                continue
            xs.append(rec[k, FEAT])
            ys.append(target)
    return np.asarray(xs, dtype=np.float32), np.asarray(ys, dtype=np.float32)


def _to_device_struct(m: GbMlp):
    import torch
    buf = torch.empty(C.sizeof(GbMlp), dtype=torch.uint8, device="cuda")
    host = torch.frombuffer(bytearray(bytes(m)), dtype=torch.uint8)
    buf.copy_(host)
    return buf


def _from_device_struct(buf) -> GbMlp:
    raw = bytes(buf.cpu().numpy().tobytes())
    return GbMlp.from_buffer_copy(raw)


def _val_loss(m: GbMlp, x: np.ndarray, y: np.ndarray, over_weight: float) -> float:
    """Mean asymmetric squared error of the FP32 forward pass (library kernel)."""
    import torch
    w = _to_device_struct(m)
    xd = torch.as_tensor(np.ascontiguousarray(x), device="cuda")
    yd = torch.empty(len(y), dtype=torch.float32, device="cuda")
    check(lib().gb_mlp_forward_f32(w.data_ptr(), xd.data_ptr(), yd.data_ptr(), len(y), None,
                                   None), "gb_mlp_forward_f32")
    d = yd.cpu().numpy() - y
    return float(np.mean(np.where(d > 0, over_weight, 1.0) * d * d))


def train(x: np.ndarray, y: np.ndarray, epochs: int = 3000, lr: float = 3e-3,
          over_weight: float = 3.0, seed: int = 0, val_frac: float = 0.0,
          epoch_grid=(100, 300, 1000, 3000)):
    """Returns (trained gb_mlp in host memory, final loss).  With val_frac > 0
    a seeded random share of the samples is held out and the training length
    is chosen from epoch_grid by the held-out loss (early stopping)."""
    if val_frac > 0.0:
        rng = np.random.default_rng(seed + 1)
        perm = rng.permutation(len(y))
        nv = max(1, int(len(y) * val_frac))
        vi, ti = perm[:nv], perm[nv:]
        best = None
        for e in epoch_grid:
            m, _ = train(x[ti], y[ti], epochs=e, lr=lr, over_weight=over_weight, seed=seed)
            v = _val_loss(m, x[vi], y[vi], over_weight)
            if best is None or v < best[0]:
                best = (v, m)
        return best[1], best[0]
    import torch
    m = GbMlp()
    check(lib().gb_mlp_init(C.byref(m), seed), "gb_mlp_init")
    mean = x.mean(0)
    std = x.std(0)
    scale = np.where(std > 1e-6, 1.0 / np.maximum(std, 1e-6), 0.0)
    for k in range(16):
        m.in_mean[k] = float(mean[k])
        m.in_scale[k] = float(scale[k])
    m.out_bias = float(y.mean())
    m.out_scale = float(max(y.std(), 1e-3))
    w = _to_device_struct(m)
    xd = torch.as_tensor(np.ascontiguousarray(x), device="cuda")
    yd = torch.as_tensor(np.ascontiguousarray(y), device="cuda")
    loss = C.c_float(0)
    check(lib().gb_mlp_train(w.data_ptr(), xd.data_ptr(), yd.data_ptr(), len(y), epochs, lr,
                             over_weight, C.byref(loss), None), "gb_mlp_train")
    torch.cuda.synchronize()
    return _from_device_struct(w), float(loss.value)


def fit(seeds, n: int, softening: float, tab: str, tol: float, tf: float, attempts: int,
        rounds: int = 2, rho: float = 0.6, epochs: int = 3000, over_weight: float = 2.0,
        ic: str = "plummer"):
    """Logs of the reference and PI controllers, a first fit, then rounds of
    logs collected under the learned controller itself (so the data cover the
    states it visits) and refits.  Returns (network, info)."""
    q = min(tableau(tab).p, tableau(tab).pt)
    logs = collect_logs(seeds, n, softening, tab, tol, tf, attempts, controller="reference",
                        ic=ic)
    logs += collect_logs(seeds, n, softening, tab, tol, tf, attempts, controller="pi", ic=ic)
    info = []
    m = None
    for r in range(max(rounds, 1)):
        if m is not None:
            logs += collect_logs(seeds, n, softening, tab, tol, tf, attempts,
                                 controller="learned", mlp=m, ic=ic)
        x, y = build_dataset(logs, q, rho)
        m, loss = train(x, y, epochs=epochs, over_weight=over_weight, val_frac=0.2)
        info.append({"round": r, "samples": int(len(y)), "val_loss": loss})
    return m, info


def run_window(n: int, softening: float, tab: str, tol: float, t_end: float, seed: int,
               controller: str, mlp: GbMlp | None = None, precision: str = "mixed",
               ic: str = "plummer") -> dict:
    import torch
    x0 = initial_state(ic, n, seed)
    stream = torch.cuda.Stream()
    exe = Gb300Executor(precision=precision, controller=controller, attempts_per_sync=16,
                        mlp=mlp)
    it = Integrator(tab, NBodyODE(n, softening, 1.0 / n), exe, stream=stream)
    e0 = energy(x0, n, softening, 1.0 / n)
    it.start(x0, 0.0, t_end, tol, tol)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = it.advance(0)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    st = it.stats()
    xs, t = it.state()
    e1 = energy(xs, n, softening, 1.0 / n)
    it.close()
    return {"controller": controller, "status": rc, "t": t, "wall_s": wall,
            "accepted": st["n_accepted"], "rejected": st["n_rejected"],
            "attempts": st["n_attempts"], "rhs": st["n_rhs"],
            "rejected_fraction": st["n_rejected"] / max(st["n_attempts"], 1),
            "accepted_steps_per_s": st["n_accepted"] / wall,
            "learned_proposals": st["n_learned_proposals"],
            "learned_rejected": st["n_learned_rejected"],
            "energy_rel_err": abs(e1["e"] - e0["e"]) / abs(e0["e"]), "state": xs}


def evaluate(n, softening, tab, tol, t_end, seeds, mlp, precision="mixed", ic="plummer"):
    out = {}
    for ctl in ("reference", "pi", "learned"):
        rows = [run_window(*member(n, softening, i), tab, tol, t_end, s, ctl,
                           mlp if ctl == "learned" else None, precision, ic)
                for i, s in enumerate(seeds)]
        agg = {k: float(np.sum([r[k] for r in rows])) for k in
               ("wall_s", "accepted", "rejected", "attempts", "rhs", "learned_proposals",
                "learned_rejected")}
        agg["rejected_fraction"] = agg["rejected"] / max(agg["attempts"], 1)
        agg["energy_rel_err_max"] = float(max(r["energy_rel_err"] for r in rows))
        agg["simulated_time_per_s"] = len(seeds) * t_end / agg["wall_s"]
        agg["states"] = [r["state"] for r in rows]
        out[ctl] = agg
    return out


# Workloads the proposer is trained and evaluated on (seed set A trains,
# seed set B evaluates).
CONFIGS = {
    # N = 16384 Plummer sphere, RKF78, tol 1e-8 (the single large system)
    "plummer16384_rkf78": dict(ic="plummer", n=16384, softening=0.005, tab="RKF78", tol=1e-8,
                               tf=2.0, attempts=400),
    # the same family at N = 4096 over t in [0, 0.5] (quick to train)
    "plummer4096_rkf78": dict(ic="plummer", n=4096, softening=0.005, tab="RKF78", tol=1e-8,
                              tf=0.5, attempts=300),
    # binary-rich Plummer spheres, DOPRI5, tol 1e-8
    "binary2048_dopri5": dict(ic="binary", n=2048, softening=1e-4, tab="DOPRI5", tol=1e-8,
                              tf=0.02, attempts=300),
    # the single large system at tol 1e-11, where its relative energy error
    # over t in [0, 2] is below 1e-8
    "plummer16384_rkf78_tol1e-11": dict(ic="plummer", n=16384, softening=0.005, tab="RKF78",
                                        tol=1e-11, tf=2.0, attempts=800),
    # configuration 3's integrator on one of its mid-size members: Plummer
    # N = 512, eps = 0.01 * 4 / 512^(1/3) = 0.005, DOPRI5, tol 1e-9, t in [0, 1]
    # (one size only: on the batch it took many more steps than the reference
    # controller, hence the multi-size configuration below)
    "plummer512_dopri5_tol1e-9": dict(ic="plummer", n=512, softening=0.005, tab="DOPRI5",
                                      tol=1e-9, tf=1.0, attempts=600),
    # the single large system over tolerances 1e-8 .. 1e-12: one network for
    # all of them, with log max(atol, rtol) as a feature (every seed of the set
    # is run at each tolerance)
    "plummer16384_rkf78_multitol": dict(ic="plummer", n=16384, softening=0.005, tab="RKF78",
                                        tol=[1e-8, 1e-9, 1e-10, 1e-11, 1e-12], tf=2.0,
                                        attempts=1200),
    # configuration 3's members: Plummer spheres with virial ratio in [0.5, 1.5),
    # N cycling through 64 .. 4096 (log-spaced), eps = 0.01 * 4 / N^(1/3),
    # DOPRI5, tol 1e-9, t in [0, 1] (the proposer the batched C3 workload runs)
    "batch3_dopri5_tol1e-9": dict(ic="virial", n=[64, 128, 256, 512, 1024, 2048, 4096, 181],
                                  softening="c3", tab="DOPRI5", tol=1e-9, tf=1.0, attempts=800),
}
SEEDS_A = list(range(1, 17))
SEEDS_B = list(range(101, 117))


def train_config(name: str, seeds=None, rounds: int = 3, rho: float = 0.38, epochs: int = 3000):
    c = CONFIGS[name]
    return fit(seeds or SEEDS_A[:8], c["n"], c["softening"], c["tab"], c["tol"], c["tf"],
               c["attempts"], rounds=rounds, rho=rho, epochs=epochs, ic=c["ic"])


def evaluate_config(name: str, mlp: GbMlp, seeds=None, tol=None) -> dict:
    """Reference, PI and learned controllers on held-out seeds, plus the
    learned run's gain over the reference controller.  A config with several
    tolerances is evaluated at each (a dict keyed by tolerance) unless tol
    picks one."""
    c = CONFIGS[name]
    tols = tolerances(c["tol"]) if tol is None else [tol]
    if len(tols) > 1:
        return {f"{t:g}": evaluate_config(name, mlp, seeds, t) for t in tols}
    ev = evaluate(c["n"], c["softening"], c["tab"], tols[0], c["tf"], seeds or SEEDS_B[:4], mlp,
                  ic=c["ic"])
    states = {k: v.pop("states") for k, v in ev.items()}
    ref, lrn = ev["reference"], ev["learned"]
    ev["gain"] = {
        "rhs_saved_fraction": 1.0 - lrn["rhs"] / ref["rhs"],
        "rejected_fraction_reference": ref["rejected_fraction"],
        "rejected_fraction_learned": lrn["rejected_fraction"],
        "energy_err_ratio": lrn["energy_rel_err_max"] / max(ref["energy_rel_err_max"], 1e-300),
        "wall_speedup": ref["wall_s"] / lrn["wall_s"],
        "max_state_diff_vs_reference": max(float((a - b).abs().max().item())
                                           for a, b in zip(states["learned"],
                                                           states["reference"])),
    }
    return ev


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train the learned step-size proposer")
    ap.add_argument("--config", default="plummer16384_rkf78", choices=sorted(CONFIGS))
    ap.add_argument("--out", required=True, help="weights file (raw gb_mlp)")
    ap.add_argument("--rho", type=float, default=0.38)
    ap.add_argument("--rounds", type=int, default=3)
    ap.add_argument("--seeds", type=int, default=8, help="seeds 1..k of seed set A")
    ap.add_argument("--eval-seeds", type=int, default=4, help="seeds of seed set B evaluated")
    a = ap.parse_args(argv)
    t0 = time.time()
    m, info = train_config(a.config, SEEDS_A[:a.seeds], rounds=a.rounds, rho=a.rho)
    with open(a.out, "wb") as f:
        f.write(bytes(m))
    ev = evaluate_config(a.config, m, SEEDS_B[:a.eval_seeds])
    print(json.dumps({"config": a.config, "train": info, "train_s": time.time() - t0,
                      "evaluation": ev}, indent=1))


if __name__ == "__main__":
    main()
