"""Benchmark: particle-days/s of the batched device IAS15 (FP64) on GB300.

Workload (the learned-warm-start evaluation configuration of ASSIST's
test-particle path): 262,144 independent particles of a 40% main-belt, 30%
NEO, 20% Jupiter-Trojan-like, 10% trans-Neptunian mixture (10% with Marsden
non-gravitational A1, A2 ~ +-logU[1e-12, 1e-9] AU/d^2), each integrated one
year with its own adaptive IAS15 steps (epsilon 1e-9), full ASSIST force
model (Sun, planets, 16 asteroids, Earth J2-J4, Sun J2, EIH GR).  Ephemeris:
seeded synthetic .440 + 16-asteroid SPK (the JPL files are not available).
The warm-start network is trained in the run, outside the timed region, on
(features, target) pairs logged from a separate 65,536-particle population
of the same mixture with lengths ~ logU[30 d, 10 yr].

One step = one pass of the hot path over the whole batch: every particle
integrated from t0 to its t_end by the persistent kernel.

  value : particle-days/s of the default path (plain IAS15 predictor) with
          inputs resident in HBM, CUDA events around the kernel on its
          stream, L2 flushed (256 MB write) between steps.
  learned_warm_start : the same with the learned warm start, timed beside it.
  e2e   : the default path through the public host-array C entry point
          assist_gb300_integrate_batch (H2D + kernel + D2H in the timed region).
  roofline : FP64 pipe; achieved = algorithmic FP64 flops (oracle op count per
          force evaluation x evaluations + IAS15 bookkeeping) / kernel time;
          peak = FP64 FMA throughput measured in this run.
  cpu_baseline : the oracle (CPU restatement of ASSIST's forces + IAS15) on all
          host cores over a bounded random sample of the same population.

--impl reference times that CPU path alone (the reference arm).
Multi-GPU (torchrun): weak scaling, each rank integrates its own batch of the
same size; no collective on the data path.
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

N_PARTICLES = 262144          # evaluation population, one year each
N_TRAIN = 65536               # pair-logging population, lengths logU[30 d, 10 yr]
LENGTH = 365.25
SEED_EPHEM = 20240611
SEED_POP = 12345
T0 = 8000.0
WORKLOAD = "262144-mixture-1yr-learned-warm-start-vs-plain"
METRIC = "particle-days/s FP64 on 1 GB300: learned-warm-start vs plain IAS15 vs CPU ref"
UNIT = "particle-days/s"


def make_inputs(tmpdir: str):
    from assist_gb300 import synth
    pl, ast, system = synth.write_ephemeris(tmpdir, seed=SEED_EPHEM, t_beg=T0 - 40.0, t_end=T0 + 3700.0)
    pop = synth.population(system, "mix", N_PARTICLES, seed=SEED_POP, t0=T0, length=LENGTH, nongrav_frac=0.1)
    return pl, ast, system, pop


def algorithmic_flops(pl, ast, pop, stats):
    """FP64 operations the outputs need: oracle op count of one force
    evaluation (ephemeris of all bodies at the particle's own time + every
    force term; sqrt and div counted as 1) times the evaluations, plus the
    IAS15 predictor/corrector bookkeeping per evaluation and per step."""
    from tests.oracle_py import Oracle
    o = Oracle(pl, ast)
    i_plain = int(np.nonzero(np.abs(pop.params).sum(1) == 0)[0][0])
    c = o.count_ops(T0, pop.state[i_plain])
    per_eval = c["add"] + c["mul"] + c["div"] + c["sqrt"] + c["pow"]
    ias_per_eval = 3 * (34 + 16)          # predictor x,v (9 + 8 terms) and divided-difference/b update
    ias_per_step = 3 * (2 * 9 + 2 * 8 + 8 + 7 * 8)   # accept update, compensated sums, next-step prediction
    flops = stats["force_evals"] * (per_eval + ias_per_eval) + stats["steps_accepted"] * ias_per_step
    return flops, per_eval, c


def train_warm_start(eph, system, dev, n_train: int = N_TRAIN, steps: int = 1500):
    """Log (features, target) pairs from one plain integration of a separate
    seeded population of the same mixture (lengths logU[30 d, 10 yr]) and
    train the warm-start network with the device kernels (outside the timed
    region)."""
    import torch
    from assist_gb300 import synth, warm
    tp = synth.population(system, "mix", n_train, seed=SEED_POP + 1, t0=T0, log_len=(30.0, 3652.5), nongrav_frac=0.1)
    t = time.perf_counter()
    warm.init(SEED_POP)
    X, T, _ = warm.collect(eph, torch.tensor(tp.t0, device=dev), torch.tensor(tp.t_end, device=dev),
                           torch.tensor(tp.state, device=dev), params=torch.tensor(tp.params, device=dev),
                           capacity=5 << 20, every=1)
    perm = torch.randperm(X.shape[0], device=dev, generator=torch.Generator(device=dev).manual_seed(0))
    X, T = X[perm].contiguous(), T[perm].clamp(-4, 4).contiguous()
    l0, _ = warm.grad(X[:4096], T[:4096])
    loss = warm.train(X, T, steps=steps, batch=4096, lr=1e-3, seed=1)
    torch.cuda.synchronize()
    return {"pairs": int(X.shape[0]), "train_particles": n_train, "train_steps": steps, "batch": 4096,
            "loss_initial": l0, "loss_final": loss, "train_s": time.perf_counter() - t}


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._p = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                        "--format=csv,noheader,nounits", "-lms", "200"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self._p = None

    def _read(self):
        for line in self._p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self._p:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(pl, ast, pop, target_s: float = 15.0, threads=None):
    """Oracle batch integration on the host cores over a random sample."""
    from tests.oracle_py import Oracle
    o = Oracle(pl, ast)
    threads = threads or os.cpu_count() or 1
    rng = np.random.default_rng(7)
    n_pilot = 4 * threads
    idx = rng.choice(pop.t0.size, size=n_pilot, replace=False)
    t = time.perf_counter()
    o.integrate_batch(pop.t0[idx], pop.t_end[idx], pop.state[idx], params=pop.params[idx], threads=threads)
    pilot = time.perf_counter() - t
    n = int(min(pop.t0.size, max(n_pilot, n_pilot * target_s / max(pilot, 1e-3))))
    idx = rng.choice(pop.t0.size, size=n, replace=False)
    t = time.perf_counter()
    _, _, st, _ = o.integrate_batch(pop.t0[idx], pop.t_end[idx], pop.state[idx], params=pop.params[idx],
                                    threads=threads, return_all=True)
    dt = time.perf_counter() - t
    pdays = float(np.abs(pop.t_end[idx] - pop.t0[idx])[st == 0].sum())
    return {"value": pdays / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of the %d particles (random, seed 7), their full integrations: %.3g particle-days in %.1f s"
                      % (n, pop.t0.size, pdays, dt)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    tmp = tempfile.mkdtemp(prefix="assist_bench_")
    pl, ast, system, pop = make_inputs(tmp)
    from tests.oracle_py import Oracle
    o = Oracle(pl, ast)
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(11)
    # step = a bounded sample of the workload (same distribution), sized to ~8 s
    n_pilot = 4 * threads
    idx = rng.choice(pop.t0.size, size=n_pilot, replace=False)
    t = time.perf_counter()
    o.integrate_batch(pop.t0[idx], pop.t_end[idx], pop.state[idx], params=pop.params[idx], threads=threads)
    pilot = time.perf_counter() - t
    n = int(min(pop.t0.size, max(n_pilot, n_pilot * 8.0 / max(pilot, 1e-3))))
    for _ in range(args.warmup):
        idx = rng.choice(pop.t0.size, size=min(n, n_pilot), replace=False)
        o.integrate_batch(pop.t0[idx], pop.t_end[idx], pop.state[idx], params=pop.params[idx], threads=threads)
    tot_days, tot_s = 0.0, 0.0
    for _ in range(args.steps):
        idx = rng.choice(pop.t0.size, size=n, replace=False)
        t = time.perf_counter()
        _, _, st, _ = o.integrate_batch(pop.t0[idx], pop.t_end[idx], pop.state[idx], params=pop.params[idx],
                                        threads=threads, return_all=True)
        tot_s += time.perf_counter() - t
        tot_days += float(np.abs(pop.t_end[idx] - pop.t0[idx])[st == 0].sum())
    v = tot_days / tot_s
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ephemeris + population)",
            "config": {"workload": WORKLOAD, "n_particles": N_PARTICLES,
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d random particles of the workload per step (full integrations)" % n},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-warm", action="store_true", help="plain predictor only (no learned warm start)")
    ap.add_argument("--blocks-per-sm", type=int, default=0,
                    help="block-cooperative kernel residency: 0 automatic (the library's choice), 2 or 3")
    ap.add_argument("--particles", type=int, default=None, help="override the batch size (profiling only)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    global N_PARTICLES
    if args.particles:
        N_PARTICLES = args.particles
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from assist_gb300 import Ephem, batch
    tmp = tempfile.mkdtemp(prefix="assist_bench_")
    pl, ast, system, pop = make_inputs(tmp)
    eph = Ephem(pl, ast)
    dev = torch.device("cuda", local)
    t0 = torch.tensor(pop.t0, device=dev)
    te = torch.tensor(pop.t_end, device=dev)
    st0 = torch.tensor(pop.state, device=dev)
    prm = torch.tensor(pop.params, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MB > L2
    stream = torch.cuda.current_stream(dev)
    opts = batch.options(group_steps=2, warm_start=0, blocks_per_sm=args.blocks_per_sm)
    warm_opts = batch.options(group_steps=2, warm_start=1)
    warm_info = None
    if not args.no_warm:
        warm_info = train_warm_start(eph, system, dev)

    def timed(o):
        st = st0.clone()
        status = torch.zeros(N_PARTICLES, dtype=torch.int32, device=dev)
        for _ in range(args.warmup):
            st.copy_(st0)
            batch.integrate_batch_device(eph, t0, te, st, params=prm, status=status, opts=o, stream=stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        evs, acc = [], None
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            st.copy_(st0)
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s = batch.integrate_batch_device(eph, t0, te, st, params=prm, status=status, opts=o, stream=stream)
            e1.record(stream)
            evs.append((e0, e1))
            if acc is None:
                acc = dict(s)
            else:
                for k in ("steps_accepted", "steps_rejected", "force_evals", "pc_iterations", "kernel_ms",
                          "warm_start_used", "warm_start_fallback"):
                    acc[k] += s[k]
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        wall = time.perf_counter() - wall0
        ms = sum(a.elapsed_time(b) for a, b in evs)
        if world > 1:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, acc, status.cpu().numpy(), st, wall

    # the learned warm start, measured beside the plain predictor (the default path)
    learned = None
    if not args.no_warm:
        lms, lacc, lstat, lst, _ = timed(warm_opts)
        ldone = lstat == 0
        learned = {"value": world * float(np.abs(pop.t_end - pop.t0)[ldone].sum()) * args.steps / (lms / 1e3),
                   "unit": UNIT, "ms_per_step": lms / args.steps,
                   "iterations_per_step": lacc["pc_iterations"] / max(lacc["steps_accepted"] + lacc["steps_rejected"], 1),
                   "force_evals": lacc["force_evals"] // args.steps,
                   "used": lacc["warm_start_used"] // args.steps, "fallback": lacc["warm_start_fallback"] // args.steps}
    clocks = ClockSampler(local)
    clocks.start()
    ms, stats_acc, st_host, st_dev, wall = timed(opts)
    clocks.stop()
    # particle-days of the particles that reached t_end (a particle that hits a
    # body stops with status 4 and its span is not counted)
    done = st_host == 0
    pdays = float(np.abs(pop.t_end - pop.t0)[done].sum())
    bad = int((~done).sum())
    status_counts = {str(k): int(v) for k, v in zip(*np.unique(st_host, return_counts=True))}
    value = world * pdays * args.steps / (ms / 1e3)
    if learned is not None:
        both = done & ldone
        d = np.abs(st_dev.cpu().numpy()[both, :3] - lst.cpu().numpy()[both, :3]).max(axis=1)
        learned["ratio_to_plain"] = learned["value"] / (world * pdays * args.steps / (ms / 1e3))
        learned["end_state_vs_plain_au"] = {"median": float(np.median(d)), "max": float(d.max()),
                                            "particles_over_1e-9": int((d > 1e-9).sum()),
                                            "status_mismatches": int((st_host != lstat).sum())}
        learned.update(warm_info)
    # e2e through the host-array C entry point
    e2e = None
    if rank == 0:
        h_st = pop.state.copy()
        t = time.perf_counter()
        out, _, hstat, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, h_st, params=pop.params, opts=opts)
        e2e_s = time.perf_counter() - t
        h2d = pop.t0.nbytes * 2 + pop.state.nbytes + pop.params.nbytes
        d2h = pop.state.nbytes + hstat.nbytes
        e2e = {"value": float(np.abs(pop.t_end - pop.t0)[hstat == 0].sum()) / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    flops, per_eval, counts = algorithmic_flops(pl, ast, pop, stats_acc)
    kernel_s = stats_acc["kernel_ms"] / 1e3
    peak = batch.fp64_peak_gflops() * 1e9
    achieved = flops / kernel_s
    # DRAM bytes per launch: 0.351 B per particle-day, from one ncu capture of
    # this kernel (three-blocks-per-SM build) on the 32,768-particle case of
    # this workload (dram__bytes_read + dram__bytes_write: 4.20 MB for 11.97M
    # particle-days), scaled by the particle-days of a full launch
    traffic = 0.351 * pdays
    roof = {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic, "traffic_unit": "bytes per launch (scaled from ncu)",
            "peak_source": "measured in this run (FP64 FMA chains; MEASURED_PEAKS.json has no FP64 figure)",
            "flops_per_force_eval": per_eval, "op_counts_per_eval": counts}
    cpu = None if args.no_cpu_baseline else cpu_baseline(pl, ast, pop)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded .440/SPK ephemeris, seeded population)",
            "config": {"workload": WORKLOAD, "n_particles": N_PARTICLES,
                       "particle_days_per_step": pdays, "epsilon": 1e-9, "forces": "0x7F (ASSIST default)",
                       "warm_start": "plain predictor (the default; the learned warm start is measured "
                                     "beside it under learned_warm_start)",
                       "l2": "flushed (256 MB write) between steps", "kernel": "block-cooperative groups (group_steps=2)",
                       "parallelism": "dp%d (independent batches, no collective)" % world},
            # per step: the encounter pilot's two kernels and the IAS15 kernel
            "gpu_launches": 3 * args.steps,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "ias15": {"kernel_ms_per_step": stats_acc["kernel_ms"] / args.steps,
                      "steps_accepted": stats_acc["steps_accepted"] // args.steps,
                      "steps_rejected": stats_acc["steps_rejected"] // args.steps,
                      "force_evals": stats_acc["force_evals"] // args.steps,
                      "iterations_per_step": stats_acc["pc_iterations"] / max(stats_acc["steps_accepted"] +
                                                                              stats_acc["steps_rejected"], 1)},
            "unfinished_particles": bad, "status_counts": status_counts, "wall_s_timed_region": wall,
            "learned_warm_start": learned}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
