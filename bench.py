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
          inputs resident in HBM, CUDA events around the call on its stream,
          L2 flushed (256 MB write) between steps.
  learned_warm_start : the same with the learned warm start, timed beside it.
  e2e   : the default path through the public host-array C entry point
          assist_gb300_integrate_batch (H2D + grouping + kernel + D2H in the
          timed region), averaged over --steps calls.
  roofline : FP64 pipe.  achieved = the FP64 work the kernel does / kernel
          time: per force evaluation the particle-dependent force terms, per
          body table (all bodies at one time, one per group and node time)
          the ephemeris and the particle-independent force-term parts, plus
          IAS15 bookkeeping (op counts from the oracle's counting type);
          peak = FP64 FMA throughput measured in this run.
  cpu_baseline : the oracle (CPU restatement of ASSIST's forces + IAS15) on all
          host cores over the population (bounded by a time budget).
  parity : the GPU end states (plain and learned paths) against the oracle's
          for every particle the CPU baseline integrated.
  configs : the batched mixed-length population (65,536 particles, lengths
          logU[30 d, 10 yr]) and the variational population (1,048,576
          particles x 6 variational particles, lengths logU[30 d, 5 yr], 1% on
          close Earth approaches), each timed with an oracle parity sample;
          and the shared-step drop-in (one REBOUND simulation through
          sim.integrate) at 1,024 main-belt particles over one year and at
          4,096 NEOs x 6 variational particles over ten years and back, each
          beside the oracle's shared-step IAS15 on one CPU thread.

--impl reference times that CPU path alone (the reference arm); it loads no
part of this library.  Multi-GPU (torchrun): weak scaling, each rank
integrates its own batch of the same size; no collective on the data path.
"""
from __future__ import annotations

import argparse
import importlib.util
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

# IAS15 bookkeeping per force evaluation (predictor of x and v, divided
# differences and b update) and per accepted step (compensated x, v update,
# next-step prediction), FP64 operations per particle
IAS_PER_EVAL = 3 * (34 + 16)
IAS_PER_STEP = 3 * (2 * 9 + 2 * 8 + 8 + 7 * 8)

# From one ncu capture of the block-cooperative kernel (three-blocks-per-SM
# build) on the 32,768-particle case of this workload
# (profiles/ag_k_coop_32768_mixture_1yr.md: 4.64 MB read + written for 11.97M
# particle-days): DRAM bytes per particle-day of a launch, scaled to a full
# launch by its particle-days.
DRAM_BYTES_PER_PARTICLE_DAY = 0.388


def _synth():
    """assist_gb300/synth.py loaded by path: it needs only numpy, and the
    reference arm must not load the library (importing the package does)."""
    name = "assist_gb300_synth_standalone"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, "assist_gb300", "synth.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def make_inputs(tmpdir: str):
    synth = _synth()
    pl, ast, system = synth.write_ephemeris(tmpdir, seed=SEED_EPHEM, t_beg=T0 - 40.0, t_end=T0 + 3700.0)
    pop = synth.population(system, "mix", N_PARTICLES, seed=SEED_POP, t0=T0, length=LENGTH, nongrav_frac=0.1)
    return pl, ast, system, pop


def op_model(pl, ast, pop):
    """FP64 operations of one force evaluation from the oracle's counting
    type (add, sub, mul = 1; div and sqrt = 1 each; no FMA credit), split into
    the part that depends on the particle and the part a shared body table
    does once: all bodies at one time plus the particle-independent pieces of
    the force terms (origin-minus-body offsets, EIH source-source sums).
    For a particle without non-gravitational parameters (90 % of the mix)."""
    from tests.oracle_py import Oracle
    o = Oracle(pl, ast)
    i_plain = int(np.nonzero(np.abs(pop.params).sum(1) == 0)[0][0])
    c = o.count_ops(T0, pop.state[i_plain])
    s = lambda d: int(sum(d[k] for k in ("add", "mul", "div", "sqrt", "pow")))
    bodies, shared, total = s(c["bodies"]), s(c["shared"]), s(c)
    return {"per_eval_particle": total - bodies, "per_body_table": bodies + shared,
            "per_eval_independent": total + shared, "ias15_per_eval": IAS_PER_EVAL, "ias15_per_step": IAS_PER_STEP,
            "op_counts": {k: c[k] for k in ("add", "mul", "div", "sqrt", "pow")},
            "op_counts_bodies": c["bodies"], "op_counts_shared": c["shared"]}


def roofline(stats, model, kernel_s, peak, pdays):
    """FP64 roofline of the IAS15 kernel from its counters."""
    ev, tabs, acc = stats["force_evals"], stats["tables_built"], stats["steps_accepted"]
    work = ev * (model["per_eval_particle"] + IAS_PER_EVAL) + tabs * model["per_body_table"] + acc * IAS_PER_STEP
    indep = ev * (model["per_eval_independent"] + IAS_PER_EVAL) + acc * IAS_PER_STEP
    roof = {"bound": "fp64", "achieved": work / kernel_s / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": work / kernel_s / peak, "traffic": DRAM_BYTES_PER_PARTICLE_DAY * pdays,
            "traffic_unit": "DRAM bytes per launch (ncu, 32,768-particle case of this kernel, scaled by particle-days)",
            "peak_source": "measured in this run (FP64 FMA chains; MEASURED_PEAKS.json has no FP64 figure)",
            "work": "per force evaluation %d flop of particle-dependent force terms + %d IAS15; per body table "
                    "%d flop (ephemeris + particle-independent force-term parts); per accepted step %d"
                    % (model["per_eval_particle"], IAS_PER_EVAL, model["per_body_table"], IAS_PER_STEP),
            "flops_per_launch": work, "force_evals": ev, "body_tables": tabs,
            "frac_vs_independent": indep / kernel_s / peak,
            "frac_vs_independent_note": "the work of independent steps (every evaluation evaluating all bodies at "
                                        "its own time, %d flop + IAS15) per the kernel's evaluations: a throughput "
                                        "ratio against that algorithm, not pipe occupancy" % model["per_eval_independent"],
            "model": model}
    return roof


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
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


def oracle_batch(o, pop, idx, threads, var=None, chunk=16384, budget_s=None):
    """The oracle's independent integrations of particles idx (in chunks, all
    threads), stopping after the chunk that passes budget_s.  Returns the
    indices done, their end states, statuses (and variational states) and
    the wall time."""
    done, states, stats, vstates = [], [], [], []
    t = time.perf_counter()
    for k in range(0, len(idx), chunk):
        j = idx[k:k + chunk]
        st, vs, s, _ = o.integrate_batch(pop.t0[j], pop.t_end[j], pop.state[j], params=pop.params[j],
                                         var_state=None if var is None else var[j], threads=threads, return_all=True)
        done.append(j); states.append(st); stats.append(s)
        if var is not None:
            vstates.append(vs)
        if budget_s is not None and time.perf_counter() - t > budget_s:
            break
    wall = time.perf_counter() - t
    return (np.concatenate(done), np.concatenate(states), np.concatenate(stats),
            np.concatenate(vstates) if vstates else None, wall)


def parity(idx, ref, rstat, gpu, gstat, vref=None, vgpu=None):
    """End-state agreement on the particles idx (both completed)."""
    both = (rstat == 0) & (gstat[idx] == 0)
    d = np.abs(gpu[idx][both, :3] - ref[both, :3]).max(axis=1) if both.any() else np.zeros(1)
    mism = np.nonzero(rstat != gstat[idx])[0]
    out = {"n": int(both.sum()), "sampled": int(len(idx)), "median_au": float(np.median(d)), "max_au": float(d.max()),
           "over_1e-9": int((d > 1e-9).sum()), "status_mismatches": int(mism.size),
           "mismatched_status_gpu_oracle": [[int(gstat[idx][k]), int(rstat[k])] for k in mism[:8]]}
    if vref is not None:
        vg = vgpu[idx][both]
        vr = vref[both]
        rel = np.abs(vg - vr).max(axis=(1, 2)) / np.maximum(np.abs(vr).max(axis=(1, 2)), 1e-300)
        out["variational_rel_max"] = float(rel.max()) if rel.size else 0.0
        out["variational_rel_median"] = float(np.median(rel)) if rel.size else 0.0
    return out


def run_reference(args):
    """The reference arm: the oracle's IAS15 over the workload on all host
    threads, nothing of this library loaded."""
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


def timed_batch(batch, eph, t0, te, st0, prm, o, steps, warmup, stream, flush, world=1, var0=None, dist=None):
    """W untimed then K timed passes of integrate_batch_device over the same
    inputs (state reset before each); CUDA events around each call on its
    stream.  Returns (ms total, summed stats, status, end state, var end
    state, wall seconds)."""
    import torch
    dev = st0.device
    st = st0.clone()
    var = None if var0 is None else var0.clone()
    status = torch.zeros(st0.shape[0], dtype=torch.int32, device=dev)
    for _ in range(warmup):
        st.copy_(st0)
        if var is not None:
            var.copy_(var0)
        batch.integrate_batch_device(eph, t0, te, st, params=prm, var_state=var, status=status, opts=o, stream=stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    evs, acc = [], None
    wall0 = time.perf_counter()
    for _ in range(steps):
        flush.fill_(1.0)
        st.copy_(st0)
        if var is not None:
            var.copy_(var0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s = batch.integrate_batch_device(eph, t0, te, st, params=prm, var_state=var, status=status, opts=o,
                                         stream=stream)
        e1.record(stream)
        evs.append((e0, e1))
        if acc is None:
            acc = dict(s)
        else:
            for k in s:
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
    return ms, acc, status.cpu().numpy(), st.cpu().numpy(), None if var is None else var.cpu().numpy(), wall


def ias15_summary(acc, steps):
    return {"kernel_ms_per_step": acc["kernel_ms"] / steps,
            "steps_accepted": acc["steps_accepted"] // steps, "steps_rejected": acc["steps_rejected"] // steps,
            "force_evals": acc["force_evals"] // steps, "body_tables": acc["tables_built"] // steps,
            "iterations_per_step": acc["pc_iterations"] / max(acc["steps_accepted"] + acc["steps_rejected"], 1),
            "warm_start_used": acc["warm_start_used"] // steps, "warm_start_fallback": acc["warm_start_fallback"] // steps}


def extra_config(name, desc, batch, eph, o_cpu, pop, opts, steps, warmup, stream, flush, dev, sample, threads,
                 var=None):
    """One more configuration of the batched path: timed passes and an oracle
    parity sample."""
    import torch
    t0 = torch.tensor(pop.t0, device=dev)
    te = torch.tensor(pop.t_end, device=dev)
    st0 = torch.tensor(pop.state, device=dev)
    prm = torch.tensor(pop.params, device=dev)
    v0 = None if var is None else torch.tensor(var, device=dev)
    ms, acc, stat, st, vst, _ = timed_batch(batch, eph, t0, te, st0, prm, opts, steps, warmup, stream, flush, var0=v0)
    done = stat == 0
    pdays = float(np.abs(pop.t_end - pop.t0)[done].sum())
    rng = np.random.default_rng(5)
    idx = np.sort(rng.choice(pop.t0.size, size=min(sample, pop.t0.size), replace=False))
    didx, ref, rstat, vref, cpu_s = oracle_batch(o_cpu, pop, idx, threads, var=var, chunk=max(len(idx), 1))
    status_counts = {str(k): int(v) for k, v in zip(*np.unique(stat, return_counts=True))}
    del t0, te, st0, prm, v0
    return {"name": name, "description": desc, "n_particles": int(pop.t0.size),
            "n_var_per_particle": 0 if var is None else 6, "value": pdays * steps / (ms / 1e3), "unit": UNIT,
            "ms_per_step": ms / steps, "steps": steps, "warmup": warmup, "particle_days_per_step": pdays,
            "ias15": ias15_summary(acc, steps), "status_counts": status_counts,
            "parity": parity(didx, ref, rstat, st, stat, vref, vst),
            "parity_oracle_s": cpu_s}


def _dropin_sim(eph, state, var_tp=()):
    """One REBOUND simulation with ASSIST attached (the drop-in surface):
    real particles, then unit-deviation variational particles in x, y, z,
    vx, vy, vz order for each entry of var_tp."""
    from assist_gb300 import Extras, Simulation
    sim = Simulation.create()
    ex = Extras(sim, eph)
    for s in state:
        sim.add(*s)
    for k, i in enumerate(var_tp):
        p = sim.particle(sim.add_variation(int(i)))
        setattr(p, ["x", "y", "z", "vx", "vy", "vz"][k % 6], 1.0)
    sim.t = T0
    return sim, ex


def _dropin_run(sim, t1, budget_s, chunk=365.25):
    """sim.integrate(t1) in chunks of simulated time: wall seconds, or None
    when past budget_s (one shared step is as small as the smallest any
    particle asks for)."""
    start = time.perf_counter()
    d = 1.0 if t1 >= sim.t else -1.0
    while sim.t != t1:
        nxt = sim.t + d * chunk
        sim.integrate(t1 if d * (nxt - t1) >= 0 else nxt)
        if sim.status != 0 or time.perf_counter() - start > budget_s:
            return None
    return time.perf_counter() - start


def shared_configs(eph, system, o_cpu, runs):
    """The shared-step drop-in at its two configuration sizes, through the
    REBOUND/ASSIST surface (host particles in, host particles out, the host's
    step control around the device's step kernel): wall time of
    sim.integrate, parity with the oracle's shared-step IAS15 (the same
    method on the CPU, one thread, timed as the CPU baseline)."""
    synth = _synth()
    AU_M = 149597870700.0
    out = []
    # 1,024 main-belt particles, one year
    pop = synth.population(system, "mba", 1024, seed=SEED_POP + 10, t0=T0)
    sim, ex = _dropin_sim(eph, pop.state)
    _dropin_run(sim, T0 + 30.0, 60.0)                 # untimed: first use of the step kernel
    ex.detach(sim); sim.free()
    walls, steps = [], 0
    for _ in range(runs):
        sim, ex = _dropin_sim(eph, pop.state)
        w = _dropin_run(sim, T0 + LENGTH, 120.0)
        steps = sim.steps_done
        g = np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])
        ex.detach(sim); sim.free()
        if w is None:
            break
        walls.append(w)
    t = time.perf_counter()
    r, _, info = o_cpu.integrate(T0, T0 + LENGTH, pop.state)
    cpu_s = time.perf_counter() - t
    dx = np.abs(g[:, :3] - r[:, :3]).max(axis=1)
    pdays = 1024 * LENGTH
    out.append({"name": "shared-step-1024-main-belt-1yr",
                "description": "one REBOUND simulation of 1,024 main-belt particles sharing the IAS15 step "
                               "(epsilon 1e-9), 365.25 days, through sim.integrate with ASSIST attached",
                "n_particles": 1024, "value": pdays / np.mean(walls) if walls else None, "unit": UNIT,
                "wall_s": float(np.mean(walls)) if walls else None, "runs": len(walls),
                "wall_s_runs": [float(w) for w in walls], "steps": int(steps),
                "us_per_step": 1e6 * float(np.mean(walls)) / max(steps, 1) if walls else None,
                "parity": {"max_au": float(dx.max()), "median_au": float(np.median(dx)),
                           "oracle_steps": info["accepted"]},
                "cpu_baseline": {"value": pdays / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                                 "us_per_step": 1e6 * cpu_s / max(info["accepted"], 1),
                                 "sample": "the whole configuration: the oracle's shared-step IAS15, %.1f s" % cpu_s}})
    # 4,096 NEOs x 6 variational particles, ten years forward and back
    n = 4096
    pop = synth.population(system, "neo", n, seed=33, t0=T0)
    var_tp = np.repeat(np.arange(n), 6)
    sim, ex = _dropin_sim(eph, pop.state, var_tp)
    w_f = _dropin_run(sim, T0 + 3652.5, 300.0)
    steps_f = sim.steps_done
    w_b = None
    if w_f is not None:
        sim.dt = -sim.dt
        w_b = _dropin_run(sim, T0, 300.0)
    steps_b = sim.steps_done - steps_f
    g = np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])
    ex.detach(sim); sim.free()
    line = {"name": "shared-step-4096-neo-x6-variational-10yr-roundtrip",
            "description": "one REBOUND simulation of 4,096 NEOs (seed 33: no impactor over the ten years), each "
                           "with 6 variational particles (unit deviations), sharing the IAS15 step: 10 years forward, "
                           "then back to the start; value counts real particle-days both ways",
            "n_particles": n, "n_var_per_particle": 6, "unit": UNIT, "steps_forward": int(steps_f),
            "steps_back": int(steps_b)}
    if w_f is not None and w_b is not None:
        wall = w_f + w_b
        dxm = np.abs(g[:n, :3] - pop.state[:, :3]).max(axis=1) * AU_M
        var0 = np.tile(np.eye(6), (n, 1))
        dv = np.abs(g[n:] - var0).reshape(n, 6, 6).max(axis=(1, 2))
        line.update({"value": 2 * n * 3652.5 / wall, "wall_s": wall,
                     "us_per_step": 1e6 * wall / max(steps_f + steps_b, 1),
                     "roundtrip": {"position_median_m": float(np.median(dxm)), "position_max_m": float(dxm.max()),
                                   "variational_identity_median": float(np.median(dv)),
                                   "variational_identity_max": float(dv.max())}})
    else:
        line.update({"value": None, "unfinished": "past its wall budget or a status"})
    # parity and CPU baseline: the first 10 days against the oracle
    sim, ex = _dropin_sim(eph, pop.state, var_tp)
    sim.integrate(T0 + 10.0)
    g = np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])
    gsteps = sim.steps_done
    ex.detach(sim); sim.free()
    t = time.perf_counter()
    r, rv, info = o_cpu.integrate(T0, T0 + 10.0, pop.state, var_state=np.tile(np.eye(6), (n, 1)),
                                  var_tp=var_tp.astype(np.int32))
    cpu_s = time.perf_counter() - t
    rel = np.abs(g[n:] - rv).reshape(n, 6, 6).max(axis=(1, 2)) / np.abs(rv).reshape(n, 6, 6).max(axis=(1, 2))
    line["parity_first_10_days"] = {"max_au": float(np.abs(g[:n, :3] - r[:, :3]).max()),
                                    "variational_rel_max": float(rel.max()), "steps": int(gsteps),
                                    "oracle_steps": info["accepted"]}
    line["cpu_baseline"] = {"value": n * 10.0 / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                            "us_per_step": 1e6 * cpu_s / max(info["accepted"], 1),
                            "sample": "the first 10 days (steps there are shorter than the ten-year average: "
                                      "compare us_per_step), the oracle's shared-step IAS15 with the variational "
                                      "particles, %.1f s" % cpu_s}
    out.append(line)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-warm", action="store_true", help="plain predictor only (no learned warm start)")
    ap.add_argument("--no-configs", action="store_true", help="skip the extra configuration lines")
    ap.add_argument("--blocks-per-sm", type=int, default=0,
                    help="block-cooperative kernel residency: 0 automatic (the library's choice), 2 or 3")
    ap.add_argument("--ephem-staging", type=int, default=0,
                    help="block-cooperative kernel: 0 automatic, 1 .440 record staged in shared memory, 2 not")
    ap.add_argument("--group-order", type=int, default=0, help="grouping of the batch (options.group_order)")
    ap.add_argument("--particles", type=int, default=None, help="override the batch size (profiling only)")
    ap.add_argument("--cpu-budget-s", type=float, default=60.0,
                    help="time budget of the oracle's CPU baseline / parity pass over the population")
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
    from assist_gb300 import Ephem, batch, warm
    tmp = tempfile.mkdtemp(prefix="assist_bench_")
    pl, ast, system, pop = make_inputs(tmp)
    synth = _synth()
    eph = Ephem(pl, ast)
    dev = torch.device("cuda", local)
    t0 = torch.tensor(pop.t0, device=dev)
    te = torch.tensor(pop.t_end, device=dev)
    st0 = torch.tensor(pop.state, device=dev)
    prm = torch.tensor(pop.params, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MB > L2
    stream = torch.cuda.current_stream(dev)
    opts = batch.options(group_steps=2, warm_start=0, blocks_per_sm=args.blocks_per_sm,
                         ephem_staging=args.ephem_staging, group_order=args.group_order)
    warm_opts = batch.options(group_steps=2, warm_start=1)
    warm_info = None
    if not args.no_warm:
        # pairs logged from a plain run of a separate population, training by
        # the device kernels (outside every timed region)
        tp = synth.population(system, "mix", N_TRAIN, seed=SEED_POP + 1, t0=T0, log_len=(30.0, 3652.5),
                              nongrav_frac=0.1)
        t = time.perf_counter()
        warm.init(SEED_POP)
        X, T, _ = warm.collect(eph, torch.tensor(tp.t0, device=dev), torch.tensor(tp.t_end, device=dev),
                               torch.tensor(tp.state, device=dev), params=torch.tensor(tp.params, device=dev),
                               capacity=5 << 20, every=1)
        perm = torch.randperm(X.shape[0], device=dev, generator=torch.Generator(device=dev).manual_seed(0))
        X, T = X[perm].contiguous(), T[perm].clamp(-4, 4).contiguous()
        l0, _ = warm.grad(X[:4096], T[:4096])
        loss = warm.train(X, T, steps=1500, batch=4096, lr=1e-3, seed=1)
        torch.cuda.synchronize()
        warm_info = {"pairs": int(X.shape[0]), "train_particles": N_TRAIN, "train_steps": 1500, "batch": 4096,
                     "loss_initial": l0, "loss_final": loss, "train_s": time.perf_counter() - t}
        del X, T

    # build selection (outside every timed region): the autotuner times the
    # default kernel's builds on this batch and records the fastest, which
    # the automatic mode then uses; with the learned warm start requested it
    # also times the learned build against them
    tune = (batch.autotune_device(eph, t0, te, st0, params=prm, opts=opts)
            if args.blocks_per_sm == 0 and args.ephem_staging == 0 else None)
    tune_warm = None
    if not args.no_warm:
        tune_warm = batch.autotune_device(eph, t0, te, st0, params=prm, opts=warm_opts)

    def learned_line(o, steps, warmup):
        lms, lacc, lstat_, lst_, _, _ = timed_batch(batch, eph, t0, te, st0, prm, o, steps, warmup, stream, flush,
                                                    world, dist=dist)
        ldone = lstat_ == 0
        d = {"value": world * float(np.abs(pop.t_end - pop.t0)[ldone].sum()) * steps / (lms / 1e3),
             "unit": UNIT, "ms_per_step": lms / steps, "steps": steps, "warmup": warmup,
             "iterations_per_step": lacc["pc_iterations"] / max(lacc["steps_accepted"] + lacc["steps_rejected"], 1),
             "force_evals": lacc["force_evals"] // steps,
             "used": lacc["warm_start_used"] // steps, "fallback": lacc["warm_start_fallback"] // steps}
        return d, lstat_, lst_

    # the learned warm start, measured beside the plain predictor (the default
    # path): warm_start = 1 (learned unless the autotuner found the plain
    # predictor faster on this batch; groups and members fall back on their
    # own), then the learned build regardless (2) and on every step without
    # the time test (3), the last two as diagnostics over fewer steps
    learned, lstat, lst = None, None, None
    if not args.no_warm:
        learned, lstat, lst = learned_line(warm_opts, args.steps, args.warmup)
        learned["mode"] = "warm_start=1: learned unless the autotuner recorded the plain predictor faster"
        learned["autotune"] = tune_warm
        forced, _, _ = learned_line(batch.options(group_steps=2, warm_start=2), min(args.steps, 2), 1)
        every, _, _ = learned_line(batch.options(group_steps=2, warm_start=3), min(args.steps, 2), 1)
        learned["learned_build_forced"] = forced
        learned["every_step_no_time_test"] = every
    clocks = ClockSampler(local)
    clocks.start()
    ms, stats_acc, st_host, st_end, _, wall = timed_batch(batch, eph, t0, te, st0, prm, opts, args.steps, args.warmup,
                                                           stream, flush, world, dist=dist)
    clocks.stop()
    # particle-days of the particles that reached t_end (a particle that hits a
    # body stops with status 4 and its span is not counted)
    done = st_host == 0
    pdays = float(np.abs(pop.t_end - pop.t0)[done].sum())
    status_counts = {str(k): int(v) for k, v in zip(*np.unique(st_host, return_counts=True))}
    value = world * pdays * args.steps / (ms / 1e3)
    if learned is not None:
        both = done & (lstat == 0)
        d = np.abs(st_end[both, :3] - lst[both, :3]).max(axis=1)
        learned["ratio_to_plain"] = learned["value"] / value
        learned["learned_build_forced"]["ratio_to_plain"] = learned["learned_build_forced"]["value"] / value
        learned["every_step_no_time_test"]["ratio_to_plain"] = learned["every_step_no_time_test"]["value"] / value
        learned["end_state_vs_plain_au"] = {"median": float(np.median(d)), "max": float(d.max()),
                                            "particles_over_1e-9": int((d > 1e-9).sum()),
                                            "status_mismatches": int((st_host != lstat).sum())}
        learned.update(warm_info)
    # e2e through the host-array C entry point (inputs from host memory, end
    # states and statuses back to it every call), averaged over --steps calls
    e2e = None
    if rank == 0:
        h_st = pop.state.copy()
        batch.integrate_batch(eph, pop.t0, pop.t_end, h_st, params=pop.params, opts=opts)     # untimed
        e2e_s, e2e_days = 0.0, 0.0
        for _ in range(args.steps):
            t = time.perf_counter()
            out, _, hstat, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, h_st, params=pop.params, opts=opts)
            e2e_s += time.perf_counter() - t
            e2e_days += float(np.abs(pop.t_end - pop.t0)[hstat == 0].sum())
        h2d = pop.t0.nbytes * 2 + pop.state.nbytes + pop.params.nbytes
        d2h = pop.state.nbytes + hstat.nbytes
        e2e = {"value": e2e_days / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "calls": args.steps, "ms_per_call": 1e3 * e2e_s / args.steps}
    # the same batch as a plan: host work once, each step a CUDA-graph replay
    graph = None
    if rank == 0:
        gst = st0.clone()
        gstat = torch.zeros(N_PARTICLES, dtype=torch.int32, device=dev)
        plan = batch.Plan(eph, t0, te, gst, params=prm, status=gstat, opts=opts, stream=stream)
        gms = 0.0
        for k in range(args.warmup + args.steps):
            flush.fill_(1.0)
            gst.copy_(st0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.launch(stream)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= args.warmup:
                gms += e0.elapsed_time(e1)
        gstats = plan.stats()
        plan.close()
        same = bool(torch.equal(gst.cpu(), torch.tensor(st_end)))
        graph = {"value": pdays * args.steps / (gms / 1e3), "unit": UNIT, "ms_per_step": gms / args.steps,
                 "force_evals": gstats["force_evals"], "end_states_equal_direct_call": same,
                 "note": "assist_gb300_plan_*: grouping once, each step a CUDA-graph replay of the device work"}
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    model = op_model(pl, ast, pop)
    kernel_s = stats_acc["kernel_ms"] / 1e3
    peak = batch.fp64_peak_gflops() * 1e9
    roof = roofline(stats_acc, model, kernel_s, peak, pdays)
    # CPU baseline and parity: the oracle over the population (random order,
    # all host threads, bounded by --cpu-budget-s), its end states compared
    # with the GPU's
    from tests.oracle_py import Oracle
    o_cpu = Oracle(pl, ast)
    threads = os.cpu_count() or 1
    cpu, par, par_learned = None, None, None
    if not args.no_cpu_baseline:
        order = np.random.default_rng(7).permutation(pop.t0.size)
        didx, ref, rstat, _, cpu_s = oracle_batch(o_cpu, pop, order, threads, budget_s=args.cpu_budget_s)
        cdays = float(np.abs(pop.t_end[didx] - pop.t0[didx])[rstat == 0].sum())
        cpu = {"value": cdays / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d of the %d particles (random order, seed 7), their full integrations: %.4g particle-days "
                         "in %.1f s" % (len(didx), pop.t0.size, cdays, cpu_s)}
        par = parity(didx, ref, rstat, st_end, st_host)
        if learned is not None:
            par_learned = parity(didx, ref, rstat, lst, lstat)
            learned["parity_vs_oracle"] = par_learned
    configs = None
    if not args.no_configs and world == 1:
        configs = []
        p2 = synth.population(system, "mix", 65536, seed=SEED_POP + 2, t0=T0, log_len=(30.0, 3652.5),
                              nongrav_frac=0.1)
        configs.append(extra_config(
            "batched-65536-mixture-10yr", "65,536 independent particles of the 40/30/20/10 mixture, lengths "
            "logU[30 d, 10 yr], 10% non-gravitational, block-cooperative groups", batch, eph, o_cpu, p2,
            batch.options(group_steps=2), 3, 3, stream, flush, dev, 2048, threads))
        del p2
        p4 = synth.population(system, "mix", 1 << 20, seed=SEED_POP + 4, t0=T0, log_len=(30.0, 1826.25),
                              nongrav_frac=0.1, close_frac=0.01)
        v4 = np.tile(np.eye(6)[None], (p4.t0.size, 1, 1))
        w4 = 0 if args.no_warm else 1
        configs.append(extra_config(
            "variational-1048576x6-mixture-5yr", "1,048,576 particles of the mixture, each with 6 first-order "
            "variational particles (unit deviations), lengths logU[30 d, 5 yr], 10% non-gravitational, 1% on close "
            "Earth approaches (q_min logU[1e-4, 1e-2] AU); " +
            ("learned warm start with the plain-predictor fallbacks" if w4 else "plain predictor") +
            "; value counts real particle-days",
            batch, eph, o_cpu, p4, batch.options(group_steps=2, warm_start=w4), 1, 1, stream, flush, dev, 512,
            threads, var=v4))
        del p4, v4
        configs.extend(shared_configs(eph, system, o_cpu, 3))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded .440/SPK ephemeris, seeded population)",
            "config": {"workload": WORKLOAD, "n_particles": N_PARTICLES,
                       "particle_days_per_step": pdays, "epsilon": 1e-9, "forces": "0x7F (ASSIST default)",
                       "warm_start": "plain predictor (the default; the learned warm start is measured "
                                     "beside it under learned_warm_start)",
                       "l2": "flushed (256 MB write) between steps", "kernel": "block-cooperative groups (group_steps=2)",
                       "precision": "FP64 throughout, except the asteroids' direct terms beyond 0.02 AU of the "
                                    "particle: float pairs (about 48 bits) on the FP32 pipes, below 1e-17 of the "
                                    "acceleration",
                       "parallelism": "dp%d (independent batches, no collective)" % world},
            # per step: the encounter pilot's two kernels and the IAS15 kernel
            "gpu_launches": 3 * args.steps,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "parity": par,
            "clocks": clocks.summary(),
            "ias15": ias15_summary(stats_acc, args.steps),
            "unfinished_particles": int((~done).sum()), "status_counts": status_counts,
            "wall_s_timed_region": wall, "learned_warm_start": learned, "autotune": tune, "graph_replay": graph,
            "configs": configs}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
