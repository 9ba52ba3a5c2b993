"""Device IAS15 (batched persistent kernel and shared-step drop-in) against
the oracle's IAS15 on the oracle's forces: end states within 1e-9 AU (the
bar), round trips, variational equations vs finite differences, and the
error of both paths against the double-double oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
AU_M = 149597870700.0


def _eph(paths):
    from assist_gb300 import Ephem
    return Ephem(*paths)


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_vs_oracle_mixture(synth_files, group_steps):
    """Independent steps (group_steps=0) reproduce the oracle's per-particle
    integrations step for step; warp-synchronous groups (1) take the group's
    smallest step and must stay within the 1e-9 AU end-state bar."""
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "mix", 1024, seed=3, t0=8000.0, log_len=(30.0, 900.0), nongrav_frac=0.1,
                           close_frac=0.01)
    o = batch.options(group_steps=group_steps)
    out, _, status, stats = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, params=pop.params, opts=o)
    ref, _, rstat, rstats = O.integrate_batch(pop.t0, pop.t_end, pop.state, params=pop.params, return_all=True)
    # the 1 % close-approach class holds a few Earth impactors: both sides
    # stop them with the step-underflow status, the rest complete
    assert np.array_equal(status, rstat), (np.nonzero(status)[0], np.nonzero(rstat)[0])
    assert set(np.unique(rstat)) <= {0, 4} and (rstat == 0).mean() > 0.98
    ok = rstat == 0
    dx = np.abs(out[ok, :3] - ref[ok, :3]).max(axis=1)
    assert dx.max() < 1e-9, dx.max()
    if group_steps == 0:
        assert np.median(dx) < 1e-12
        assert abs(stats["steps_accepted"] - rstats["accepted"]) <= 0.01 * rstats["accepted"]
    else:
        assert np.median(dx) < 1e-11


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_fixed_step_from_record_edge(golden_paths, group_steps):
    """Fixed steps from a start time a rounding below a 32-day record
    boundary (the body tables of the step start sit at a record fraction a
    hair below zero) reproduce the oracle's, in every batched kernel."""
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    eph = _eph(golden_paths); O = Oracle(*golden_paths)
    system = synth.SolarSystem(4242)
    t0 = 8000.0 - 1e-10
    pop = synth.population(system, "mix", 64, seed=21, t0=t0, length=2.0)
    o = batch.options(group_steps=group_steps, epsilon=0.0, dt0=0.25)
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, opts=o)
    ref, _, rstat, _ = O.integrate_batch(pop.t0, pop.t_end, pop.state, epsilon=0.0, dt0=0.25, return_all=True)
    assert (status == 0).all() and (rstat == 0).all()
    assert np.abs(out[:, :3] - ref[:, :3]).max() < 1e-13


def test_batch_variational_vs_oracle(synth_files):
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "neo", 64, seed=5, t0=8000.0, log_len=(30.0, 400.0))
    var = np.tile(np.eye(6)[None], (64, 1, 1))
    out, vout, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, var_state=var)
    ref, vref, rstat, _ = O.integrate_batch(pop.t0, pop.t_end, pop.state, var_state=var, return_all=True)
    assert (status == 0).all()
    assert np.abs(out[:, :3] - ref[:, :3]).max() < 1e-9
    rel = np.abs(vout - vref).max(axis=(1, 2)) / np.abs(vref).max(axis=(1, 2))
    assert rel.max() < 1e-7


def test_batch_variational_vs_finite_difference(synth_files):
    """Mirror of the reference's unit_tests/variational_*: 10 m offset vs the
    variational particle, relative difference < 1e-5 after 1 and 100 days."""
    from assist_gb300 import batch, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    p0 = synth.population(system, "mba", 1, seed=6, t0=8000.0).state[0]
    dx = 10.0 / AU_M
    p1 = p0.copy(); p1[0] += dx
    var = np.zeros((2, 6, 6)); var[:, 0, 0] = 1.0
    for t1 in (8001.0, 8100.0):
        out, vout, status, _ = batch.integrate_batch(eph, [8000.0, 8000.0], [t1, t1], np.stack([p0, p1]), var_state=var)
        d1 = out[1, 0] - out[0, 0]
        d2 = vout[0, 0, 0] * dx
        assert abs((d1 - d2) / d1) < 1e-5


def test_batch_roundtrip(synth_files):
    from assist_gb300 import batch, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    pop = synth.population(system, "mix", 256, seed=7, t0=8000.0, length=300.0)
    fwd, _, s1, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state)
    back, _, s2, _ = batch.integrate_batch(eph, pop.t_end, pop.t0, fwd)
    assert (s1 == 0).all() and (s2 == 0).all()
    assert np.abs(back[:, :3] - pop.state[:, :3]).max() * AU_M < 1.0      # < 1 m over 600 days


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_error_vs_double_double(synth_files, group_steps):
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "mix", 8, seed=8, t0=8000.0, length=200.0)
    out, _, _, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, opts=batch.options(group_steps=group_steps))
    for i in range(8):
        dd, _, _ = O.integrate(pop.t0[i], pop.t_end[i], pop.state[i:i + 1], dd=True)
        assert np.abs(out[i, :3] - dd[0, :3]).max() < 1e-11


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_coverage_status(synth_files, group_steps):
    from assist_gb300 import batch, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    pop = synth.population(system, "mba", 4, seed=9, t0=8000.0)
    t_end = np.array([8100.0, 20000.0, 8050.0, 8000.0])
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, t_end, pop.state,
                                              opts=batch.options(group_steps=group_steps))
    assert status[1] == 1 and status[3] == 0
    if group_steps == 0:
        assert status[0] == 0 and status[2] == 0
    assert np.array_equal(out[3], pop.state[3])


def test_shared_step_drop_in_vs_oracle(synth_files):
    from assist_gb300 import Extras, Simulation, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "neo", 48, seed=10, t0=8000.0)
    sim = Simulation.create(); ex = Extras(sim, eph)
    for i in range(48):
        sim.add(*pop.state[i])
    var_tp = []
    for i in range(0, 48, 8):
        for k in range(6):
            idx = sim.add_variation(i)
            p = sim.particle(idx)
            setattr(p, ["x", "y", "z", "vx", "vy", "vz"][k], 1.0)
            var_tp.append(i)
    sim.t = 8000.0
    sim.integrate(8200.0)
    assert sim.status == 0 and sim.t == 8200.0
    g = np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])
    var0 = np.zeros((len(var_tp), 6))
    for q in range(len(var_tp)):
        var0[q, q % 6] = 1.0
    r, rv, info = O.integrate(8000.0, 8200.0, pop.state, var_state=var0, var_tp=np.array(var_tp, np.int32))
    assert np.abs(g[:48, :3] - r[:, :3]).max() < 1e-9
    rel = np.abs(g[48:] - rv).max() / np.abs(rv).max()
    assert rel < 1e-7
    assert sim.steps_done == info["accepted"]
    ex.detach(sim); sim.free()


def test_shared_step_cooperative_launch_equals_per_iteration(synth_files, monkeypatch):
    """Several blocks run a step in one cooperative launch (their maxima meet
    across a grid barrier and every block takes the convergence decision) or
    one launch per iteration (the host decides): the same arithmetic and the
    same decisions, so the same end states bit for bit, real and variational
    particles (5 blocks, some with variational particles)."""
    from assist_gb300 import Extras, Simulation, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    pop = synth.population(system, "neo", 150, seed=12, t0=8000.0)

    def run():
        sim = Simulation.create(); ex = Extras(sim, eph)
        for s in pop.state:
            sim.add(*s)
        for i in range(0, 150, 25):
            for k in range(6):
                setattr(sim.particle(sim.add_variation(i)), ["x", "y", "z", "vx", "vy", "vz"][k], 1.0)
        sim.t = 8000.0
        sim.integrate(8150.0)
        g = np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])
        out = (sim.status, sim.steps_done, g)
        ex.detach(sim); sim.free()
        return out

    st_c, n_c, g_c = run()
    monkeypatch.setenv("ASSIST_GB300_SHARED_COOP", "0")
    st_i, n_i, g_i = run()
    assert st_c == 0 and st_i == 0 and n_c == n_i
    assert np.array_equal(g_c, g_i)


@pytest.mark.parametrize("n", [8, 40])
def test_shared_step_nongrav_variational_vs_oracle(synth_files, n):
    """Shared-step drop-in with Marsden parameters on every real particle and
    variational particles of three kinds per particle: a state deviation, a
    deviation of A1 alone and of A2 alone (ASSIST's particle_params rows
    N_real + v hold the variational particles' parameter deviations).  One
    step-kernel block (8 particles) and two (40)."""
    from assist_gb300 import Extras, Simulation, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "neo", n, seed=12, t0=8000.0)
    rng = np.random.default_rng(4)
    A = np.zeros((n, 3))
    A[:, 0] = rng.choice([-1.0, 1.0], n) * 10 ** rng.uniform(-12, -9, n)
    A[:, 1] = rng.choice([-1.0, 1.0], n) * 10 ** rng.uniform(-12, -9, n)
    A[:, 2] = 10 ** rng.uniform(-13, -11, n)
    var_tp = np.repeat(np.arange(n), 3).astype(np.int32)
    m = var_tp.size
    var0 = np.zeros((m, 6))
    dA = np.zeros((m, 3))
    var0[0::3, 0] = 1.0          # x deviation
    dA[1::3, 0] = 1.0            # A1 deviation
    dA[2::3, 1] = 1.0            # A2 deviation
    sim = Simulation.create(); ex = Extras(sim, eph)
    for i in range(n):
        sim.add(*pop.state[i])
    for k in range(m):
        p = sim.particle(sim.add_variation(int(var_tp[k])))
        p.x, p.y, p.z, p.vx, p.vy, p.vz = var0[k]
    params = np.concatenate([A, dA])
    ex.particle_params = params.ravel()
    sim.t = 8000.0
    sim.integrate(8100.0)
    assert sim.status == 0 and sim.t == 8100.0
    g = np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])
    r, rv, info = O.integrate(8000.0, 8100.0, pop.state, var_state=var0, var_tp=var_tp, params=params)
    assert info["status"] == 0
    assert np.abs(g[:n, :3] - r[:, :3]).max() < 1e-9
    scale = np.abs(rv).max(axis=1)
    assert (scale[1::3] > 0).all() and (scale[2::3] > 0).all()
    rel = np.abs(g[n:] - rv).max(axis=1) / scale
    assert rel.max() < 1e-7
    assert abs(sim.steps_done - info["accepted"]) <= 1
    ex.detach(sim); sim.free()


@pytest.mark.parametrize("n", [6, 48])
@pytest.mark.parametrize("kind", ["geocentric", "spk-planets"])
def test_shared_step_frames_and_formats_vs_oracle(synth_files, synth_files_spk, kind, n):
    """The drop-in's step kernel in ASSIST's geocentric frame (`geocentric =
    1`: states about the Earth, the Earth's acceleration removed) and with the
    planets from an SPK file; every third particle carries one variational
    particle.  One block (6 particles) and two (48)."""
    from assist_gb300 import Extras, Simulation, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files_spk if kind == "spk-planets" else synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "neo", n, seed=24, t0=8000.0)
    state = pop.state.copy()
    geo = 1 if kind == "geocentric" else 0
    if geo:
        earth = np.array(system.body(3, np.array(8000.0))).reshape(2, 3)
        state[:, :3] -= earth[0]; state[:, 3:] -= earth[1]
    var_tp = np.arange(0, n, 3).astype(np.int32)
    var0 = np.zeros((var_tp.size, 6))
    var0[np.arange(var_tp.size), np.arange(var_tp.size) % 6] = 1.0
    sim = Simulation.create(); ex = Extras(sim, eph)
    ex.geocentric = geo
    for s in state:
        sim.add(*s)
    for k, i in enumerate(var_tp):
        p = sim.particle(sim.add_variation(int(i)))
        p.x, p.y, p.z, p.vx, p.vy, p.vz = var0[k]
    sim.t = 8000.0
    sim.integrate(8060.0)
    assert sim.status == 0 and sim.t == 8060.0
    g = np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])
    r, rv, info = O.integrate(8000.0, 8060.0, state, var_state=var0, var_tp=var_tp, geocentric=geo)
    assert info["status"] == 0
    assert np.abs(g[:n, :3] - r[:, :3]).max() < 1e-9
    rel = np.abs(g[n:] - rv).max(axis=1) / np.abs(rv).max(axis=1)
    assert rel.max() < 1e-7
    assert abs(sim.steps_done - info["accepted"]) <= 1
    ex.detach(sim); sim.free()


@pytest.mark.parametrize("n", [1, 200])
def test_shared_step_past_coverage_sets_status(golden_paths, n):
    """A drop-in integration that runs past the ephemeris' end stops with
    ASSIST's coverage error at a time still inside the coverage, with one step
    kernel block (1 particle: the whole corrector loop in one launch) and with
    two (200 particles: one launch per iteration)."""
    from assist_gb300 import Extras, Simulation
    eph = _eph(golden_paths)
    tb, te = eph.time_bounds()
    sim = Simulation.create(); ex = Extras(sim, eph)
    rng = np.random.default_rng(3)
    for _ in range(n):
        a = rng.uniform(2.2, 3.2)
        sim.add(a, 0.0, 0.0, 0.0, 0.01720209895 / np.sqrt(a), 0.0)
    sim.t = te - 40.0
    sim.integrate(te + 40.0)
    assert sim.status == 1 and b"coverage" in sim.error_message
    assert te - 40.0 < sim.t <= te
    assert np.isfinite([sim.particle(i).x for i in range(n)]).all()
    ex.detach(sim); sim.free()


def test_shared_step_roundtrip(synth_files):
    """Mirror of the reference's unit_tests/roundtrip_adaptive_*: forward and back."""
    from assist_gb300 import Extras, Simulation, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    pop = synth.population(system, "mba", 3, seed=11, t0=8000.0)
    sim = Simulation.create(); ex = Extras(sim, eph)
    for i in range(3):
        sim.add(*pop.state[i])
    sim.t = 8000.0
    sim.integrate(8500.0)
    sim.dt = -sim.dt
    sim.integrate(8000.0)
    g = np.array([[p.x, p.y, p.z] for p in sim.particles])
    assert np.abs(g - pop.state[:, :3]).max() * AU_M < 1e-1
    ex.detach(sim); sim.free()


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_fixed_step_bitwise(synth_files, group_steps):
    """epsilon = 0 (fixed dt): the device reproduces the oracle bit for bit."""
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "mix", 64, seed=12, t0=8000.0, length=40.0)
    o = batch.options(epsilon=0.0, dt0=4.0, group_steps=group_steps)
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, opts=o)
    ref = O.integrate_batch(pop.t0, pop.t_end, pop.state, epsilon=0.0, dt0=4.0)
    assert (status == 0).all()
    assert np.abs(out - ref).max() <= 1e-15 * np.abs(ref).max()


@pytest.mark.parametrize("group_steps", [0, 2])
def test_batch_geocentric_vs_oracle(synth_files, group_steps):
    """Geocentric frame (ASSIST's `geocentric = 1`, src/forces.c:72-87, 157-172):
    states relative to the Earth, the Earth's acceleration removed."""
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "neo", 64, seed=23, t0=8000.0, log_len=(20.0, 200.0))
    earth = np.array(system.body(3, np.array(8000.0))).reshape(2, 3)
    geo = pop.state.copy()
    geo[:, :3] -= earth[0]; geo[:, 3:] -= earth[1]
    o = batch.options(group_steps=group_steps, geocentric=1)
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, geo, opts=o)
    ref, _, rstat, _ = O.integrate_batch(pop.t0, pop.t_end, geo, geocentric=1, return_all=True)
    assert np.array_equal(status, rstat)
    ok = rstat == 0
    assert np.abs(out[ok, :3] - ref[ok, :3]).max() < 1e-9


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_spk_planets_vs_oracle(synth_files_spk, group_steps):
    """Planets from an SPK file (ASSIST's default de440.bsp layout: Earth and
    Moon about the Earth-Moon barycentre, constants from the comment area):
    every batched kernel against the oracle."""
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files_spk
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "mix", 256, seed=17, t0=8000.0, log_len=(30.0, 600.0), nongrav_frac=0.1)
    o = batch.options(group_steps=group_steps)
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, params=pop.params, opts=o)
    ref, _, rstat, _ = O.integrate_batch(pop.t0, pop.t_end, pop.state, params=pop.params, return_all=True)
    assert np.array_equal(status, rstat)
    ok = rstat == 0
    dx = np.abs(out[ok, :3] - ref[ok, :3]).max(axis=1)
    assert dx.max() < 1e-9, dx.max()
    if group_steps == 0:
        assert np.median(dx) < 1e-12


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_watchdog_marks_every_unfinished_particle(synth_files, monkeypatch, group_steps):
    """With a run-time budget far below what the batch needs, the kernel
    stops early: every particle it did not finish (taken or still queued)
    says ASSIST_GB300_TIMEOUT (5); a particle reported complete (0) holds
    its end state."""
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    pop = synth.population(system, "mix", 4096, seed=41, t0=8000.0, log_len=(1.0, 400.0))
    monkeypatch.setenv("ASSIST_GB300_WATCHDOG_S", "2e-4")
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state,
                                              opts=batch.options(group_steps=group_steps))
    monkeypatch.delenv("ASSIST_GB300_WATCHDOG_S")
    assert set(np.unique(status)) <= {0, 5}, np.unique(status)
    assert (status == 5).sum() > 2048
    ok = np.nonzero(status == 0)[0]
    if ok.size:
        ref = O.integrate_batch(pop.t0[ok], pop.t_end[ok], pop.state[ok])
        assert np.abs(out[ok, :3] - ref[:, :3]).max() < 1e-9


def test_coop_builds_bitwise_identical(synth_files):
    """The block-cooperative kernel's builds (two and three resident blocks
    per SM; the .440 record staged in shared memory by bulk copies or read
    from global memory) run each group's arithmetic identically: the same
    end states bit for bit, the same step counts."""
    from assist_gb300 import batch, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    pop = synth.population(system, "mix", 2048, seed=43, t0=8000.0, log_len=(30.0, 900.0), nongrav_frac=0.1,
                           close_frac=0.01)
    runs = {}
    for name, kw in (("occ2", dict(blocks_per_sm=2, ephem_staging=2)), ("occ3", dict(blocks_per_sm=3)),
                     ("staged", dict(ephem_staging=1))):
        out, _, status, stats = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, params=pop.params,
                                                      opts=batch.options(group_steps=2, **kw))
        runs[name] = (out, status, stats)
    ref = runs["occ2"]
    for name in ("occ3", "staged"):
        out, status, stats = runs[name]
        assert np.array_equal(status, ref[1]), name
        assert np.array_equal(out, ref[0]), (name, np.abs(out - ref[0]).max())
        assert stats["steps_accepted"] == ref[2]["steps_accepted"] and stats["force_evals"] == ref[2]["force_evals"]


def test_autotune_records_and_uses_a_build(synth_files, tmp_path, monkeypatch):
    """The autotuner times the default kernel's builds on the batch, writes
    its choice under the batch's signature, and an automatic-mode call of a
    batch with that signature gives the forced builds' results."""
    import torch
    from assist_gb300 import batch, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    pop = synth.population(system, "mix", 4096, seed=44, t0=8000.0, log_len=(30.0, 600.0), nongrav_frac=0.1)
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("ASSIST_GB300_TUNE_CACHE", str(cache))
    dev = torch.device("cuda:0")
    t0 = torch.tensor(pop.t0, device=dev); te = torch.tensor(pop.t_end, device=dev)
    st = torch.tensor(pop.state, device=dev); prm = torch.tensor(pop.params, device=dev)
    r = batch.autotune_device(eph, t0, te, st, params=prm)
    assert r["chosen"] in (2, 3, 4) and len(r["candidates_ms"]) == 3
    assert all(v > 0 for v in r["candidates_ms"].values())
    assert torch.equal(st, torch.tensor(pop.state, device=dev))          # the caller's state is not changed
    assert r["signature"] in cache.read_text()
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, params=pop.params)
    ref, _, rstatus, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, params=pop.params,
                                               opts=batch.options(blocks_per_sm=2, ephem_staging=2))
    assert np.array_equal(status, rstatus) and np.array_equal(out, ref)


@pytest.mark.parametrize("group_steps", [0, 2])
def test_plan_graph_replay_bitwise(synth_files, group_steps):
    """A plan's CUDA-graph replays reproduce the direct call bit for bit
    (same inputs, so the same grouping), launch after launch."""
    import torch
    from assist_gb300 import batch, synth
    pl, ast, system = synth_files
    eph = _eph((pl, ast))
    pop = synth.population(system, "mix", 3000, seed=45, t0=8000.0, log_len=(30.0, 600.0), nongrav_frac=0.1)
    dev = torch.device("cuda:0")
    t0 = torch.tensor(pop.t0, device=dev); te = torch.tensor(pop.t_end, device=dev)
    s0 = torch.tensor(pop.state, device=dev); prm = torch.tensor(pop.params, device=dev)
    o = batch.options(group_steps=group_steps)
    direct = s0.clone()
    dstat = torch.zeros(3000, dtype=torch.int32, device=dev)
    ref_stats = batch.integrate_batch_device(eph, t0, te, direct, params=prm, status=dstat, opts=o)
    st = s0.clone()
    status = torch.zeros(3000, dtype=torch.int32, device=dev)
    plan = batch.Plan(eph, t0, te, st, params=prm, status=status, opts=o)
    for _ in range(2):
        st.copy_(s0)
        status.zero_()
        plan.launch()
        stats = plan.stats()
        assert torch.equal(st, direct) and torch.equal(status, dstat)
        assert stats["steps_accepted"] == ref_stats["steps_accepted"]
        assert stats["force_evals"] == ref_stats["force_evals"]
    plan.close()
