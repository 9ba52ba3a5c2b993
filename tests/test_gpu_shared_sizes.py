"""The shared-step drop-in (one REBOUND simulation whose accelerations come
from assist_additional_forces) at full population sizes: 1,024 main-belt
particles over one year, and 4,096 near-Earth particles each carrying six
first-order variational particles, over ten years forward and back.  Every
particle shares one adaptive step (ASSIST's own usage: one simulation holding
the whole population), so the oracle's shared-step IAS15 takes the same
steps and the end states agree to rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
AU_M = 149597870700.0


@pytest.fixture(scope="module")
def ten_year_files(tmp_path_factory):
    """A synthetic ephemeris covering ten years from day 8000 (seed 7)."""
    from assist_gb300 import synth
    d = str(tmp_path_factory.mktemp("synth10"))
    return synth.write_ephemeris(d, seed=7, t_beg=7980.0, t_end=8000.0 + 3652.5 + 20.0)


def _sim(eph, state, var_tp=()):
    from assist_gb300 import Extras, Simulation
    sim = Simulation.create()
    ex = Extras(sim, eph)
    for s in state:
        sim.add(*s)
    for k, i in enumerate(var_tp):
        idx = sim.add_variation(int(i))
        p = sim.particle(idx)
        setattr(p, ["x", "y", "z", "vx", "vy", "vz"][k % 6], 1.0)
    return sim, ex


def _states(sim):
    return np.array([[p.x, p.y, p.z, p.vx, p.vy, p.vz] for p in sim.particles])


def test_shared_step_1024_main_belt_one_year(synth_files):
    from assist_gb300 import Ephem, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = Ephem(pl, ast); O = Oracle(pl, ast)
    pop = synth.population(system, "mba", 1024, seed=31, t0=8000.0)
    sim, ex = _sim(eph, pop.state)
    sim.t = 8000.0
    sim.integrate(8365.25)
    assert sim.status == 0 and sim.t == 8365.25
    g = _states(sim)
    r, _, info = O.integrate(8000.0, 8365.25, pop.state)
    assert info["status"] == 0
    dx = np.abs(g[:, :3] - r[:, :3]).max(axis=1)
    print("1024 main-belt, one year, shared step: %d steps; |dx| median %.2e max %.2e AU"
          % (sim.steps_done, np.median(dx), dx.max()))
    assert dx.max() < 1e-9
    # the step size comes from maxima over 1,024 particles whose last bits
    # differ between the device's summation orders and the oracle's: the
    # step before the end can come out either side of it
    assert abs(sim.steps_done - info["accepted"]) <= 1
    ex.detach(sim); sim.free()


def _integrate_guarded(sim, t1, budget_s, chunk=365.25):
    """sim.integrate(t1) in chunks, failing the test (not hanging it) when the
    wall time passes budget_s: one simulation takes the smallest step any of
    its particles asks for, and a particle on an impact course (ASSIST keeps
    integrating it, as does this drop-in) would shrink that step without end."""
    import time
    start = time.perf_counter()
    d = 1.0 if t1 >= sim.t else -1.0
    while sim.t != t1:
        nxt = sim.t + d * chunk
        sim.integrate(t1 if d * (nxt - t1) >= 0 else nxt)
        assert sim.status == 0, sim.status
        if time.perf_counter() - start > budget_s:
            pytest.fail("shared-step integration past its %.0f s budget at t = %.2f" % (budget_s, sim.t))


def test_shared_step_4096_neo_variational_ten_years_and_back(ten_year_files):
    """4,096 NEOs (q ~ U[0.9, 1.3] AU), each with six variational particles of
    unit initial deviation in x, y, z, vx, vy, vz: against the oracle over the
    first 30 days, then on to ten years and back to the start.  Back at the
    start the positions return to their initial values and the variational
    states to the identity (the linearised flow and its inverse).  The seed's
    population holds no impactor over the ten years (the oracle, integrating
    each particle alone with a 1e-6 day step floor, stops none of them); about
    half of such populations do, and one shared-step simulation cannot leave
    such a particle behind."""
    from assist_gb300 import Ephem, synth
    from tests.oracle_py import Oracle
    pl, ast, system = ten_year_files
    eph = Ephem(pl, ast); O = Oracle(pl, ast)
    n = 4096
    pop = synth.population(system, "neo", n, seed=33, t0=8000.0)
    var_tp = np.repeat(np.arange(n), 6)
    sim, ex = _sim(eph, pop.state, var_tp)
    assert sim.N == 7 * n
    sim.t = 8000.0
    sim.integrate(8030.0)
    assert sim.status == 0
    g = _states(sim)
    var0 = np.tile(np.eye(6), (n, 1))
    r, rv, info = O.integrate(8000.0, 8030.0, pop.state, var_state=var0, var_tp=var_tp.astype(np.int32))
    # one shared step for 4,096 particles: its size comes from maxima over
    # them, whose last bits differ between the device's and the oracle's
    # summation orders, and the last step before 8030 can come out either way
    assert info["status"] == 0 and abs(sim.steps_done - info["accepted"]) <= 1
    assert np.abs(g[:n, :3] - r[:, :3]).max() < 1e-9
    rel = np.abs(g[n:] - rv).reshape(n, 6, 6).max(axis=(1, 2)) / np.abs(rv).reshape(n, 6, 6).max(axis=(1, 2))
    assert rel.max() < 1e-7
    t1 = 8000.0 + 3652.5
    _integrate_guarded(sim, t1, 600.0)
    assert sim.status == 0 and sim.t == t1
    steps_fwd = sim.steps_done
    sim.dt = -sim.dt
    _integrate_guarded(sim, 8000.0, 600.0)
    assert sim.status == 0 and sim.t == 8000.0
    g = _states(sim)
    dx = np.abs(g[:n, :3] - pop.state[:, :3]).max(axis=1)
    dv = np.abs(g[n:] - var0).reshape(n, 6, 6).max(axis=(1, 2))
    print("4096 NEO x 6 variational, 10 yr forward (%d steps) and back (%d): round trip |dx| median %.2e m, "
          "max %.2e m; variational |Phi(-T) Phi(T) - I| median %.2e max %.2e"
          % (steps_fwd, sim.steps_done - steps_fwd, np.median(dx) * AU_M, dx.max() * AU_M, np.median(dv), dv.max()))
    assert np.isfinite(g).all()
    assert np.median(dx) * AU_M < 1.0
    assert np.median(dv) < 1e-6
    ex.detach(sim); sim.free()
