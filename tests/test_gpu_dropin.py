"""The drop-in simulation path (assist_attach + reb_simulation_integrate +
assist_integrate_or_interpolate) on the reference's own invariants, re-run
on the synthetic ephemeris: on-the-fly interpolation against direct
integration (unit_tests/onthefly_interpolation,
onthefly_backwards_interpolation: < 2e-13 AU), the fixed-step round trip
(unit_tests/roundtrip_*: epsilon = 0, dt = 10 days), and the two planets
formats agreeing (unit_tests/apophis_drift, test_compare_constants_masses)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

def _sim(eph, state, t0):
    from assist_gb300 import Extras, Simulation
    sim = Simulation.create()
    ex = Extras(sim, eph)
    sim.t = t0
    sim.add(*state)
    return sim, ex


@pytest.mark.parametrize("direction", [1.0, -1.0])
def test_onthefly_interpolation_matches_direct_integration(synth_files, direction):
    from assist_gb300 import Ephem, synth
    pl, ast, system = synth_files
    eph = Ephem(pl, ast)
    # the reference's spacings: 40 days forward, 10 days backward
    t0 = 8000.0 if direction > 0 else 8700.0
    state = synth.population(system, "mba", 1, seed=4, t0=t0).state[0]
    ts = [t0 + direction * (40.0 if direction > 0 else 10.0) * (i + 1) for i in range(20)]
    s1, e1 = _sim(eph, state, t0)
    direct = []
    for t in ts:
        s1.integrate(t)
        direct.append(s1.particle(0).x)
    s2, e2 = _sim(eph, state, t0)
    interp = []
    for t in ts:
        e2.integrate_or_interpolate(t)
        interp.append(s2.particle(0).x)
    assert s1.status == 0 and s2.status == 0
    assert np.abs(np.array(direct) - np.array(interp)).max() < 2e-13
    e1.detach(s1); s1.free(); e2.detach(s2); s2.free()


def test_fixed_step_roundtrip(synth_files):
    from assist_gb300 import Ephem, synth
    pl, ast, system = synth_files
    eph = Ephem(pl, ast)
    state = synth.population(system, "mba", 1, seed=8, t0=8000.0).state[0]
    sim, ex = _sim(eph, state, 8000.0)
    sim.ri_ias15.epsilon = 0.0
    sim.dt = 10.0
    sim.integrate(8500.0)
    assert abs(sim.t - 8500.0) < 1e-9
    sim.dt = -10.0
    sim.integrate(8000.0)
    p = sim.particle(0)
    back = np.array([p.x, p.y, p.z])
    # the reference's bar for the fixed-step round trip is 0.1 m
    assert np.abs(back - np.array(state[:3])).max() * 1.495978707e11 < 0.1
    ex.detach(sim); sim.free()


def test_planets_formats_agree(synth_files, synth_files_spk):
    """Constants and GMs of the .440 and the SPK planets file are equal; the
    bodies agree to the fits; an integration differs only by the fits."""
    from assist_gb300 import Ephem, synth
    pl, ast, system = synth_files
    pb, _, _ = synth_files_spk
    ea, eb = Ephem(pl, ast), Ephem(pb, ast)
    for k in ("AU", "EMRAT", "J2E", "J3E", "J4E", "J2SUN", "RE", "CLIGHT", "ASUN", "Re_eq", "Rs_eq", "over_c_squared"):
        assert getattr(ea, k) == pytest.approx(getattr(eb, k), rel=1e-15), k
    for i in range(27):
        pa, pb_ = ea.get_particle(i, 8123.4), eb.get_particle(i, 8123.4)
        assert pa.m == pytest.approx(pb_.m, rel=1e-14), i
        assert max(abs(pa.x - pb_.x), abs(pa.y - pb_.y), abs(pa.z - pb_.z)) < 1e-13, i
    state = synth.population(system, "neo", 1, seed=6, t0=8000.0).state[0]
    sa, xa = _sim(ea, state, 8000.0)
    sb, xb = _sim(eb, state, 8000.0)
    sa.integrate(8365.0); sb.integrate(8365.0)
    d = max(abs(sa.particle(0).x - sb.particle(0).x), abs(sa.particle(0).y - sb.particle(0).y),
            abs(sa.particle(0).z - sb.particle(0).z))
    assert 0.0 <= d < 1e-10
    xa.detach(sa); sa.free(); xb.detach(sb); sb.free()
