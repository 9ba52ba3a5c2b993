"""The close-encounter pilot that orders the grouped kernels' queue: a
particle sharing Jupiter's orbit a few hundredths of an AU from it gets a
large encounter ratio, orbits far from every planet get none, and a batch
integrates to the same end states whatever order its groups are taken in."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _states(eph, t0):
    jup = eph.get_particle("Jupiter", t0)
    sun = eph.get_particle("Sun", t0)
    gm = 2.9591220828411951e-04
    rows = []
    # 1: Jupiter's state moved 0.05 AU outward along its heliocentric radius
    hx = np.array([jup.x - sun.x, jup.y - sun.y, jup.z - sun.z])
    u = hx / np.linalg.norm(hx)
    rows.append([jup.x + 0.05 * u[0], jup.y + 0.05 * u[1], jup.z + 0.05 * u[2], jup.vx, jup.vy, jup.vz])
    # 2, 3: circular ecliptic orbits at 2.6 AU and 40 AU on the far side of the Sun from Jupiter
    for r in (2.6, 40.0):
        ang = np.arctan2(-u[1], -u[0])
        v = np.sqrt(gm / r)
        rows.append([sun.x + r * np.cos(ang), sun.y + r * np.sin(ang), sun.z,
                     sun.vx - v * np.sin(ang), sun.vy + v * np.cos(ang), sun.vz])
    return np.array(rows)


def test_encounter_ratio(synth_files):
    import torch
    from assist_gb300 import Ephem, batch
    pl, ast, _ = synth_files
    eph = Ephem(pl, ast)
    t0 = 8000.0
    st = _states(eph, t0)
    dev = torch.device("cuda", 0)
    n = st.shape[0]
    t = torch.full((n,), t0, dtype=torch.float64, device=dev)
    te = torch.full((n,), t0 + 365.25, dtype=torch.float64, device=dev)
    r = batch.encounter_ratio_device(eph, t, te, torch.tensor(st, device=dev)).cpu().numpy()
    assert r[0] > 1.0, r          # deep inside Jupiter's sphere of influence all year
    assert r[1] < 1e-3 and r[2] < 1e-3, r
    # backward integrations and zero-length intervals are accepted
    st_end = _states(eph, t0 + 365.25)
    r2 = batch.encounter_ratio_device(eph, te, t, torch.tensor(st_end, device=dev)).cpu().numpy()
    assert np.all(np.isfinite(r2)) and r2[0] > 1.0 and r2[1] < 1e-3, r2
    r3 = batch.encounter_ratio_device(eph, t, t, torch.tensor(st, device=dev)).cpu().numpy()
    assert np.all(r3 == 0.0)


def test_queue_order_does_not_change_results(synth_files):
    """Groups integrate independently: the same batch with its particles in
    reversed input order (other group boundaries, other queue positions)
    gives each particle's end state within the grouped bar, and the groups of
    a repeated call are bit-identical."""
    from assist_gb300 import Ephem, batch, synth
    pl, ast, system = synth_files
    eph = Ephem(pl, ast)
    pop = synth.population(system, "mix", 2048, seed=11, t0=8000.0, log_len=(30.0, 400.0), nongrav_frac=0.1)
    o = batch.options(group_steps=2)
    a, _, sa, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, params=pop.params, opts=o)
    b, _, sb, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, params=pop.params, opts=o)
    assert np.array_equal(a, b) and np.array_equal(sa, sb)
    rev = np.arange(pop.state.shape[0])[::-1]
    c, _, sc, _ = batch.integrate_batch(eph, pop.t0[rev], pop.t_end[rev], pop.state[rev], params=pop.params[rev],
                                        opts=o)
    c, sc = c[rev], sc[rev]
    ok = (sa == 0) & (sc == 0)
    assert ok.mean() > 0.99
    assert np.abs(a[ok, :3] - c[ok, :3]).max() < 1e-9


def test_batch_rejects_non_finite_times(synth_files):
    """A NaN or infinite start or end time is an argument error, not a
    particle status (the grouping sorts by time)."""
    from assist_gb300 import Ephem, batch, synth
    pl, ast, system = synth_files
    eph = Ephem(pl, ast)
    pop = synth.population(system, "mix", 64, seed=3, t0=8000.0, length=30.0)
    for bad in (np.nan, np.inf):
        te = pop.t_end.copy(); te[5] = bad
        with pytest.raises(RuntimeError):
            batch.integrate_batch(eph, pop.t0, te, pop.state, opts=batch.options(group_steps=2))
