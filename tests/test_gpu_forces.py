"""Device force model against the oracle (and the reference's golden
outputs).  Accelerations: ||a_gpu - a_ref|| <= 1e-14 ||a_ref|| per particle.
Variational accelerations a = J delta are measured against the scale of the
particle's linear map: ||da_q|| <= 1e-14 max_q' ||a_q'|| over the
variational particles of the same real particle (one delta can make J delta
cancel to far below ||J|| ||delta||)."""
import numpy as np
import pytest

from tests.conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-14


@pytest.fixture(scope="module")
def dev():
    import torch
    assert torch.cuda.is_available()
    return torch.device("cuda:0")


def _eph(paths):
    from assist_gb300 import Ephem
    return Ephem(*paths)


def test_forces_against_reference_golden(golden, golden_paths, dev):
    """Drop-in callback (shared time, arbitrary var_config) vs the reference's
    own assist_additional_forces outputs."""
    from assist_gb300 import Extras, Simulation
    eph = _eph(golden_paths)
    st = golden["force_state"]; vs = golden["force_var_state"]; tp = golden["force_var_tp"]
    n, m = st.shape[0], vs.shape[0]
    for c, ref in zip(golden["force_cases"], golden["force_acc"]):
        flags, gr, geo, with_p = (int(v) for v in c)
        sim = Simulation.create()
        ex = Extras(sim, eph)
        ex._forces = flags
        ex.gr_eih_sources = gr
        ex.geocentric = geo
        for i in range(n):
            sim.add(*st[i])
        for k in range(m):
            idx = sim.add_variation(int(tp[k]))
            p = sim.particle(idx)
            p.x, p.y, p.z, p.vx, p.vy, p.vz = vs[k]
        if with_p:
            ex.particle_params = golden["force_params"]
        sim.t = float(golden["force_t"])
        sim.update_acceleration()
        assert sim.status <= 0
        acc = np.array([[p.ax, p.ay, p.az] for p in sim.particles])
        e = rel_err(acc, ref)
        assert e[:n].max() < TOL, (hex(flags), e[:n].max())
        for j in np.unique(tp):
            q = n + np.nonzero(tp == j)[0]
            scale = np.linalg.norm(ref[q], axis=1).max()
            assert np.linalg.norm(acc[q] - ref[q], axis=1).max() <= TOL * scale, (hex(flags), "var", int(j))
        ex.detach(sim)
        sim.free()


def test_forces_each_time_vs_oracle(synth_files, dev):
    """Batched evaluation with per-particle times and 6 variational particles each."""
    import torch
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    rng = np.random.default_rng(0)
    n = 300
    pop = synth.population(system, "mix", n, seed=2, t0=8000.0, nongrav_frac=0.3, close_frac=0.02)
    tt = pop.t0 + rng.uniform(-150.0, 900.0, n)
    var = rng.normal(size=(n, 6, 6))
    for flags, gr, geo in [(0x7F, 1, 0), (0x1FF, 11, 0), (0x7F, 4, 1), (0x01, 1, 0), (0x08, 1, 0), (0x10, 1, 0),
                           (0x20, 1, 0), (0x40, 2, 0), (0x80, 1, 0), (0x100, 1, 0)]:
        o = batch.options(forces=flags, gr_eih_sources=gr, geocentric=geo)
        T = torch.tensor(tt, device=dev); S = torch.tensor(pop.state, device=dev)
        P = torch.tensor(pop.params, device=dev); V = torch.tensor(var, device=dev)
        acc, vacc = batch.forces_device(eph, T, S, params=P, var_state=V, opts=o)
        acc = acc.cpu().numpy(); vacc = vacc.cpu().numpy()
        for i in range(n):
            ref = O.forces(tt[i], pop.state[i:i + 1], params=pop.params[i:i + 1], var_state=var[i],
                           var_tp=np.zeros(6, np.int32), forces=flags, gr_eih_sources=gr, geocentric=geo)
            assert rel_err(acc[i], ref[0]).max() < TOL, (hex(flags), i, rel_err(acc[i], ref[0]))
            scale = np.linalg.norm(ref[1:], axis=1).max()
            assert np.linalg.norm(vacc[i] - ref[1:], axis=1).max() <= TOL * scale, (hex(flags), i, "var")


def test_bodies_vs_oracle(synth_files, dev):
    import torch
    from assist_gb300 import batch
    from tests.oracle_py import Oracle
    pl, ast, _ = synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    ts = np.linspace(7800.0, 9000.0, 61)
    B = batch.bodies_device(eph, torch.tensor(ts, device=dev)).cpu().numpy()
    for k, t in enumerate(ts):
        for i in range(27):
            st, ref = O.body(i, t)
            assert st == 0
            m = np.isfinite(ref)
            assert np.array_equal(np.isfinite(B[k, i]), m)
            scale = np.abs(ref[m]).max()
            assert np.abs(B[k, i, m] - ref[m]).max() <= 4e-16 * max(scale, 1.0), (t, i)


def test_edge_bodies_vs_reference_golden(golden, golden_paths, dev):
    """Bodies at record and sub-interval edges (a time a rounding below a
    record boundary: the record fraction is a hair below zero, where the
    reference's fmod keeps the record's start) against the reference."""
    import torch
    from assist_gb300 import batch
    eph = _eph(golden_paths)
    ts = golden["edge_times"]
    B = batch.bodies_device(eph, torch.tensor(ts, device=dev)).cpu().numpy()
    for k, t in enumerate(ts):
        for i in range(27):
            ref = golden["edge_bodies"][k, i]
            m = np.isfinite(ref)
            assert np.array_equal(np.isfinite(B[k, i]), m)
            scale = np.abs(ref[m]).max()
            assert np.abs(B[k, i, m] - ref[m]).max() <= 4e-16 * max(scale, 1.0), (t, i, B[k, i] - ref)


def test_get_particle_and_coverage(golden, golden_paths, dev):
    eph = _eph(golden_paths)
    p = eph.get_particle("Sun", float(golden["body_times"][3]))
    ref = golden["bodies"][3, 0]
    assert abs(p.x - ref[1]) < 1e-16 and p.m == ref[0]
    p = eph.get_particle(20, float(golden["body_times"][5]))
    assert abs(p.y - golden["bodies"][5, 20, 2]) < 1e-15
    with pytest.raises(RuntimeError, match="outside the coverage"):
        eph.get_particle(0, 9999.0)
    tb, te = eph.time_bounds()
    assert (tb, te) == (pytest.approx(7968.0), pytest.approx(8256.0))


def test_drop_in_coverage_error_sets_status(golden_paths, dev):
    from assist_gb300 import Extras, Simulation
    eph = _eph(golden_paths)
    sim = Simulation.create()
    ex = Extras(sim, eph)
    sim.add(2.5, 0.1, 0.0, 0.0, 0.01, 0.0)
    sim.t = 20000.0
    sim.update_acceleration()
    assert sim.status == 1 and b"coverage" in sim.error_message
    ex.detach(sim); sim.free()


@pytest.mark.parametrize("case", ["default", "nongrav", "geocentric", "eih3", "spk-planets", "no-asteroids",
                                  "gr-potential", "gr-simple"])
def test_shared_time_cooperative_forces_vs_oracle(synth_files, synth_files_spk, dev, case):
    """The block-cooperative evaluation the batched and shared-step kernels
    run (assist_gb300_forces_shared_time_device: four warps split each
    particle's terms, the asteroids' terms in double-float arithmetic) against
    the oracle, per particle at 1e-14, on 96 particles of the mixture plus
    particles placed 0.005 AU (the FP64 path) and 0.03 AU (the float-pair
    path) from each asteroid."""
    import torch
    from assist_gb300 import batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = synth_files_spk if case == "spk-planets" else synth_files
    eph = _eph((pl, ast)); O = Oracle(pl, ast)
    t = 8123.375
    pop = synth.population(system, "mix", 96, seed=51, t0=t, nongrav_frac=0.5 if case == "nongrav" else 0.0)
    near = []
    rng = np.random.default_rng(52)
    for m in range(16):
        a = eph.get_particle(11 + m, t)
        for dist in (0.005, 0.03):
            u = rng.normal(size=3); u /= np.linalg.norm(u)
            r = np.hypot(a.x, a.y)
            vc = 0.01720209895 / np.sqrt(r)      # circular speed (AU/day); the ephemeris has no asteroid velocities
            near.append([a.x + dist * u[0], a.y + dist * u[1], a.z + dist * u[2],
                         -vc * a.y / r + 1e-3 * u[1], vc * a.x / r - 1e-3 * u[0], 1e-3 * u[2]])
    state = np.concatenate([pop.state, np.array(near)])
    params = np.concatenate([pop.params, np.zeros((len(near), 3))])
    kw = {}
    if case == "geocentric":
        earth = eph.get_particle(3, t)
        state = state - np.array([earth.x, earth.y, earth.z, earth.vx, earth.vy, earth.vz])
        kw["geocentric"] = 1
    if case == "eih3":
        kw["gr_eih_sources"] = 3
    if case == "no-asteroids":
        kw["forces"] = 0x7F & ~0x04
    if case == "gr-potential":
        kw["forces"] = (0x7F & ~0x40) | 0x100
    if case == "gr-simple":
        kw["forces"] = (0x7F & ~0x40) | 0x80
    o = batch.options(**kw)
    st = torch.tensor(state, device=dev)
    prm = torch.tensor(params, device=dev)
    status = torch.full((state.shape[0],), -1, dtype=torch.int32, device=dev)
    acc = batch.forces_shared_time_device(eph, t, st, params=prm, status=status, opts=o).cpu().numpy()
    assert (status.cpu().numpy() == 0).all()
    ref = O.forces(t, state, params=params, **kw)
    e = rel_err(acc, ref)
    assert e.max() < TOL, (case, e.max(), int(e.argmax()))


def test_shared_time_cooperative_forces_coverage(synth_files, dev):
    import torch
    from assist_gb300 import batch
    pl, ast, _ = synth_files
    eph = _eph((pl, ast))
    st = torch.zeros((5, 6), dtype=torch.float64, device=dev)
    st[:, 0] = 2.5
    st[:, 4] = 0.01
    status = torch.zeros(5, dtype=torch.int32, device=dev)
    batch.forces_shared_time_device(eph, 20000.0, st, status=status)
    assert (status.cpu().numpy() == 5).all()
