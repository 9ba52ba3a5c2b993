"""Edge cases of the batched entry points against the oracle: one batch mixing
forward, backward and zero-length spans (the group key separates the
directions; a zero-length span returns its initial state untouched, as
ASSIST's integrate does when t == tmax), an empty batch, and a batch whose
groups hold fewer than 32 particles (partly filled blocks)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def edge_files(tmp_path_factory):
    """A synthetic ephemeris covering [7600, 8400] days (seed 7)."""
    from assist_gb300 import synth
    d = str(tmp_path_factory.mktemp("synth_edges"))
    return synth.write_ephemeris(d, seed=7, t_beg=7600.0, t_end=8400.0)


@pytest.mark.parametrize("group_steps", [0, 1, 2])
def test_batch_mixed_directions_and_zero_spans(edge_files, group_steps):
    from assist_gb300 import Ephem, batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = edge_files
    eph = Ephem(pl, ast); O = Oracle(pl, ast)
    pop = synth.population(system, "mix", 96, seed=41, t0=8000.0, log_len=(20.0, 300.0), nongrav_frac=0.2)
    t_end = pop.t_end.copy()
    t_end[::4] = pop.t0[::4]                                          # zero-length spans
    t_end[1::4] = pop.t0[1::4] - (pop.t_end[1::4] - pop.t0[1::4])     # backward spans
    o = batch.options(group_steps=group_steps)
    out, _, status, stats = batch.integrate_batch(eph, pop.t0, t_end, pop.state, params=pop.params, opts=o)
    ref, _, rstat, _ = O.integrate_batch(pop.t0, t_end, pop.state, params=pop.params, return_all=True)
    assert np.array_equal(status, rstat)
    assert np.array_equal(out[::4], pop.state[::4])
    ok = rstat == 0
    assert ok.sum() == 96
    assert np.abs(out[ok, :3] - ref[ok, :3]).max() < 1e-9


def test_batch_empty(edge_files):
    from assist_gb300 import Ephem, batch
    pl, ast, _ = edge_files
    eph = Ephem(pl, ast)
    z = np.zeros(0)
    out, _, status, stats = batch.integrate_batch(eph, z, z, np.zeros((0, 6)))
    assert out.shape == (0, 6) and status.shape == (0,)
    assert stats["steps_accepted"] == 0


@pytest.mark.parametrize("n", [1, 5, 37])
def test_batch_partly_filled_groups(edge_files, n):
    """Batches of 1, 5 and 37 NEOs: groups of fewer than 32 members (the
    block-cooperative kernel's idle lanes) give the oracle's end states."""
    from assist_gb300 import Ephem, batch, synth
    from tests.oracle_py import Oracle
    pl, ast, system = edge_files
    eph = Ephem(pl, ast); O = Oracle(pl, ast)
    pop = synth.population(system, "neo", n, seed=43, t0=8000.0, log_len=(30.0, 300.0))
    out, _, status, _ = batch.integrate_batch(eph, pop.t0, pop.t_end, pop.state, opts=batch.options(group_steps=2))
    ref, _, rstat, _ = O.integrate_batch(pop.t0, pop.t_end, pop.state, return_all=True)
    assert np.array_equal(status, rstat)
    ok = rstat == 0
    assert np.abs(out[ok, :3] - ref[ok, :3]).max() < 1e-9
