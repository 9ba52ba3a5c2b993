"""Batched dense output: each particle's state at its own output times,
interpolated on the device from the IAS15 step that contains each time
(ASSIST's assist_integrate_or_interpolate, src/assist.c:642-680, on a whole
batch).  Checked the way the reference's onthefly_interpolation test does:
against integrating each particle to each output time directly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_dense(eph, pop, times, opts=None):
    import torch
    from assist_gb300 import batch
    dev = torch.device("cuda", 0)
    n = len(pop.t0)
    starts = np.zeros(n + 1, np.int32)
    starts[1:] = np.cumsum([len(t) for t in times])
    flat = np.concatenate(times)
    st = torch.tensor(pop.state, device=dev)
    out = torch.full((flat.size, 6), np.nan, dtype=torch.float64, device=dev)
    status = torch.zeros(n, dtype=torch.int32, device=dev)
    batch.integrate_batch_dense_device(eph, torch.tensor(pop.t0, device=dev), torch.tensor(pop.t_end, device=dev), st,
                                       torch.tensor(starts, device=dev), torch.tensor(flat, device=dev), out,
                                       params=torch.tensor(pop.params, device=dev), status=status, opts=opts)
    torch.cuda.synchronize()
    return out.cpu().numpy(), st.cpu().numpy(), status.cpu().numpy(), starts


@pytest.mark.parametrize("kind,bar", [("mba", 2e-13), ("mix", 1e-10)])
def test_dense_output_matches_direct_integration(synth_files, kind, bar):
    import torch
    from assist_gb300 import Ephem, batch, synth
    pl, ast, system = synth_files
    eph = Ephem(pl, ast)
    pop = synth.population(system, kind, 96, seed=41, t0=8000.0, length=800.0, nongrav_frac=0.1)
    rng = np.random.default_rng(5)
    # sorted, unevenly spaced output times inside each particle's span (some at its ends)
    times = []
    for i in range(len(pop.t0)):
        k = 1 + i % 7
        ts = np.sort(rng.uniform(pop.t0[i], pop.t_end[i], k))
        if i % 5 == 0:
            ts = np.concatenate([[pop.t0[i]], ts, [pop.t_end[i]]])
        times.append(ts)
    out, end, status, starts = _run_dense(eph, pop, times)
    assert (status == 0).all()
    # direct: every (particle, time) pair integrated from t0 to that time
    idx = np.repeat(np.arange(len(pop.t0)), [len(t) for t in times])
    flat = np.concatenate(times)
    dev = torch.device("cuda", 0)
    st = torch.tensor(pop.state[idx], device=dev)
    s2 = torch.zeros(idx.size, dtype=torch.int32, device=dev)
    batch.integrate_batch_device(eph, torch.tensor(pop.t0[idx], device=dev), torch.tensor(flat, device=dev), st,
                                 params=torch.tensor(pop.params[idx], device=dev), status=s2)
    torch.cuda.synchronize()
    direct = st.cpu().numpy()
    assert (s2.cpu().numpy() == 0).all()
    d = np.abs(out[:, :3] - direct[:, :3]).max(axis=1)
    assert np.isfinite(out).all()
    assert d.max() < bar, (d.max(), np.argmax(d))
    # velocities to the same relative order
    assert np.abs(out[:, 3:] - direct[:, 3:]).max() < bar * 1e-1 + 1e-15


def test_dense_output_rejects_times_outside_span(synth_files):
    import torch
    from assist_gb300 import Ephem, synth
    pl, ast, system = synth_files
    eph = Ephem(pl, ast)
    pop = synth.population(system, "mba", 4, seed=2, t0=8000.0, length=100.0)
    times = [np.array([8050.0]), np.array([8150.0]), np.array([8020.0, 8010.0]), np.array([])]
    with pytest.raises(RuntimeError, match="output time"):
        _run_dense(eph, pop, times)
