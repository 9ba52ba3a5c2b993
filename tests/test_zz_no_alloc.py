"""assist_gb300_integrate_batch_device_static (the batched IAS15 entry point
that allocates nothing: scratch in a fixed __device__ array) against the
allocating entry point assist_gb300_integrate_batch_device with independent
steps.  The file name sorts last so the test also runs after every other
device test in the same process."""
import ctypes

import numpy as np
import pytest


@pytest.mark.gpu
def test_static_scratch_batch_matches_allocating_entry_point(synth_files):
    torch = pytest.importorskip("torch")
    from assist_gb300 import Ephem, batch, synth
    pl, ast, system = synth_files
    eph = Ephem(pl, ast)
    pop = synth.population(system, "mix", 700, seed=21, t0=8000.0, log_len=(30.0, 400.0), nongrav_frac=0.1)
    n = len(pop.t0)
    dev = torch.device("cuda", 0)
    t0 = torch.tensor(pop.t0, device=dev)
    te = torch.tensor(pop.t_end, device=dev)
    prm = torch.tensor(pop.params, device=dev)
    ref = torch.tensor(pop.state, device=dev)
    ref_status = torch.zeros(n, dtype=torch.int32, device=dev)
    ref_stats = batch.integrate_batch_device(eph, t0, te, ref, params=prm, status=ref_status,
                                             opts=batch.options(group_steps=0))
    torch.cuda.synchronize()
    scale = ref.abs().max().item()
    for _ in range(2):                       # two calls in a row reuse the same scratch
        st = torch.tensor(pop.state, device=dev)
        status = torch.full((n,), -7, dtype=torch.int32, device=dev)
        stats = batch.integrate_batch_device_static(eph, t0, te, st, params=prm, status=status)
        torch.cuda.synchronize()
        assert torch.equal(status, ref_status)
        assert (st - ref).abs().max().item() <= 1e-15 * scale
        assert stats["steps_accepted"] == ref_stats["steps_accepted"]
        assert stats["force_evals"] == ref_stats["force_evals"]


def test_static_scratch_batch_rejects_oversized_batch():
    """More particles than the fixed scratch holds: a clear error before any
    device work (no ephemeris needed)."""
    from assist_gb300 import batch
    from assist_gb300._lib import STATIC_MAX_PARTICLES, clib, last_error
    o = batch.options()
    rc = clib.assist_gb300_integrate_batch_device_static(None, ctypes.byref(o), STATIC_MAX_PARTICLES + 1, None, None,
                                                         None, None, None, None, None)
    assert rc != 0
    assert "at most %d" % STATIC_MAX_PARTICLES in last_error()
