"""The oracle (CPU restatement) against outputs of the UNMODIFIED reference
sources (tests/golden/, written by tests/golden/make_golden.py).  The oracle
is built with the same evaluation order as the reference, so agreement is
bit-exact."""
import numpy as np
import pytest

from tests.oracle_py import Oracle


def test_bodies_bitwise(golden, oracle_golden):
    for k, t in enumerate(golden["body_times"]):
        for i in range(27):
            st, out = oracle_golden.body(i, t)
            assert st == 0
            ref = golden["bodies"][k, i]
            assert np.array_equal(np.isnan(out), np.isnan(ref))
            m = ~np.isnan(ref)
            assert np.array_equal(out[m], ref[m]), (t, i, out - ref)


def test_edge_bodies_bitwise(golden, oracle_golden):
    """Record and sub-interval edges: a time a rounding below a record
    boundary (its Julian date rounds up across it, the record fraction comes
    out a hair below zero), the boundaries, sub-interval boundaries."""
    for k, t in enumerate(golden["edge_times"]):
        for i in range(27):
            st, out = oracle_golden.body(i, t)
            assert st == 0
            ref = golden["edge_bodies"][k, i]
            m = ~np.isnan(ref)
            assert np.array_equal(np.isnan(out), np.isnan(ref))
            assert np.array_equal(out[m], ref[m]), (t, i, out - ref)


def test_edge_bodies_continuous(golden, oracle_golden):
    """Just below a record boundary the bodies are where they are at the
    boundary (to their motion over the gap), not a sub-interval away."""
    for t in golden["edge_times"]:
        if t == round(t) or abs(t - round(t)) > 1e-9:
            continue
        tb = float(round(t))
        for i in range(27):
            _, a = oracle_golden.body(i, t)
            _, b = oracle_golden.body(i, tb)
            assert np.abs(a[1:4] - b[1:4]).max() < 1e-11, (t, i, a[1:4] - b[1:4])


def test_forces_bitwise(golden, oracle_golden):
    st = golden["force_state"]
    n = st.shape[0]
    for c, ref in zip(golden["force_cases"], golden["force_acc"]):
        flags, gr, geo, with_p = (int(v) for v in c)
        acc = oracle_golden.forces(float(golden["force_t"]), st, params=golden["force_params"] if with_p else None,
                                   var_state=golden["force_var_state"], var_tp=golden["force_var_tp"], forces=flags,
                                   gr_eih_sources=gr, geocentric=geo)
        assert np.array_equal(acc, ref), (hex(flags), np.abs(acc - ref).max())
    assert n > 0


def test_ias15_end_states_with_reference_forces(golden, oracle_golden):
    """The oracle's IAS15 with its own forces reproduces the run that drove
    the reference's assist_additional_forces, step for step."""
    for s0, end in zip(golden["int_state0"], golden["int_end"]):
        out, _, info = oracle_golden.integrate(float(golden["int_t0"]), float(golden["int_t1"]), s0[None, :])
        assert np.array_equal(out[0], end[:6])
        assert info["accepted"] == int(end[6]) and info["evals"] == int(end[8])


def test_time_bounds(golden_paths):
    o = Oracle(*golden_paths)
    tb, te = o.time_bounds()
    assert tb == pytest.approx(7968.0) and te == pytest.approx(8256.0)


def test_coverage_error(oracle_golden):
    st, _ = oracle_golden.body(0, 9000.0)
    assert st == 5
    st, _ = oracle_golden.body(20, 7000.0)
    assert st == 5
