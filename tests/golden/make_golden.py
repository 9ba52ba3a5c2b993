"""Generate the golden fixtures under tests/golden/ from the ASSIST reference.

Run in a container where the ASSIST sources are present (default
/root/reference, override with ASSIST_REFERENCE):

    sh oracle/build_ref.sh && python tests/golden/make_golden.py

Writes
  golden_planets.440, golden_planets.bsp,
  golden_asteroids.bsp                      -- a small synthetic ephemeris
                                               (the same planets as a .440
                                               file and as an SPK file)
  golden.npz, golden_spk.npz                -- reference outputs on it with
                                               each planets file:
      body states, accelerations for several force configurations
      (variational particles, non-grav parameters, geocentric, EIH sources),
      and IAS15 end states with the reference's forces.
  detection.npz                             -- header samples embedded in the
      reference's own format-detection test (unit_tests/spk_detection).
The reference outputs come from the UNMODIFIED ASSIST sources compiled into
oracle/_ref/libassist_ref.so; IAS15 runs use the oracle's integrator driving
the reference's assist_additional_forces through its force callback.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from assist_gb300 import synth  # noqa: E402
from tests.oracle_py import DEFAULT_LAW, load_lib  # noqa: E402

REF = os.environ.get("ASSIST_REFERENCE", "/root/reference")
D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
L = C.POINTER(C.c_longlong)


def p(a):
    return None if a is None else a.ctypes.data_as(D)


def ref_lib():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libassist_ref.so"))
    lib.refh_ephem_create.restype = C.c_void_p
    lib.refh_ephem_create.argtypes = [C.c_char_p, C.c_char_p]
    lib.refh_get_body.argtypes = [C.c_void_p, C.c_int, C.c_double, D]
    lib.refh_ctx_create.restype = C.c_void_p
    lib.refh_ctx_create.argtypes = [C.c_void_p, C.c_int, C.c_int, I, D, C.c_int, C.c_int, C.c_int] + [C.c_double] * 5 + [C.c_int]
    lib.refh_ctx_eval.argtypes = [C.c_void_p, C.c_double, C.c_double, D, D, D]
    lib.refh_ctx_free.argtypes = [C.c_void_p]
    return lib


def detection_samples():
    src = open(os.path.join(REF, "unit_tests", "spk_detection", "problem.c")).read()
    out = {}
    for name in ("valid_bsp_sample", "ascii_bin_sample"):
        m = re.search(name + r"\[\]\s*=\s*\{(.*?)\};", src, re.S)
        vals = [int(v, 16) for v in re.findall(r"0x[0-9a-fA-F]+", m.group(1))]
        out[name] = np.array(vals, dtype=np.uint8)
    m = re.search(r'ascii_source_sample\[\]\s*=\s*"(.*?)";', src, re.S)
    out["ascii_source_sample"] = np.frombuffer(m.group(1).encode().decode("unicode_escape").encode(), dtype=np.uint8)
    return out


def main():
    pl = os.path.join(HERE, "golden_planets.440")
    plb = os.path.join(HERE, "golden_planets.bsp")
    ast = os.path.join(HERE, "golden_asteroids.bsp")
    system = synth.SolarSystem(4242)
    synth.write_ascii_ephem(pl, system, synth.JD_J2000 + 32.0 * 249, 9)        # t in [7968, 8256]
    synth.write_spk_planets(plb, system, synth.JD_J2000 + 32.0 * 249, synth.JD_J2000 + 32.0 * 258)
    synth.write_spk_asteroids(ast, system, synth.JD_J2000 + 32.0 * 248, synth.JD_J2000 + 32.0 * 259)
    R = ref_lib()
    for planets, out in ((pl, "golden.npz"), (plb, "golden_spk.npz")):
        e = R.refh_ephem_create(planets.encode(), ast.encode())
        assert e, "reference could not load the golden ephemeris " + planets
        g = reference_outputs(R, e, system)
        np.savez_compressed(os.path.join(HERE, out), **g)
        print("wrote", out, sorted(g))
    np.savez_compressed(os.path.join(HERE, "detection.npz"), **detection_samples())


def reference_outputs(R, e, system):
    """Body states, accelerations of the force cases and IAS15 end states of
    the reference on one ephemeris (planets file + asteroids file)."""
    g = {}
    # body states
    times = np.linspace(7970.0, 8250.0, 29)
    bodies = np.zeros((len(times), 27, 10))
    for k, t in enumerate(times):
        for i in range(27):
            o = np.zeros(10)
            assert R.refh_get_body(e, i, t, p(o)) == 0
            bodies[k, i] = o
    g["body_times"] = times
    g["bodies"] = bodies
    # body states at record and sub-interval edges: times a rounding below a
    # 32-day record boundary (the Julian date rounds up across it, so the
    # record fraction comes out a hair below zero), the boundaries themselves,
    # and sub-interval boundaries inside a record
    edges = np.array([8000.0 - 1e-10, 8032.0 - 2e-10, 8096.0 - 5e-11, 8160.0 - 2.2e-10, 8000.0, 8128.0,
                      8008.0 - 1e-10, 8040.0, 8128.0 + 1e-10, 8004.0 - 3e-11])
    eb = np.zeros((len(edges), 27, 10))
    for k, t in enumerate(edges):
        for i in range(27):
            o = np.zeros(10)
            assert R.refh_get_body(e, i, t, p(o)) == 0
            eb[k, i] = o
    g["edge_times"] = edges
    g["edge_bodies"] = eb
    # force cases
    rng = np.random.default_rng(77)
    mba = synth.population(system, "mba", 12, seed=11, t0=8100.0)
    neo = synth.population(system, "neo", 12, seed=12, t0=8100.0, close_frac=0.25)
    state = np.concatenate([mba.state, neo.state])
    n = state.shape[0]
    nvar = 30
    vtp = rng.integers(0, n, nvar).astype(np.int32)
    vstate = np.concatenate([rng.normal(size=(nvar, 3)), 1e-2 * rng.normal(size=(nvar, 3))], axis=1)
    params = np.zeros((n + nvar, 3))
    params[:n] = rng.choice([-1, 1], (n, 3)) * np.exp(rng.uniform(np.log(1e-12), np.log(1e-9), (n, 3)))
    params[: n // 3] = 0.0
    params[n:] = rng.integers(0, 2, (nvar, 3))
    cases = [(0x7F, 1, 0, True), (0x1FF, 11, 0, True), (0x7F, 3, 1, True), (0x01, 1, 0, True), (0x02, 1, 0, True),
             (0x04, 1, 0, True), (0x08, 1, 0, True), (0x10, 1, 0, True), (0x20, 1, 0, True), (0x40, 1, 0, True),
             (0x80, 1, 0, True), (0x100, 1, 0, True), (0x7F, 1, 0, False)]
    law = np.array(DEFAULT_LAW)
    X = np.concatenate([state[:, :3], vstate[:, :3]]).ravel().copy()
    V = np.concatenate([state[:, 3:], vstate[:, 3:]]).ravel().copy()
    acc_cases = []
    t_f = 8100.0
    for (f, gr, geo, with_p) in cases:
        prm = params.ravel().copy() if with_p else None
        ctx = R.refh_ctx_create(e, n, nvar, vtp.ctypes.data_as(I), p(prm), f, gr, geo, *law, 1)
        a = np.zeros(3 * (n + nvar))
        assert R.refh_ctx_eval(ctx, t_f, 1.0, p(X), p(V), p(a)) == 0
        R.refh_ctx_free(ctx)
        acc_cases.append(a.reshape(-1, 3))
    g["force_t"] = np.array(t_f)
    g["force_state"] = state
    g["force_var_tp"] = vtp
    g["force_var_state"] = vstate
    g["force_params"] = params
    g["force_cases"] = np.array([[c[0], c[1], c[2], int(c[3])] for c in cases], dtype=np.int64)
    g["force_acc"] = np.stack(acc_cases)
    # IAS15 end states with the reference's forces (oracle integrator driving the reference callback)
    O = load_lib()
    O.orc_integrate_cb.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int, D, C.c_double,
                                   C.c_double, C.c_double, C.c_int, L]
    cb = C.cast(R.refh_force_cb, C.c_void_p)
    integ = []
    int_state = np.concatenate([mba.state[:3], neo.state[:3]])
    for i in range(int_state.shape[0]):
        ctx = R.refh_ctx_create(e, 1, 0, None, None, 0x7F, 1, 0, *law, 1)
        buf = int_state[i].copy()
        stats = np.zeros(5, dtype=np.int64)
        r = O.orc_integrate_cb(cb, ctx, 8000.0, 8200.0, 1, 1, p(buf), 1e-9, 0.0, 0.001, 0, stats.ctypes.data_as(L))
        R.refh_ctx_free(ctx)
        assert r == 0
        integ.append(np.concatenate([buf, stats[:4].astype(float)]))
    g["int_t0"] = np.array(8000.0)
    g["int_t1"] = np.array(8200.0)
    g["int_state0"] = int_state
    g["int_end"] = np.array(integ)
    return g


if __name__ == "__main__":
    main()
