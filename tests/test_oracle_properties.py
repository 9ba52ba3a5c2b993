"""Size-independent properties of the oracle's IAS15 (the end-state checker):
round trips, variational equations against finite differences (the
reference's unit_tests/variational_* criterion), double-double agreement, and
the Gauss-Radau constants against the generated device header."""
import os
import re

import numpy as np

from assist_gb300 import synth
from tests.conftest import ROOT
from tests.oracle_py import Oracle

AU_M = 149597870700.0


def test_roundtrip(synth_files):
    pl, ast, system = synth_files
    o = Oracle(pl, ast)
    pop = synth.population(system, "mba", 3, seed=5, t0=8000.0)
    fwd, _, info = o.integrate(8000.0, 8300.0, pop.state)
    back, _, _ = o.integrate(8300.0, 8000.0, fwd, dt0=info["dt"])
    assert np.abs(back[:, :3] - pop.state[:, :3]).max() * AU_M < 1e-3      # < 1 mm


def test_variational_vs_finite_difference(synth_files):
    pl, ast, system = synth_files
    o = Oracle(pl, ast)
    p0 = synth.population(system, "mba", 1, seed=6, t0=8000.0).state[0]
    dx = 10.0 / AU_M
    p1 = p0.copy(); p1[0] += dx
    var = np.array([[1.0, 0, 0, 0, 0, 0]])
    for t1 in (8001.0, 8100.0):
        real, v, _ = o.integrate(8000.0, t1, np.stack([p0, p1]), var_state=var, var_tp=np.array([0], np.int32))
        d1 = real[1, 0] - real[0, 0]
        d2 = v[0, 0] * dx
        assert abs((d1 - d2) / d1) < 1e-5


def test_double_double_agreement(synth_files):
    pl, ast, system = synth_files
    o = Oracle(pl, ast)
    pop = synth.population(system, "neo", 2, seed=8, t0=8000.0)
    a, _, _ = o.integrate(8000.0, 8200.0, pop.state)
    b, _, _ = o.integrate(8000.0, 8200.0, pop.state, dd=True)
    assert np.abs(a[:, :3] - b[:, :3]).max() < 1e-12


def test_gauss_radau_constants_match_device_header():
    o = Oracle.__new__(Oracle)
    from tests.oracle_py import load_lib
    lib = load_lib()
    h = np.zeros(8); c = np.zeros(49); d = np.zeros(49)
    lib.orc_ias15_constants(h.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double)),
                            c.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double)),
                            d.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double)))
    txt = open(os.path.join(ROOT, "assist_gb300", "csrc", "ias15_constants.h")).read()
    def arr(name):
        m = re.search(r"#define %s \{(.*?)\}" % name, txt)
        return np.array([float(v) for v in m.group(1).split(",")])
    assert np.array_equal(arr("IAS15_H_INIT"), h)
    cc = arr("IAS15_C_INIT")
    q = 0
    for j in range(1, 7):
        for k in range(j):
            assert abs(cc[q] - c[7 * j + k]) <= 4e-16 * max(1, abs(cc[q]))
            q += 1
    dd = arr("IAS15_D_INIT")
    q = 0
    for j in range(6):
        for k in range(j + 1, 7):
            assert abs(dd[q] - d[7 * j + k]) <= 4e-16 * max(1, abs(dd[q]))
            q += 1
