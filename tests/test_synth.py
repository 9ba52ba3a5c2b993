"""The synthetic ephemeris files: layout of the reference's readers and
Chebyshev fits that reproduce the Keplerian model."""
import struct

import numpy as np

from assist_gb300 import synth
from tests.oracle_py import Oracle


def test_record_layout(synth_files):
    pl, _, _ = synth_files
    b = open(pl, "rb").read()
    beg, end, inc, num = struct.unpack("<dddi", b[0xA5C:0xA5C + 28])
    assert inc == 32.0 and num >= 400
    rec = 2 + sum(ncf * niv * ncm for ncf, niv, ncm in synth.LAYOUT)
    assert rec == 1018 and len(b) % (8 * rec) == 0
    assert b[0xFC:0xFC + 6] == b"DENUM "


def test_fits_reproduce_model(synth_files):
    pl, ast, system = synth_files
    o = Oracle(pl, ast)
    worst = 0.0
    for t in np.linspace(7850.0, 8950.0, 23):
        for i in range(27):
            st, out = o.body(i, t)
            assert st == 0
            pos, _ = system.body(i, np.array(t))
            worst = max(worst, np.abs(out[1:4] - pos).max())
    assert worst < 2e-13      # AU; the 10-coefficient Venus column is the limit


def test_populations():
    system = synth.SolarSystem(1)
    pop = synth.population(system, "mix", 1000, seed=2, t0=8000.0, nongrav_frac=0.1, close_frac=0.01)
    assert pop.state.shape == (1000, 6)
    assert (pop.t_end - pop.t0 >= 30.0 - 1e-9).all() and (pop.t_end - pop.t0 <= 3652.5 + 1e-9).all()
    assert (np.abs(pop.params[:, :2]).max(axis=1) > 0).sum() == 100 and (pop.params[:, 2] == 0).all()
    assert (pop.kind == "close").sum() == 10
