"""What any IAS15 warm start can gain, measured on the oracle (no GPU).

Every accepted step of a one-year integration of the 40/30/20/10 mixture is
replayed from its own start with the predictor's b replaced by the step's
converged b times (1 + e u), u uniform in [-1, 1] per coefficient.  The
corrector's iterations per step then bound what a predictor of accuracy e
can save: with the exact start the corrector stops after one iteration (8
force evaluations a step against about 20 with the plain predictor, a
2.5x ceiling), but the start has to be good to about 1e-9 of b to save
much, and a start off by 1e-6 is no better than the plain predictor.  In a
group that shares its steps the corrector runs until every member has
converged, which raises the bar further.  A network with BF16 weights and
FP32 arithmetic predicts b's step-to-step correction to about its own size,
many orders of magnitude short of this."""
import numpy as np

from tests.oracle_py import Oracle


def _mean_it(row):
    return float((row * np.arange(row.size)).sum() / max(row.sum(), 1))


def test_warm_start_ceiling(tmp_path):
    from assist_gb300 import synth
    pl, ast, system = synth.write_ephemeris(str(tmp_path), seed=20240611, t_beg=7960.0, t_end=8400.0)
    pop = synth.population(system, "mix", 512, seed=12345, t0=8000.0, length=365.25)
    o = Oracle(pl, ast)
    errs = [0.0, 1e-12, 1e-9, 1e-6, 1e-3]
    rows = {}
    for group in (1, 32):
        h = o.warm_start_study(pop.t0, pop.t_end, pop.state, errs, group=group)
        it = [_mean_it(r) for r in h]
        rows[group] = it
        print("group %2d: plain %.3f it/step (%.1f evaluations); start error " % (group, it[0], 1 + 7 * it[0]) +
              ", ".join("%.0e: %.3f" % (e, v) for e, v in zip(errs, it[1:])))
        assert h[0].sum() > 1000 // group
        assert it[1] < 1.05                      # exact start: one iteration
        assert it[2] < 1.1                       # 1e-12: still one
        assert it[4] > 0.9 * it[0]               # 1e-6: no better than plain
        assert it[5] > it[0]                     # 1e-3: worse than plain
    assert rows[32][3] > rows[1][3]              # shared steps need every member converged
