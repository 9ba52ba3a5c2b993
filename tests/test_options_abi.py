"""The ctypes mirror of struct assist_gb300_options has the C layout: the
library's defaults land in the expected fields and the C side writes nothing
past the mirror's end (no GPU needed)."""
import ctypes

from assist_gb300 import batch
from assist_gb300._lib import Options, clib


def test_default_options_fill_the_mirror_exactly():
    n = ctypes.sizeof(Options)
    buf = (ctypes.c_ubyte * (n + 64))(*([0xAB] * (n + 64)))
    clib.assist_gb300_default_options(ctypes.cast(buf, ctypes.POINTER(Options)))
    assert all(b == 0xAB for b in bytes(buf)[n:]), "the C struct is larger than its ctypes mirror"
    o = Options.from_buffer(buf)
    assert o.forces == 0x7F and o.gr_eih_sources == 1 and o.geocentric == 0
    assert (o.alpha, o.nk, o.nm, o.nn, o.r0) == (1.0, 0.0, 2.0, 5.093, 1.0)
    assert o.epsilon == 1e-9 and o.min_dt == 0.0 and o.dt0 == 0.001 and o.max_steps == 1000000
    assert o.warm_start == 0 and o.threads_per_block == 0 and o.group_steps == 2
    assert o.dt_floor == 1e-8 and o.group_order == 0 and o.blocks_per_sm == 0 and o.ephem_staging == 0


def test_options_keywords():
    o = batch.options(blocks_per_sm=3, group_order=1, epsilon=1e-10)
    assert o.blocks_per_sm == 3 and o.group_order == 1 and o.epsilon == 1e-10
    try:
        batch.options(no_such_option=1)
    except AttributeError:
        pass
    else:
        raise AssertionError("unknown option accepted")


def test_batch_stats_mirror_size():
    """An empty batch only zeroes the stats: the C side writes exactly the
    mirror's bytes."""
    from assist_gb300._lib import BatchStats
    n = ctypes.sizeof(BatchStats)
    buf = (ctypes.c_ubyte * (n + 64))(*([0xAB] * (n + 64)))
    o = batch.options()
    rc = clib.assist_gb300_integrate_batch(None, ctypes.byref(o), 0, None, None, None, None, 0, None, None,
                                           ctypes.cast(buf, ctypes.POINTER(BatchStats)))
    assert rc == 0
    assert all(b == 0 for b in bytes(buf)[:n])
    assert all(b == 0xAB for b in bytes(buf)[n:]), "the C stats struct is larger than its ctypes mirror"
