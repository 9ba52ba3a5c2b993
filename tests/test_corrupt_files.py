"""Truncated and corrupt ephemeris files are refused on the host, before any
device work (no GPU needed): the planets file gives ASSIST_ERROR_EPHEM_FILE
from assist_ephem_init, a bad asteroid file leaves the ephemeris without
asteroids (ASSIST's warning), as for the reference's own rejection test
(unit_tests/ascii_reject: an ASCII source file is neither a .440 file nor an
SPK file).  ASSIST itself maps such files and reads past their ends; this
library checks every offset against the file size."""
import ctypes
import os
import struct

import pytest

from assist_gb300 import Ephem, clib
from tests.conftest import GOLDEN

PL440 = os.path.join(GOLDEN, "golden_planets.440")
PLBSP = os.path.join(GOLDEN, "golden_planets.bsp")
AST = os.path.join(GOLDEN, "golden_asteroids.bsp")
ASCII_SOURCE = b"JPL EPHEMERIS ASCII SOURCE\n...\n"


def _write(tmp_path, name, data):
    p = tmp_path / name
    p.write_bytes(data)
    return str(p)


def _n_bodies(e):
    return clib.assist_gb300_n_bodies(ctypes.byref(e))


def test_valid_files_load_without_a_device():
    e = Ephem(PL440, AST)
    assert _n_bodies(e) == 27
    tb, te = e.time_bounds()
    assert (tb, te) == (pytest.approx(7968.0), pytest.approx(8256.0))
    e = Ephem(PLBSP, AST)
    assert _n_bodies(e) == 27


@pytest.mark.parametrize("cut", [0, 64, 0x0A5C, 0x0B28 + 20, 8144, 2 * 8144 - 8])
def test_truncated_440_refused(tmp_path, cut):
    data = open(PL440, "rb").read()[:cut]
    p = _write(tmp_path, "cut.440", data)
    with pytest.raises(RuntimeError, match="planet ephemeris file"):
        Ephem(p, AST)


def _patched_440(field_offset, fmt, value):
    data = bytearray(open(PL440, "rb").read())
    struct.pack_into(fmt, data, field_offset, value)
    return bytes(data)


@pytest.mark.parametrize("what,off,fmt,val", [
    ("record length zero", 0x0A5C + 16, "<d", 0.0),                  # days per record
    ("negative constant count", 0x0A5C + 24, "<i", -1),
    ("absurd constant count", 0x0A5C + 24, "<i", 10 ** 7),
    ("coefficient count too large", 0x0A5C + 44 + 4, "<i", 99),      # Mercury's coefficients per component
    ("negative sub-interval count", 0x0A5C + 44 + 8, "<i", -3),
    ("column past the record", 0x0A5C + 44, "<i", 100000),           # Mercury's offset
])
def test_corrupt_440_header_refused(tmp_path, what, off, fmt, val):
    p = _write(tmp_path, "bad.440", _patched_440(off, fmt, val))
    with pytest.raises(RuntimeError, match="planet ephemeris file"):
        Ephem(p, AST)


def test_440_truncated_inside_its_data_loads_with_fewer_records(tmp_path):
    """A file cut after a few whole records still loads (its header keeps the
    full coverage, the missing records give coverage errors on the device)."""
    data = open(PL440, "rb").read()
    p = _write(tmp_path, "short.440", data[:6 * 8144])
    e = Ephem(p, AST)
    assert _n_bodies(e) == 27


def test_ascii_source_refused_as_planets(tmp_path):
    p = _write(tmp_path, "source.txt", ASCII_SOURCE)
    with pytest.raises(RuntimeError, match="planet ephemeris file"):
        Ephem(p, AST)


@pytest.mark.parametrize("kind", ["ascii-source", "cut-1000", "cut-half", "bad-nd", "summary-past-end"])
def test_bad_asteroid_file_leaves_no_asteroids(tmp_path, capfd, kind):
    data = bytearray(open(AST, "rb").read())
    if kind == "ascii-source":
        data = bytearray(ASCII_SOURCE)
    elif kind == "cut-1000":
        data = data[:1000]
    elif kind == "cut-half":
        data = data[:len(data) // 2]
    elif kind == "bad-nd":
        struct.pack_into("<i", data, 8, 7)
    elif kind == "summary-past-end":
        fward = struct.unpack_from("<i", data, 76)[0]
        so = (fward - 1) * 1024 + 24
        struct.pack_into("<i", data, so + 36, len(data) // 8 + 1000)   # first segment's end address
    p = _write(tmp_path, "bad.bsp", bytes(data))
    e = Ephem(PL440, p)
    assert _n_bodies(e) == 11
    assert "asteroid" in capfd.readouterr().err.lower()


@pytest.mark.parametrize("cut", [0, 1000, 3000])
def test_truncated_planets_spk_refused(tmp_path, cut):
    p = _write(tmp_path, "cut.bsp", open(PLBSP, "rb").read()[:cut])
    with pytest.raises(RuntimeError, match="planet ephemeris file"):
        Ephem(p, AST)
