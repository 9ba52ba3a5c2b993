"""The C ABI: libassist_gb300.so loads and exports every symbol that
include/*.h declares; host-only entry points (format detection, discovery,
error strings) behave as ASSIST's (src/assist.c:52-154) without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT


def declared_symbols():
    funcs, data = set(), set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if not name.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", name)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        txt = re.sub(r"#[^\n]*", "", txt)
        txt = txt.replace('extern "C" {', "")
        txt = re.sub(r"(?m)^\s*\}\s*$", "", txt)          # the closing brace of extern "C"
        while True:
            t2 = re.sub(r"\{[^{}]*\}", "", txt)
            if t2 == txt:
                break
            txt = t2
        for stmt in txt.split(";"):
            s = " ".join(stmt.split())
            if not s or s.startswith("typedef") or s.startswith("struct") and "(" not in s:
                continue
            if s.startswith("extern") and "(" not in s:
                data.add(re.findall(r"(\w+)(?:\[\])?\s*$", s)[0])
                continue
            m = re.search(r"\b(\w+)\s*\(", s)
            if m and "(*" not in s[: m.end() + 2]:
                funcs.add(m.group(1))
    funcs.discard("extern")
    return funcs, data


@pytest.fixture(scope="module")
def lib():
    from assist_gb300 import clib
    return clib


def test_exports_every_declared_symbol(lib):
    funcs, data = declared_symbols()
    assert len(funcs) >= 37
    missing = [f for f in sorted(funcs) if not hasattr(lib, f)]
    assert not missing, missing
    for d in data:
        assert ctypes.c_void_p.in_dll(lib, d) is not None


def test_error_messages(lib):
    from assist_gb300 import assist_error_messages
    assert assist_error_messages(0) == "No error has occured."
    assert assist_error_messages(5) == "The requested time is outside the coverage provided by the ephemeris file."
    with pytest.raises(RuntimeError):
        assist_error_messages(6)


def _detect(lib, data: bytes, tmp_path):
    p = tmp_path / "f.bin"
    p.write_bytes(data)
    fd = os.open(str(p), os.O_RDONLY)
    try:
        return lib.assist_detect_ephemeris_file_format(fd)
    finally:
        os.close(fd)


def test_format_detection_on_reference_samples(lib, tmp_path):
    s = np.load(os.path.join(GOLDEN, "detection.npz"))
    assert _detect(lib, s["valid_bsp_sample"].tobytes(), tmp_path) == 0          # FILE_FORMAT_VALID_BSP
    assert _detect(lib, s["ascii_bin_sample"].tobytes(), tmp_path) == 2          # FILE_FORMAT_ASCII_BIN
    assert _detect(lib, s["ascii_source_sample"].tobytes(), tmp_path) == 3       # FILE_FORMAT_UNKNOWN
    assert _detect(lib, b"", tmp_path) == 3


def test_format_detection_on_golden_files(lib):
    for name, fmt in (("golden_planets.440", 2), ("golden_asteroids.bsp", 0)):
        fd = os.open(os.path.join(GOLDEN, name), os.O_RDONLY)
        assert lib.assist_detect_ephemeris_file_format(fd) == fmt
        os.close(fd)


def test_discovery_order(lib, tmp_path):
    buf = ctypes.create_string_buffer(1024)
    assert lib.assist_discover_planets_path(buf, 1024, str(tmp_path).encode()) == 0
    (tmp_path / "data").mkdir()
    (tmp_path / "data" / "linux_p1550p2650.440").write_bytes(b"x")
    assert lib.assist_discover_planets_path(buf, 1024, str(tmp_path).encode()) == 1
    assert buf.value.decode().endswith("/data/linux_p1550p2650.440")
    (tmp_path / "data" / "de440.bsp").write_bytes(b"x")
    assert lib.assist_discover_planets_path(buf, 1024, str(tmp_path).encode()) == 1
    assert buf.value.decode().endswith("/data/de440.bsp")


def test_struct_layouts_match_reference_ctypes_mirrors():
    """Field order/types of the ASSIST ctypes mirrors (assist/ephem.py:95-120,
    assist/extras.py:84-101): offsets of the mirrored structs."""
    from assist_gb300 import Ephem, Extras, Particle
    assert ctypes.sizeof(Particle) == 128
    assert Ephem.AU.offset == 96   # jd_ref, 3 pointers, int (+pad), fn pointer, 11 ints, int
    assert Extras.alpha.offset > Extras.gr_eih_sources.offset
