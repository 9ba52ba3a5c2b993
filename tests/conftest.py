"""Shared fixtures.  Tests marked `gpu` need a CUDA device (GB300); everything
else runs on the CPU: the oracle against the reference's golden outputs, the
host-side logic, and that libassist_gb300.so loads and exports its C ABI."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (sm_103a)")
    if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    lib = os.path.join(ROOT, "assist_gb300", "libassist_gb300.so")
    if not os.path.exists(lib) and (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        import importlib.util
        spec = importlib.util.spec_from_file_location("assist_gb300_build", os.path.join(ROOT, "assist_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build_library()


@pytest.fixture(scope="session", params=["440", "bsp"])
def planets_format(request):
    """The golden planets as a .440 file and as an SPK file (same orbits)."""
    return request.param


@pytest.fixture(scope="session")
def golden(planets_format):
    return dict(np.load(os.path.join(GOLDEN, "golden.npz" if planets_format == "440" else "golden_spk.npz")))


@pytest.fixture(scope="session")
def golden_paths(planets_format):
    return (os.path.join(GOLDEN, "golden_planets." + planets_format),
            os.path.join(GOLDEN, "golden_asteroids.bsp"))


@pytest.fixture(scope="session")
def oracle_golden(golden_paths):
    from tests.oracle_py import Oracle
    return Oracle(*golden_paths)


@pytest.fixture(scope="session")
def synth_files(tmp_path_factory):
    """A synthetic ephemeris covering [7800, 9000] days (seed 7) and its model."""
    from assist_gb300 import synth
    d = str(tmp_path_factory.mktemp("synth"))
    pl, ast, system = synth.write_ephemeris(d, seed=7, t_beg=7800.0, t_end=9000.0)
    return pl, ast, system


@pytest.fixture(scope="session")
def synth_files_spk(synth_files, tmp_path_factory):
    """The same synthetic planets as an SPK file (with the same asteroids)."""
    from assist_gb300 import synth
    pl, ast, system = synth_files
    d = str(tmp_path_factory.mktemp("synth_spk"))
    return synth.write_planets_spk(d, system, 7, 7800.0, 9000.0), ast, system


def rel_err(a, b):
    """Per-row ||a - b|| / ||b|| (the 1e-14 acceleration criterion)."""
    a = np.asarray(a).reshape(-1, 3)
    b = np.asarray(b).reshape(-1, 3)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
