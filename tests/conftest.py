import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def kat():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "kat.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "ref_vectors.npz"))


@pytest.fixture(scope="session")
def native():
    """The in-tree native library (built on first use)."""
    from bbscite_gb300 import build, native as N
    build.build()
    N.lib()
    return N


@pytest.fixture(scope="session")
def probe(native):
    """tests/cpp/wrapper_probe.cpp built against the library: run(lines)
    returns (stdout lines, stderr)."""
    import subprocess
    from bbscite_gb300 import build as B
    src = os.path.join(ROOT, "tests", "cpp", "wrapper_probe.cpp")
    exe = os.path.join(B.BUILD, "wrapper_probe")
    os.makedirs(B.BUILD, exist_ok=True)
    if (not os.path.exists(exe) or not B.elf_matches_host(exe)
            or os.path.getmtime(exe) < max(
                os.path.getmtime(src), os.path.getmtime(B.LIB),
                os.path.getmtime(os.path.join(ROOT, "include",
                                              "bbscite_gb300.hpp")))):
        subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off",
                        "-I" + os.path.join(ROOT, "include"), src, "-o", exe,
                        "-L" + B.PKG, "-lbbscite_gb300",
                        "-Wl,-rpath," + B.PKG], check=True)

    def run(lines):
        r = subprocess.run([exe], input="\n".join(lines) + "\n",
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        return r.stdout.splitlines(), r.stderr
    return run


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
