"""The build with device checks (BBS_CHECKED, libbbscite_gb300_checked.so).

Device-side index checks stand in for a memory checker: the nodes of every
realised move, work-list entries and dataset numbers are tested on the GPU,
and a failure comes back as BBS_ERR_DEVICE_CHECK instead of a stray access.
Here the recorder is shown to work (a check that fails on purpose, with no
access at the bad index), and the parity, learned-move and checkpoint
suites run again against the checked library in a subprocess
(BBSCITE_GB300_LIB), where every run must pass every check and give the
results the tests expect.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SELFTEST = """
import ctypes as C
from bbscite_gb300 import native as N
e, code, value, limit = C.c_int(), C.c_uint32(), C.c_uint32(), C.c_uint32()
N.check(N.lib().bbs_device_check_selftest(C.byref(e), C.byref(code),
                                          C.byref(value), C.byref(limit)))
print(N.LIB_PATH, e.value, code.value, value.value, limit.value)
"""


@pytest.fixture(scope="module")
def checked_lib(native):
    from bbscite_gb300 import build as B
    return B.build_checked()


def run_with(lib, args, timeout):
    env = dict(os.environ, BBSCITE_GB300_LIB=lib)
    return subprocess.run([sys.executable, *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=timeout)


def test_selftest_records_one_failed_check(native, checked_lib):
    import ctypes as C
    e, code, value, limit = C.c_int(), C.c_uint32(), C.c_uint32(), C.c_uint32()
    native.check(native.lib().bbs_device_check_selftest(
        C.byref(e), C.byref(code), C.byref(value), C.byref(limit)))
    assert (e.value, code.value) == (0, 0)  # the normal build checks nothing
    r = run_with(checked_lib, ["-c", SELFTEST], 300)
    assert r.returncode == 0, r.stderr
    path, enabled, code, value, limit = r.stdout.split()
    assert path == checked_lib
    assert (enabled, code, value, limit) == ("1", "4", "7", "5")


def test_suites_pass_under_device_checks(checked_lib):
    r = run_with(checked_lib,
                 ["-m", "pytest", "-q", "-x", "-m", "gpu", "-p",
                  "no:cacheprovider", "tests/test_gpu_parity.py",
                  "tests/test_gpu_learned.py", "tests/test_gpu_checkpoint.py"],
                 1500)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    import re
    passed = re.search(r"(\d+) passed", r.stdout)
    assert passed and int(passed.group(1)) >= 75, r.stdout[-2000:]
