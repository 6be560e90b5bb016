"""Builds the native library and the CLI in-tree.

    python -m bbscite_gb300.build        # or __graft_entry__.build()

    python -m bbscite_gb300.build --checked   # the build with device checks

Outputs (git-ignored):
  bbscite_gb300/libbbscite_gb300.so   kernels + C ABI (sm_103a)
  bbscite_gb300/bin/bbscite           SCITE-compatible command line
  bbscite_gb300/libbbscite_gb300_checked.so   the same with BBS_CHECKED:
      device-side index checks that report BBS_ERR_DEVICE_CHECK
Translation units are compiled in parallel; nothing is rebuilt when the
object is newer than every source it depends on.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbbscite_gb300.so")
BUILD_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(PKG, "libbbscite_gb300_checked.so")
CLI = os.path.join(PKG, "bin", "bbscite")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code rounds every float operation as written (no FMA contraction),
# like the reference's scorer constants and the oracle.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off",
              "-Xcompiler", "-fvisibility=hidden", "-I" + INCLUDE,
              "-I" + CSRC]
UNITS = ["bbs_mcmc_lo.cu", "bbs_mcmc_lo_rec.cu", "bbs_mcmc_hi.cu",
         "bbs_mcmc_hi_rec.cu", "bbs_aux.cu", "bbs_api.cu",
         "bbs_batch.cu", "bbs_batch_multi.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required")


def elf_matches_host(path: str) -> bool:
    """True when `path` is an ELF file built for this machine."""
    import platform
    want = {"x86_64": 0x3E, "aarch64": 0xB7, "arm64": 0xB7}.get(
        platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    return want is None or int.from_bytes(head[18:20], "little") == want


def _deps() -> float:
    files = glob.glob(os.path.join(CSRC, "*")) + [
        os.path.join(INCLUDE, "bbscite_gb300.h"),
        os.path.join(INCLUDE, "bbscite_gb300.hpp")]
    return max(os.path.getmtime(f) for f in files)


def _compile(unit: str, newest: float, verbose: bool,
             checked: bool = False) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD_CHECKED if checked else BUILD,
                       unit.replace(".cu", ".o"))
    if (os.path.exists(obj) and os.path.getmtime(obj) >= newest
            and elf_matches_host(obj)):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *(["-DBBS_CHECKED"] if checked else []),
           "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build_checked(verbose: bool = False, jobs: int | None = None) -> str:
    """The library with device checks (BBS_CHECKED), for tests and
    debugging; the CLI is not rebuilt."""
    os.makedirs(BUILD_CHECKED, exist_ok=True)
    newest = _deps()
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    jobs = jobs or min(len(units), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda u: _compile(u, newest, verbose, True), units))
    if not elf_matches_host(LIB_CHECKED) or os.path.getmtime(LIB_CHECKED) < max(
            os.path.getmtime(o) for o in objs):
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", LIB_CHECKED, *objs,
                            "-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB_CHECKED


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    newest = _deps()
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    jobs = jobs or min(len(units), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda u: _compile(u, newest, verbose), units))
    if not elf_matches_host(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(o) for o in objs):
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs,
                            "-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    cli_src = os.path.join(CSRC, "cli", "bbscite_main.cpp")
    if os.path.exists(cli_src) and (
            not elf_matches_host(CLI) or os.path.getmtime(CLI) <
            max(os.path.getmtime(LIB), os.path.getmtime(cli_src),
                _deps())):
        r = subprocess.run(
            ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC,
             cli_src, "-o", CLI, "-L" + PKG, "-lbbscite_gb300",
             "-Wl,-rpath,$ORIGIN/.."], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    if "--checked" in sys.argv:
        print(build_checked(verbose="-v" in sys.argv))
    else:
        print(build(verbose="-v" in sys.argv))
