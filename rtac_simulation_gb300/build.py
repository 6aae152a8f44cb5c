"""Build recipe for librtacx.so (sm_103a) and the C++ host-mirror demo.

Compiles every translation unit of ``csrc/`` in parallel with nvcc for
``sm_103a`` only and links them into ``rtac_simulation_gb300/librtacx.so``
(in-tree, git-ignored). ``python -m rtac_simulation_gb300.build`` runs it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "librtacx.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math",
              "-I", str(ROOT / "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
             "-I", str(ROOT / "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def build_library(verbose: bool = False, ptxas_info: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    srcs = sources()
    jobs = []
    for src in srcs:
        obj = OBJ / (src.name + ".o")
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
        else:
            cmd = ["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
        jobs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_run, cmd) for cmd, _ in jobs]
        for f in futs:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in jobs]])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


DEMO_SRC = ROOT / "tests" / "cpp" / "sensor_instance_demo.cpp"
DEMO_BIN = OBJ / "sensor_instance_demo"


def build_demo(verbose: bool = False) -> Path:
    """C++ program written against include/rtacx/simulation.hpp (the host
    mirror of the reference's SensorInstance API), linked to librtacx.so."""
    cuda = Path(_nvcc()).resolve().parent.parent
    OBJ.mkdir(exist_ok=True)
    _run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), "-I", str(cuda / "include"), str(DEMO_SRC),
          "-L", str(PKG), "-lrtacx", f"-Wl,-rpath,{PKG}", "-L", str(cuda / "lib64"), "-lcudart",
          f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(DEMO_BIN)])
    if verbose:
        print(f"built {DEMO_BIN}")
    return DEMO_BIN


BINDING_SRC = ROOT / "tests" / "cpp" / "binding" / "run_ping.cpp"
BINDING_BIN = OBJ / "binding_run_ping"


def build_binding(verbose: bool = False) -> Path:
    """The reference-side binding statements (tests/cpp/binding) in a
    stand-in of the reference's SensorInstance2D, linked to librtacx.so."""
    cuda = Path(_nvcc()).resolve().parent.parent
    OBJ.mkdir(exist_ok=True)
    _run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), "-I", str(cuda / "include"), str(BINDING_SRC),
          "-L", str(PKG), "-lrtacx", f"-Wl,-rpath,{PKG}", "-L", str(cuda / "lib64"), "-lcudart",
          f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(BINDING_BIN)])
    if verbose:
        print(f"built {BINDING_BIN}")
    return BINDING_BIN


if __name__ == "__main__":
    build_library(verbose=True, ptxas_info="--ptxas" in sys.argv)
    build_demo(verbose=True)
    build_binding(verbose=True)
