"""Builds the native parts in-tree.

  beam_gb300/libbeam_gb300.so  CUDA kernels (sm_103a) + host runtime + C ABI
  beam_gb300/bin/beam          the command-line front end
  oracle/bin/*                 the C oracle (test infrastructure)
  oracle/_ref/beam_ref         the reference program, only where its sources exist
                               (BEAM_REFERENCE_DIR, else a `reference` checkout
                               beside this repository)

Translation units compile in parallel; objects are reused when newer than
their sources and headers.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "beam_gb300"
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libbeam_gb300.so"
CLI = PKG / "bin" / "beam"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def reference_dir() -> Path:
    """Where the reference's sources are looked for (they need not exist)."""
    env = os.environ.get("BEAM_REFERENCE_DIR")
    return Path(env) if env else ROOT.parent / "reference"


CU_SOURCES = ["divide.cu", "merge.cu", "engine.cu", "noalloc.cu", "ranker.cu", "partition_cost.cu", "encode_gpu.cu",
              "legacy_scoring.cu"]
CPP_SOURCES = ["graph.cpp", "encode.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir() -> Path:
    nvcc = Path(_nvcc()).resolve()
    root = nvcc.parent.parent
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (root / sub / "libcudart.so").exists() or (root / sub / "libcudart_static.a").exists():
            return root / sub
    return root / "lib64"


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def build_library(jobs: int = 8, verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    (PKG / "bin").mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h*"))
    nvcc = _nvcc()
    tasks = []
    objects = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objects.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            tasks.append([nvcc, "-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
                          "-I", str(ROOT / "include"), "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        objects.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            tasks.append(["g++", "-std=c++17", "-O3", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall",
                          "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=jobs) as pool:
        list(pool.map(_run, tasks))
    if tasks or not LIB.exists():
        _run([nvcc, "-shared", ARCH, "-o", str(LIB)] + [str(o) for o in objects] + ["-lcudart"])
    cli_obj = BUILD / "cli.cpp.o"
    if _stale(cli_obj, [CSRC / "cli.cpp"] + headers):
        _run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), "-I", "/usr/local/cuda/include",
              "-c", str(CSRC / "cli.cpp"), "-o", str(cli_obj)])
    if _stale(CLI, [cli_obj, LIB]):
        _run(["g++", "-o", str(CLI), str(cli_obj), f"-L{PKG}", "-lbeam_gb300", "-Wl,-rpath,$ORIGIN/..",
              f"-L{_cuda_lib_dir()}", "-lcudart"])
    return LIB


def build_oracle(with_reference: bool | None = None) -> None:
    """Compiles the C oracle; the reference program too when its sources exist.

    Same recipe as oracle/Makefile, invoked directly so that no `make` is needed.
    """
    oracle = ROOT / "oracle"
    (oracle / "bin").mkdir(exist_ok=True)
    cflags = ["-O3", "-std=c11", "-fopenmp", "-fPIC", "-ffp-contract=off"]
    src = [str(oracle / "beam_oracle.c")]
    deps = [oracle / "beam_oracle.c", oracle / "beam_oracle.h", oracle / "oracle_cli.c"]
    jobs = []
    if _stale(oracle / "bin" / "liboracle.so", deps):
        jobs.append(["gcc", *cflags, "-shared", "-o", str(oracle / "bin" / "liboracle.so"), *src, "-lm"])
    if _stale(oracle / "bin" / "beam_oracle", deps):
        jobs.append(["gcc", *cflags, "-o", str(oracle / "bin" / "beam_oracle"), str(oracle / "oracle_cli.c"), *src,
                     "-lm"])
    ref_dir = reference_dir()
    if with_reference is None:
        with_reference = (ref_dir / "src" / "sweg.cpp").exists()
    if with_reference and not (oracle / "_ref" / "beam_ref").exists():
        (oracle / "_ref").mkdir(exist_ok=True)
        ref_srcs = ["src/main.cpp", "src/sweg.cpp", "src/quotient_graph.cpp", "src/cost_oracle.cpp",
                    "src/scoring_cpu.cpp", "src/candidate_index.cpp", "src/graph_io/graph_io.cpp",
                    "src/cuda_scoring_stub.cpp"]
        jobs.append(["g++", "-O3", "-std=c++17", "-fopenmp", "-DNDEBUG", f"-I{ref_dir / 'include'}", "-o",
                     str(oracle / "_ref" / "beam_ref"), *[str(ref_dir / s) for s in ref_srcs]])
    with ThreadPoolExecutor(max_workers=3) as pool:
        list(pool.map(_run, jobs))


def build_all(jobs: int = 8) -> None:
    with ThreadPoolExecutor(max_workers=2) as pool:
        fut_lib = pool.submit(build_library, jobs)
        fut_oracle = pool.submit(build_oracle)
        fut_lib.result()
        fut_oracle.result()


if __name__ == "__main__":
    build_all()
