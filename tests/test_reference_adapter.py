"""The reference-side adapter (beam_gb300/adapter/cuda_scoring_gb300.cpp)
compiled into the reference program in place of its CUDA scoring
translation unit (src/cuda_scoring.cu), linked against libbeam_gb300.so.

Runs wherever the reference's sources are present (BEAM_REFERENCE_DIR, else a
`reference` checkout beside this repository); skipped otherwise. The
reference's sources are compiled from where they lie; the patched build
copies them to a temporary directory first and applies the three edits that
INTEGRATION.md lists for the whole-loop hook.
"""

import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
LIB_DIR = ROOT / "beam_gb300"
ADAPTER = ROOT / "beam_gb300" / "adapter" / "cuda_scoring_gb300.cpp"
REF_SRCS = ["src/main.cpp", "src/sweg.cpp", "src/quotient_graph.cpp", "src/cost_oracle.cpp", "src/scoring_cpu.cpp",
            "src/candidate_index.cpp", "src/graph_io/graph_io.cpp"]


def reference_dir() -> Path:
    env = os.environ.get("BEAM_REFERENCE_DIR")
    return Path(env) if env else ROOT.parent / "reference"


REF = reference_dir()
pytestmark = pytest.mark.skipif(not (REF / "src" / "sweg.cpp").exists(),
                                reason="the reference's sources are not present")

# The three reference-side edits of the whole-loop hook.
HOOK_EDITS = [
    ("include/sweg.hpp", "  void Run(int iterations, int print_offset);\n",
     "  void Run(int iterations, int print_offset);\n  void RunOnGb300(int iterations);\n"),
    ("src/sweg.cpp", "void Sweg::Run(int iterations, int print_offset) {\n  ResetRuntimeStats();\n",
     "void Sweg::Run(int iterations, int print_offset) {\n  ResetRuntimeStats();\n"
     "  if (scoring_backend_ == ScoringBackend::kCuda && cost_objective_ == CostObjective::kMagsCompatible) {\n"
     "    const auto gb300_start = std::chrono::steady_clock::now();\n"
     "    RunOnGb300(iterations);\n"
     "    stats_.runtime_run_ms = ElapsedMs(gb300_start, std::chrono::steady_clock::now());\n"
     "    return;\n  }\n"),
    ("src/main.cpp", "    if (opts.cost_objective == CostObjective::kMagsCompatible &&\n"
                     "        opts.scoring_backend == ScoringBackend::kCuda) {\n", "    if (false) {\n"),
]


def build(src_root: Path, out: Path, defines=()) -> None:
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", *defines, f"-I{src_root / 'include'}", f"-I{ROOT / 'include'}",
           "-o", str(out), *[str(src_root / s) for s in REF_SRCS], str(ADAPTER), f"-L{LIB_DIR}", "-lbeam_gb300",
           f"-Wl,-rpath,{LIB_DIR}"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-4000:]


def small_graph(tmp: Path) -> Path:
    g = tmp / "g.txt"
    g.write_text("".join(f"{u} {v}\n" for u, v in [(0, 1), (1, 2), (2, 0), (3, 4), (4, 5), (5, 3), (2, 3), (5, 6)]))
    return g


def test_adapter_replaces_the_cuda_translation_unit(tmp_path):
    """Unmodified reference + adapter: links, reports the GB300 build, and its
    own CPU mode still gives the golden partition of the same graph."""
    from conftest import GOLDEN
    from beam_gb300 import REFERENCE_FLAGS
    exe = tmp_path / "beam_ref_gb300"
    build(REF, exe)
    proc = subprocess.run([str(exe), "--input", str(small_graph(tmp_path)), *REFERENCE_FLAGS],
                          capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert proc.returncode == 0, proc.stderr
    assert "CUDA scoring build: cuda" in proc.stdout
    want = next(c for c in GOLDEN["cases"] if c["name"] == "two_triangles_bridge")["metrics"]["partition_hash"]
    assert f"metric.partition_hash={want}" in proc.stdout


def test_adapter_whole_loop_hook_builds_against_the_edited_reference(tmp_path):
    """The reference with the three edits + the adapter's Run hook: compiles and
    links. Without a GPU the engine cannot be created, which must surface as
    the reference's 'Error: ...' exit 1."""
    import shutil
    src = tmp_path / "ref"
    shutil.copytree(REF / "src", src / "src")
    shutil.copytree(REF / "include", src / "include")
    for rel, old, new in HOOK_EDITS:
        p = src / rel
        text = p.read_text()
        assert text.count(old) == 1, f"edit anchor not found in {rel}"
        p.write_text(text.replace(old, new))
    exe = tmp_path / "beam_ref_gb300_hook"
    build(src, exe, ["-DBEAM_GB300_RUN_HOOK"])
    from beam_gb300 import REFERENCE_FLAGS
    flags = [("cuda" if f == "cpu" else f) for f in REFERENCE_FLAGS]
    proc = subprocess.run([str(exe), "--input", str(small_graph(tmp_path)), *flags], capture_output=True, text=True,
                          env=dict(os.environ, OMP_NUM_THREADS="2"))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        from conftest import GOLDEN
        want = next(c for c in GOLDEN["cases"] if c["name"] == "two_triangles_bridge")["metrics"]["partition_hash"]
        assert proc.returncode == 0, proc.stderr
        assert f"metric.partition_hash={want}" in proc.stdout
    else:
        assert proc.returncode == 1
        assert proc.stderr.startswith("Error:") or "Error:" in proc.stderr + proc.stdout
