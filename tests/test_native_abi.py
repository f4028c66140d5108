"""The C-ABI library loads without a GPU and exports every function declared
in include/*.h, including the reference's two C++-linkage functions; the CLI
validates its flags like the reference's (no GPU call is made)."""

import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "beam_gb300" / "bin" / "beam"


def declared_functions():
    names = set()
    text = (ROOT / "include" / "beam_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for m in re.finditer(r"\b(beam_[a-z0-9_]+)\s*\(", text):
        names.add(m.group(1))
    return sorted(names)


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "beam_gb300" / "libbeam_gb300.so")],
                         capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_library_loads_and_binds_every_declared_function():
    from beam_gb300 import _native as N
    lib = N.lib()
    declared = declared_functions()
    assert len(declared) > 40
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) <= set(N.SIGNATURES), sorted(set(declared) - set(N.SIGNATURES))


def test_every_declared_function_is_exported():
    syms = exported_symbols()
    missing = [n for n in declared_functions() if n not in syms]
    assert not missing, missing


def test_reference_cuda_scoring_functions_are_exported_with_cpp_linkage():
    syms = exported_symbols()
    # const char* CudaScoringBuildMode(); bool CudaScoringCompiled();
    assert "_Z20CudaScoringBuildModev" in syms
    assert "_Z19CudaScoringCompiledv" in syms
    hdr = (ROOT / "include" / "cuda_scoring.hpp").read_text()
    assert "const char* CudaScoringBuildMode();" in hdr and "bool CudaScoringCompiled();" in hdr


def run_cli(*args):
    return subprocess.run([str(CLI), *args], capture_output=True, text=True, timeout=60)


def test_cli_usage_and_missing_input(tmp_path):
    # src/main.cpp:428-431: usage, exit 1 without --input, exit 0 for --help after --input
    r = run_cli("--help")
    assert r.returncode == 1 and "Usage:" in r.stdout
    r = run_cli()
    assert r.returncode == 1 and "Usage:" in r.stdout
    r = run_cli("--input", str(tmp_path / "g.txt"), "--help")
    assert r.returncode == 0 and "Usage:" in r.stdout


@pytest.mark.parametrize("flag,value", [("--scoring-backend", "cpu"), ("--cost-objective", "legacy"),
                                        ("--merge-mode", "batch"), ("--commit-policy", "t4"),
                                        ("--certification", "safe"), ("--threshold-policy", "adaptive")])
def test_cli_rejects_modes_outside_the_recommended_one(tmp_path, flag, value):
    from beam_gb300 import REFERENCE_FLAGS
    g = tmp_path / "g.txt"
    g.write_text("0 1\n1 2\n")
    flags = list(REFERENCE_FLAGS)
    flags[flags.index("--scoring-backend") + 1] = "cuda"
    flags[flags.index(flag) + 1] = value
    r = run_cli("--input", str(g), *flags)
    assert r.returncode == 1 and r.stdout.startswith("Error:") and flag in r.stdout


@pytest.mark.parametrize("text,message", [("0 0\n", "Self-loop is not supported at line 1."),
                                          ("0 1\n-1 2\n", "Negative node id at line 2."),
                                          ("0 1\nx y\n", "Malformed edge list line 2"),
                                          ("", "Invalid node count."),
                                          ("# only a comment\n", "Invalid node count.")])
def test_cli_reports_input_errors_like_the_reference(tmp_path, text, message):
    from beam_gb300 import REFERENCE_FLAGS
    g = tmp_path / "g.txt"
    g.write_text(text)
    flags = list(REFERENCE_FLAGS)
    flags[flags.index("--scoring-backend") + 1] = "cuda"
    r = run_cli("--input", str(g), *flags)
    assert r.returncode == 1
    assert r.stdout.strip().endswith(message) or message in r.stdout


def test_cli_requires_out_with_write_output(tmp_path):
    g = tmp_path / "g.txt"
    g.write_text("0 1\n")
    r = run_cli("--input", str(g), "--write-output")
    assert r.returncode == 1 and "--write-output requires --out <dir>." in r.stdout
