import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

GOLDEN = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def flag_value(flags, name, default):
    if name in flags:
        i = flags.index(name)
        return flags[i + 1]
    return default


def options_from_flags(flags):
    """Engine/oracle keyword options for a list of reference flags."""
    # --merge-mode batch-ea commits group by group: blocks of one group
    batch_ea = flag_value(flags, "--merge-mode", "batch-ea-blocked") == "batch-ea"
    return {
        "top_k": int(flag_value(flags, "--top-k", 16)),
        "group_batch_size": 1 if batch_ea else int(flag_value(flags, "--group-batch-size", 64)),
        "divide_hash_dims": int(flag_value(flags, "--divide-hash-dims", 16)),
        "divide_max_group": int(flag_value(flags, "--divide-max-group", 512)),
        "ea_use_threshold": "--ea-use-threshold" in flags,
        "seed": int(flag_value(flags, "--seed", 1)),
    }


def iterations_from_flags(flags):
    return int(flag_value(flags, "--iterations", 20))


def golden_cases(include_large=True, include_huge=True):
    return [c for c in GOLDEN["cases"]
            if (include_large or not c["large"]) and (include_huge or not c.get("huge", False))]


def graph_for(case):
    from beam_gb300 import Graph
    if "spec" in case:
        return Graph.generate(case["spec"])
    u, v = zip(*case["edges"])
    return Graph.from_edges(list(u), list(v))


def file_hashes(out_dir):
    import hashlib
    return {f: hashlib.sha256((Path(out_dir) / f).read_bytes()).hexdigest()
            for f in ("G.txt", "P.txt", "Cp.txt", "Cm.txt")}


@pytest.fixture(scope="session")
def golden():
    return GOLDEN
