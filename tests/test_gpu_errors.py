"""Error paths of the GPU path: invalid states and requests are reported as
errors with the reference's messages, never as wrong results."""

import pytest

pytestmark = pytest.mark.gpu


def test_duplicate_edges_fail_like_reference(golden):
    from beam_gb300 import Engine, Graph
    from beam_gb300._native import BeamError
    case = golden["errors"][0]
    u, v = zip(*case["edges"])
    g = Graph.from_edges(list(u), list(v))
    with Engine(g) as e:
        with pytest.raises(BeamError, match=case["message"]):
            e.run(20)


def test_score_pairs_rejects_inactive_and_equal_endpoints():
    from beam_gb300 import Engine, Graph
    from beam_gb300._native import BeamError
    g = Graph.generate("gnm:n=50,m=120,seed=2")
    with Engine(g) as e:
        e.merge_pairs([0], [1])
        with pytest.raises(BeamError):
            e.score_pairs([1], [2])   # 1 was merged into 0
    with Engine(g) as e:
        with pytest.raises(BeamError):
            e.score_pairs([3], [3])
    with Engine(g) as e:
        with pytest.raises(BeamError):
            e.score_pairs([0], [g.n + 5])


def test_merge_batch_must_be_disjoint():
    from beam_gb300 import Engine, Graph
    from beam_gb300._native import BeamError
    g = Graph.generate("gnm:n=50,m=120,seed=2")
    with Engine(g) as e:
        with pytest.raises(BeamError, match="endpoint-disjoint"):
            e.merge_pairs([0, 1], [2, 0])


def test_group_limit_is_enforced():
    from beam_gb300 import Engine, Graph
    from beam_gb300._native import BeamError
    g = Graph.generate("gnm:n=50,m=120,seed=2")
    with pytest.raises(BeamError, match="divide-max-group"):
        Engine(g, divide_max_group=4096)


def test_merge_requires_divide():
    from beam_gb300 import Engine, Graph
    from beam_gb300._native import BeamError
    g = Graph.generate("gnm:n=50,m=120,seed=2")
    with Engine(g) as e:
        with pytest.raises(BeamError, match="Divide"):
            e.merge(1)


class RawCSR:
    def __init__(self, row_ptr, col_idx):
        import numpy as np
        self.row_ptr = np.asarray(row_ptr, np.int64)
        self.col_idx = np.asarray(col_idx, np.int32)
        self.n = len(row_ptr) - 1
        self.arcs = len(col_idx)


@pytest.mark.parametrize("row_ptr,col_idx", [([0, 2, 3, 4], [0, 1, 0, 0]),    # self-loop 0-0
                                             ([0, 1, 2, 3], [1, 7, 0])])      # neighbour out of range
def test_engine_rejects_invalid_csr_on_the_device(row_ptr, col_idx):
    from beam_gb300 import Engine
    from beam_gb300._native import BeamError
    with pytest.raises(BeamError, match="loop-free graph with valid neighbors"):
        Engine(RawCSR(row_ptr, col_idx))
