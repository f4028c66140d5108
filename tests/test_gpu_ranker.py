"""The learned candidate ranker on the GPU.

- Its training kernels: the gradient (and loss, logits) of one forward +
  backward pass equals the float64 CPU oracle (oracle/ranker_oracle.py)
  within fp32 accumulation error: rtol 2e-3 on every parameter, with an
  absolute floor of 1e-4 x the largest gradient entry.
- Its use in the merge loop: after training on the first iterations it
  prunes candidate pairs before exact scoring; every merge is still decided
  on exact integer gains, the cost ratio stays within 0.1 % absolute of the
  same form without the ranker, and the audit (pruned pairs scored aside)
  reports the recall."""

import numpy as np
import pytest

import ranker_oracle as R

pytestmark = pytest.mark.gpu


def data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, R.FEAT)).astype(np.float32)
    y = (rng.random(n) < 0.25).astype(np.float32)
    w = rng.uniform(0.5, 4.0, n).astype(np.float32)
    return x, y, w


@pytest.mark.parametrize("n,weighted", [(1, False), (255, True), (1000, True), (4096, False), (20000, True)])
def test_gradient_matches_oracle(n, weighted):
    from beam_gb300 import ranker_grad
    x, y, w = data(n, n)
    p = R.init_params(n)
    g, loss, z = ranker_grad(x, y, p, w if weighted else None)
    l_ref, g_ref, z_ref = R.loss_and_grad(p, x, y, w if weighted else None)
    floor = 1e-4 * np.abs(g_ref).max()
    np.testing.assert_allclose(g, g_ref, rtol=2e-3, atol=floor)
    assert abs(loss - l_ref) <= 1e-4 * max(1.0, abs(l_ref))
    np.testing.assert_allclose(z, z_ref, rtol=1e-4, atol=1e-4)


def test_gradient_is_deterministic():
    from beam_gb300 import ranker_grad
    x, y, w = data(9000, 5)
    p = R.init_params(5)
    g1, l1, _ = ranker_grad(x, y, p, w)
    g2, l2, _ = ranker_grad(x, y, p, w)
    assert np.array_equal(g1, g2) and l1 == l2


SPEC = "chunglu:n=20000,gamma=2.3,deg=8,twins=1500,seed=5"


def run(g, **kw):
    from beam_gb300 import Engine, partition_hash
    with Engine(g, group_batch_size=1 << 30, **kw) as e:
        e.run(20)
        labels, head, nxt = e.partition()
        st = e.stats()
        info = e.ranker_info() if kw.get("ranker") else None
    return partition_hash(labels), g.encode(head, nxt)["cost_ratio_mags_compatible"], st, info


def test_ranker_prunes_and_keeps_cost_ratio():
    from beam_gb300 import Graph
    g = Graph.generate(SPEC)
    _, ratio0, st0, _ = run(g)
    h1, ratio1, st1, info = run(g, ranker=True, ranker_audit=True)
    assert info["trained"] == 1 and info["samples"] >= 256 and info["positives"] > 0
    assert info["final_loss"] < info["first_loss"]
    assert info["pruned"] > 0
    # pruned pairs are not scored: fewer exact gain calls than the same form without the ranker
    assert st1["merge_exact_gain_calls"] < st0["merge_exact_gain_calls"]
    assert abs(ratio1 - ratio0) <= 1e-3
    recall = 1.0 - info["audit_lost"] / max(1, info["audit_passing"])
    assert recall >= 0.9, info
    # what the trained network gains over pruning without it: a random prune
    # of the same fraction of candidates keeps about 1 - fraction of the pairs
    # that pass the filter; the ranker keeps far more
    fraction = info["pruned"] / info["ranked"]
    assert recall >= (1.0 - fraction) + 0.25, (recall, fraction)
    # deterministic: the same run gives the same partition
    h2, _, _, _ = run(g, ranker=True, ranker_audit=True)
    assert h1 == h2
