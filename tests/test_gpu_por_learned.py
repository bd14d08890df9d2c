"""Learned cluster proposal: training kernels, exploration parity with the
oracle's restatement of the learned selection, soundness of verdicts."""
import os

import numpy as np
import pytest

from gpuexplore_gb300 import gen, gpf, learned_por
from helpers import oracle, write_net
from mlp_reference import F, H, forward_backward

pytestmark = pytest.mark.gpu


def test_gradients_match_cpu_reference(gpu):
    rng = np.random.default_rng(1)
    rows = 3000
    x = rng.integers(0, 60, size=(rows, F)).astype(np.uint8)
    y = rng.normal(1.5, 0.7, size=rows).astype(np.float32)
    w1 = rng.normal(0, 0.15, size=(H, F)).astype(np.float32)
    b1 = rng.normal(0, 0.1, size=H).astype(np.float32)
    w2 = rng.normal(0, 0.2, size=H).astype(np.float32)
    b2 = np.float32(0.2)
    loss, gw1, gb1, gw2, gb2 = gpu.por_grad(w1, b1, w2, b2, x, y)
    rl, rw1, rb1, rw2, rb2 = forward_backward(w1, b1, w2, b2, x, y)
    assert loss == pytest.approx(rl, rel=1e-4)
    for g, r in ((gw1, rw1), (gb1, rb1), (gw2, rw2)):
        assert np.allclose(g, r, rtol=2e-3, atol=2e-3 * np.abs(r).max())
    assert gb2 == pytest.approx(rb2, rel=1e-3, abs=1e-6)


def test_training_reduces_loss(gpu):
    rng = np.random.default_rng(2)
    x = rng.integers(0, 30, size=(20000, F)).astype(np.uint8)
    y = (0.05 * x[:, 2] + 0.1 * x[:, 0] + 0.02 * x[:, 9]).astype(np.float32)
    m0, l0 = gpu.por_train(x, y, epochs=1, lr=1e-4)
    m1, l1 = gpu.por_train(x, y, epochs=25)
    assert l1 < 0.2 * l0


@pytest.mark.parametrize("seed", [3, 4, 5, 6])
def test_learned_por_matches_oracle(gpu, tmp_path, seed):
    """Any weights: the GPU's learned selection equals the oracle's restatement."""
    model = learned_por.random_model(seed)
    mpath = str(tmp_path / "m.bin")
    learned_por.save(model, mpath)
    for k, net in enumerate((gen.random_network(100 + seed, nprocs=9, states=(4, 8)),
                             gen.clustered(200 + seed, nprocs=12, nclusters=(3, 4)),
                             gen.random_network(300 + seed, nprocs=20, states=(3, 6), outdeg=(1, 2)))):
        path = write_net(net, tmp_path, f"n{k}")
        for cli, kw in ((["--por", "-p"], dict(property="safety", cycle_proviso=1)),
                        (["--por", "-d"], dict(property="deadlock")),
                        (["--por", "--cycle-proviso"], dict(cycle_proviso=1))):
            o = oracle(path, cli + ["--por-model", mpath], max_states=300_000)
            m = gpu.Model.from_file(path)
            ex = gpu.Explorer(m, gpu.options(por=2, max_states=300_000, q_words=1 << 24, **kw))
            ex.set_por_model(model)
            r = ex.run()
            ex.close()
            for key in ("states", "levels", "verdict", "stopped", "set_hash"):
                assert r[key] == o[key], (seed, k, cli, key)
            plain = oracle(path, cli, max_states=300_000)
            assert o["verdict"] == plain["verdict"] or "budget" in (o["stopped"], plain["stopped"])


def test_batch_learned_jobs_match_oracle(gpu, tmp_path):
    model = learned_por.random_model(11)
    mpath = str(tmp_path / "m.bin")
    learned_por.save(model, mpath)
    models, jobs, want = [], [], []
    for k in range(10):
        path = write_net(gen.random_network(400 + k, nprocs=9, states=(4, 8)), tmp_path, f"b{k}")
        models.append(gpu.Model.from_file(path))
        jobs.append({"property": "safety", "por": 2, "cycle_proviso": 1, "max_states": 100_000})
        want.append(oracle(path, ["--por", "-p", "--por-model", mpath], max_states=100_000))
    items, st = gpu.batch_explore(models, jobs, por_model=model)
    for it, w in zip(items, want):
        for key in ("states", "levels", "verdict", "set_hash"):
            assert it[key] == w[key]


def test_candidate_log(gpu):
    rows = learned_por.log_candidates([7], budget=20_000, sample_every=4)
    assert len(rows) > 100
    assert np.all(rows["x"][:, 0] == rows["popc"])
    assert np.all(rows["x"][:, 7] == 1)
    assert np.all(rows["new_succ"] <= rows["succ"])
    # exactly one logged candidate per expanded state is plain cample's choice
    tags, counts = np.unique(rows["state_tag"][rows["cample_choice"] == 1], return_counts=True)
    assert len(tags) > 10 and counts.max() == 1


def test_trained_proposal_gains_over_cample(gpu):
    """Trained on logs of 400 config-2 networks, the proposal needs no more states
    to reach the verdict than plain cample on held-out networks BFS decides, with
    every verdict equal to unreduced BFS."""
    rows = learned_por.log_candidates(range(1, 401), budget=20_000, sample_every=128)
    model, loss = learned_por.train(rows, target="succ")
    ev = learned_por.evaluate(model, range(1_000_001, 1_000_061), budget=2_000_000)
    assert ev["verdict_mismatch_learned"] == 0 and ev["verdict_mismatch_cample"] == 0
    assert ev["decided"] >= 10
    gain = 1.0 - ev["decided_states_learned"] / ev["decided_states_cample"]
    print(f"learned proposal: {gain:.1%} fewer states to the verdict than plain cample "
          f"({ev['decided_states_learned']} vs {ev['decided_states_cample']}, {ev['decided']} decided seeds)")
    assert gain > 0.0
