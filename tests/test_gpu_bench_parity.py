"""GPU parity on the exact networks and settings the benchmark times.

The headline figure (config 2) and the other configuration lines are only as
good as the results they count, so each is compared here with the CPU oracle:
visited-state count, per-level counts, verdict, stop reason and the
order-independent hash of the visited set.  Semantics: successor generation
of G:904-1122 (GPUexplore/src/GPUexplore.cu), cluster POR with the cycle
proviso of G:1345-1675, verdicts of G:927-935, 1063-1069, 1134-1151.
"""
import os

import pytest

from gpuexplore_gb300 import workloads as W
from helpers import oracle, write_net

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 2


def _same(o, g):
    assert g["rc"] == 0, g
    for k in ("states", "levels", "verdict", "stopped", "set_hash"):
        assert g[k] == o[k], (k, g[k], o[k])


@pytest.mark.parametrize("prop,prune", [("deadlock", 1), ("deadlock", 0), ("safety", 1)])
def test_config2_sample(gpu, tmp_path, prop, prune):
    """The config-2 network, -d and -p, to the 1e7 budget (the first 9 BFS
    levels, 38.8M states), with the bench's 20 GB table; with and without
    commuting-move pruning."""
    path = write_net(W.config2_network(), tmp_path, "config2")
    cli, kw = W.PROPERTY_FLAGS[prop]
    o = oracle(path, cli, threads=THREADS, max_states=W.CONFIG2_SAMPLE_BUDGET)
    g = gpu.explore(path, check=False, q_words=W.CONFIG2_Q_WORDS, max_states=W.CONFIG2_SAMPLE_BUDGET,
                    prune_commuting=prune, **kw)
    _same(o, g)
    if prop == "safety":
        assert g["verdict"] == "safety"  # the embedded monitor's error state is reachable


def test_config2_headline(gpu, tmp_path):
    """The headline workload itself: -d to the end of the level reaching 1e8
    states (10 levels, 161.9M states) in the 20 GB table, through a reusable
    explorer's CUDA graph, two runs in a row (the second reuses the table by
    generation)."""
    path = write_net(W.config2_network(), tmp_path, "config2")
    cli, kw = W.PROPERTY_FLAGS["deadlock"]
    o = oracle(path, cli, threads=THREADS, max_states=W.CONFIG2_BUDGET)
    m = gpu.Model.from_file(path)
    ex = gpu.Explorer(m, gpu.options(q_words=W.CONFIG2_Q_WORDS, max_states=W.CONFIG2_BUDGET, **kw))
    try:
        for _ in range(2):
            _same(o, ex.run(check=False))
    finally:
        ex.close()


@pytest.mark.parametrize("seed", W.CONFIG3_SEEDS)
def test_config3(gpu, tmp_path, seed):
    """A config-3 clustered network (24 processes) under --por --cycle-proviso
    at the bench's own budget and table size."""
    net = W.config3_networks()[W.CONFIG3_SEEDS.index(seed)]
    path = write_net(net, tmp_path, f"config3_{seed}")
    cli, kw = W.PROPERTY_FLAGS["por_proviso"]
    o = oracle(path, cli, threads=THREADS, max_states=W.CONFIG3_BUDGET)
    g = gpu.explore(path, check=False, q_words=W.CONFIG3_Q_WORDS, max_states=W.CONFIG3_BUDGET, **kw)
    _same(o, g)


def test_config1_rings(gpu, tmp_path):
    """All ten config-1 rings, -d, in the 2^22-word table."""
    cli, kw = W.PROPERTY_FLAGS["deadlock"]
    for seed, net in zip(W.CONFIG1_SEEDS, W.config1_networks()):
        path = write_net(net, tmp_path, f"ring{seed}")
        o = oracle(path, cli, threads=THREADS)
        g = gpu.explore(path, check=False, q_words=W.CONFIG1_Q_WORDS, **kw)
        _same(o, g)
