"""Commuting-move pruning on the GPU (gpx_options.prune_commuting, on by
default in plain exploration): the visited set, level counts, verdicts and stop
levels equal the oracle's and the unpruned run's; every successor is either
looked up or pruned; pruning removes most lookups where moves are independent."""
import pytest

from gpuexplore_gb300 import gen
from helpers import FLAGS, oracle, write_net

pytestmark = pytest.mark.gpu

NETS = {
    "local": lambda: gen.random_network(91, nprocs=8, states=(3, 6), sync_frac=0.0, safety=False),
    "rand12": lambda: gen.random_network(12, nprocs=12, states=(4, 9)),
    "sync4": lambda: gen.random_network(92, nprocs=9, states=(3, 5), parties=(2, 4), sync_frac=0.7),
    "dead9": lambda: gen.random_network(16, nprocs=9, states=(3, 6), outdeg=(1, 2), sync_frac=0.7),
    "rand26": lambda: gen.random_network(81, nprocs=26, states=(3, 6), outdeg=(1, 2)),
    "clus16": lambda: gen.clustered(15, nprocs=16, nclusters=(4, 5), states=(3, 5)),
}


def _same(o, g):
    assert g["rc"] == 0, g
    for k in ("states", "levels", "verdict", "stopped", "set_hash"):
        assert g[k] == o[k], k


@pytest.mark.parametrize("flags", ["plain", "deadlock", "safety"])
@pytest.mark.parametrize("name", sorted(NETS))
def test_pruned_equals_unpruned(gpu, tmp_path, name, flags):
    path = write_net(NETS[name](), tmp_path, name)
    cli, kw = FLAGS[flags]
    o = oracle(path, cli, max_states=150_000)
    runs = {}
    for prune in (1, 0):
        runs[prune] = gpu.explore(path, check=False, max_states=150_000, q_words=1 << 22, prune_commuting=prune, **kw)
        _same(o, runs[prune])
    on, off = runs[1], runs[0]
    assert off["pruned"] == 0
    assert on["lookups"] + on["pruned"] == off["lookups"] == o["generated"]  # every successor, once
    assert on["inserts"] == off["inserts"] and on["expanded"] == off["expanded"]
    if name == "local" and on["states"] > 1000:
        assert on["pruned"] > 2 * on["lookups"]


@pytest.mark.parametrize("kernel_iters", [1, 3])
def test_labels_across_launches_and_replays(gpu, tmp_path, kernel_iters):
    """Labels live in device memory across -k launches and are rewritten by
    every run of a reused explorer."""
    net = gen.random_network(93, nprocs=14, states=(3, 7), outdeg=(1, 3))
    path = write_net(net, tmp_path, "k")
    cli, kw = FLAGS["deadlock"]
    o = oracle(path, cli, max_states=200_000)
    ex = gpu.Explorer(gpu.Model.from_file(path),
                      gpu.options(max_states=200_000, q_words=1 << 22, kernel_iters=kernel_iters, **kw))
    try:
        for _ in range(3):
            g = ex.run(check=False)
            _same(o, g)
            assert g["pruned"] > 0 and g["launches"] > 1
    finally:
        ex.close()


def test_overflowed_states_keep_exactness(gpu, tmp_path):
    """States placed by bounded eviction at the end of a level carry no label
    (nothing is pruned from them); the visited set stays exact."""
    net = gen.random_network(41, nprocs=28, states=(3, 6), outdeg=(1, 2), safety=False)
    path = write_net(net, tmp_path, "dense")
    o = oracle(path, [], max_states=200_000)
    q_words = (int(o["states"] * 1.06) * 16) // 4
    g = gpu.explore(path, check=False, max_states=200_000, q_words=q_words, store_states=o["states"] + 64,
                    collect_states=1)
    _same(o, g)
    assert g["evictions"] > 0 and g["pruned"] > 0 and g["table_count"] == g["states"]


def test_por_modes_do_not_prune(gpu, tmp_path):
    path = write_net(NETS["rand12"](), tmp_path, "p")
    for flags in ("por_proviso", "por_deadlock", "stubborn_deadlock"):
        cli, kw = FLAGS[flags]
        o = oracle(path, cli, max_states=100_000)
        g = gpu.explore(path, check=False, max_states=100_000, q_words=1 << 22, **kw)
        _same(o, g)
        assert g["pruned"] == 0
