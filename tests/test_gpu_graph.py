"""A run as one CUDA graph (gpx_options.launch_graph, the default with -v 0):
the exploration launches sit in a device-side while loop whose condition the
relaunch kernel sets, so -k runs need no host round trip between launches.
Results must equal both the host-driven loop and the oracle, including launch
counts, replays of the cached graph, rebuilds after set_model, and runs deeper
than the graph's own level read-back."""
import pytest

from gpuexplore_gb300 import gen, gpf
from helpers import FLAGS, oracle, write_net

pytestmark = pytest.mark.gpu

# lookups depend on which predecessor inserts a state first (commuting-move
# pruning); lookups + pruned, every successor of the expanded states, does not
KEYS = ("states", "levels", "verdict", "stopped", "set_hash", "inserts", "expanded", "successors")


def _same(o, g):
    assert g["rc"] == 0, g
    for k in ("states", "levels", "verdict", "stopped", "set_hash"):
        assert g[k] == o[k], k


@pytest.mark.parametrize("kernel_iters", [0, 1, 3])
@pytest.mark.parametrize("flags", ["deadlock", "safety", "por_proviso", "por_deadlock"])
def test_graph_equals_host_loop(gpu, tmp_path, flags, kernel_iters):
    net = gen.random_network(51, nprocs=10, states=(3, 7))
    path = write_net(net, tmp_path, "g")
    cli, kw = FLAGS[flags]
    o = oracle(path, cli, max_states=150_000)
    runs = {}
    for graph in (1, 0):
        runs[graph] = gpu.explore(path, check=False, max_states=150_000, q_words=1 << 22,
                                  kernel_iters=kernel_iters, launch_graph=graph, **kw)
        runs[graph]["successors"] = runs[graph]["lookups"] + runs[graph]["pruned"]
        _same(o, runs[graph])
    for k in KEYS + ("launches",):
        assert runs[1][k] == runs[0][k], k
    if kernel_iters:
        assert runs[1]["launches"] > 1


def test_graph_replay_and_rebuild(gpu, tmp_path):
    """The graph is built once and replayed; set_model (another launch shape and
    model size) rebuilds it."""
    nets = [gen.random_network(61, nprocs=9, states=(3, 6)), gen.ring(3),
            gen.random_network(62, nprocs=8, states=(4, 8)), gen.ring(3)]
    paths = [write_net(n, tmp_path, f"m{i}") for i, n in enumerate(nets)]
    cli, kw = FLAGS["deadlock"]
    refs = [oracle(p, cli, max_states=100_000) for p in paths]
    models = [gpu.Model.from_file(p) for p in paths]
    ex = gpu.Explorer(models[0], gpu.options(max_states=100_000, q_words=1 << 22, kernel_iters=2, **kw))
    try:
        for _ in range(3):  # replays
            _same(refs[0], ex.run(check=False))
        for m, ref in zip(models[1:], refs[1:]):
            ex.set_model(m)
            for _ in range(2):
                _same(ref, ex.run(check=False))
    finally:
        ex.close()


def test_graph_deep_chain(gpu, tmp_path):
    """5000 BFS levels: more than the graph reads back itself (4096), the rest is copied after."""
    n = 5000
    net = gpf.Network(nstates=[n], local=[[[s + 1] if s + 1 < n else [] for s in range(n)]],
                      sync=[[{} for _ in range(n)]], rules={})
    path = write_net(net, tmp_path, "chain")
    o = oracle(path, ["-d"])
    assert len(o["levels"]) == n and o["verdict"] == "deadlock"
    for graph in (1, 0):
        g = gpu.explore(path, check=False, q_words=1 << 20, property="deadlock", launch_graph=graph)
        _same(o, g)
