"""A reusable explorer keeps its hash table across runs.  With 128-bit slots and
state vectors of 64..112 bits every key carries the run's 8-bit generation and
slots of other generations read as free, so a run zeroes the table only when its
contents are unknown (the first run, a change of slot form) or once every 255
generations.  Every run must still equal the oracle: the hardest case is a
replay of the same model, where each key's probe sequence meets its own stale
copy from the previous run before anything else."""
import pytest

from gpuexplore_gb300 import gen
from helpers import FLAGS, oracle, write_net

pytestmark = pytest.mark.gpu


def _same(o, g):
    assert g["rc"] == 0, g
    for k in ("states", "levels", "verdict", "stopped", "set_hash"):
        assert g[k] == o[k], k


def _explorer(gpu, model, **kw):
    kw.setdefault("q_words", 1 << 22)
    return gpu.Explorer(model, gpu.options(**kw))


def _bits(net):
    return net.firstbit()[-1]


@pytest.mark.parametrize("flags", ["deadlock", "safety", "por_proviso", "stubborn_deadlock"])
@pytest.mark.parametrize("graph", [1, 0])
def test_replays_and_model_switch(gpu, tmp_path, flags, graph):
    nets = [gen.random_network(81, nprocs=26, states=(3, 6), outdeg=(1, 2)),
            gen.random_network(82, nprocs=22, states=(5, 9), outdeg=(1, 2))]
    assert all(63 < _bits(n) <= 112 for n in nets)
    paths = [write_net(n, tmp_path, f"m{i}") for i, n in enumerate(nets)]
    cli, kw = FLAGS[flags]
    refs = [oracle(p, cli, max_states=120_000) for p in paths]
    models = [gpu.Model.from_file(p) for p in paths]
    ex = _explorer(gpu, models[0], max_states=120_000, kernel_iters=2, launch_graph=graph, collect_states=1, **kw)
    try:
        expect_gen = 0
        for i in (0, 0, 1, 1, 0, 1, 0):
            ex.set_model(models[i])
            g = ex.run(check=False)
            _same(refs[i], g)
            expect_gen += 1
            assert g["table_generation"] == expect_gen
            assert g["table_cleared"] == (1 if expect_gen == 1 else 0)
            assert g["table_count"] == g["states"]  # slots of the current generation only
    finally:
        ex.close()


def test_generation_wraps(gpu, tmp_path):
    """Generations 1..255, then a clear and generation 1 again."""
    net = gen.random_network(83, nprocs=28, states=(3, 5), outdeg=(1, 2), safety=False)
    assert 63 < _bits(net) <= 112
    path = write_net(net, tmp_path, "w")
    o = oracle(path, ["-d"], max_states=3_000)
    ex = _explorer(gpu, gpu.Model.from_file(path), property="deadlock", max_states=3_000, q_words=1 << 16)
    try:
        seen = []
        for _ in range(262):
            g = ex.run(check=False)
            _same(o, g)
            seen.append((g["table_generation"], g["table_cleared"]))
    finally:
        ex.close()
    assert seen[:255] == [(k, int(k == 1)) for k in range(1, 256)]
    assert seen[255:] == [(1, 1)] + [(k, 0) for k in range(2, 8)]


@pytest.mark.parametrize("slots_per_state", [1.06, 1.3])
def test_high_load_replays(gpu, tmp_path, slots_per_state):
    """A table barely larger than the state space, explored again and again: each
    run's keys land among the previous run's, full probe sequences go through the
    eviction path, and the set stays exact."""
    net = gen.random_network(41, nprocs=28, states=(3, 6), outdeg=(1, 2), safety=False)
    assert 63 < _bits(net) <= 112
    path = write_net(net, tmp_path, "dense")
    o = oracle(path, [], max_states=200_000)
    q_words = (int(o["states"] * slots_per_state) * 16) // 4
    ex = _explorer(gpu, gpu.Model.from_file(path), max_states=200_000, q_words=q_words,
                   store_states=o["states"] + 64, collect_states=1)
    try:
        for k in range(1, 5):
            g = ex.run(check=False)
            _same(o, g)
            assert g["table_generation"] == k and g["table_count"] == g["states"]
    finally:
        ex.close()


def test_switch_between_128_bit_forms(gpu, tmp_path):
    """State vectors above 112 bits take the untagged form (cleared every run); a
    model switch between the forms zeroes the table once."""
    wide = gen.random_network(7, nstates=[15] * 29, outdeg=(1, 2), safety=False)   # 116 bits
    narrow = gen.random_network(84, nprocs=26, states=(3, 6), outdeg=(1, 2), safety=False)
    assert _bits(wide) == 116 and 63 < _bits(narrow) <= 112
    paths = [write_net(n, tmp_path, f"f{i}") for i, n in enumerate((narrow, wide))]
    refs = [oracle(p, ["-d"], max_states=60_000) for p in paths]
    models = [gpu.Model.from_file(p) for p in paths]
    ex = _explorer(gpu, models[0], property="deadlock", max_states=60_000)
    try:
        plan = [(0, 1, 1), (0, 2, 0), (1, 0, 1), (1, 0, 1), (0, 1, 1), (0, 2, 0)]
        for i, generation, cleared in plan:
            ex.set_model(models[i])
            g = ex.run(check=False)
            _same(refs[i], g)
            assert (g["table_generation"], g["table_cleared"]) == (generation, cleared), (i, g["table_generation"])
            assert g["slot_bytes"] == 16
    finally:
        ex.close()


def test_one_shot_calls_clear(gpu, tmp_path):
    """gpx_explore builds a fresh table every call (its first generation, cleared);
    the no-allocation entry point takes the untagged form and clears every call."""
    net = gen.random_network(85, nprocs=26, states=(3, 6), outdeg=(1, 2), safety=False)
    path = write_net(net, tmp_path, "o")
    o = oracle(path, ["-d"], max_states=40_000)
    model = gpu.Model.from_file(path)
    for _ in range(2):
        g = gpu.explore(path, check=False, property="deadlock", max_states=40_000, q_words=1 << 22)
        _same(o, g)
        assert (g["table_generation"], g["table_cleared"]) == (1, 1)
        g = gpu.explore_noalloc(model, check=False, property="deadlock", max_states=40_000, q_words=1 << 22)
        _same(o, g)
        assert (g["table_generation"], g["table_cleared"]) == (0, 1)
