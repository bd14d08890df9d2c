"""GPU parity: libgpx (CUDA, through the C ABI) against the CPU oracle.

Bit-exact on every integer result: visited-state count, per-level counts,
verdict, stop reason and the order-independent hash of the visited set; for
small models the full visited set is compared row by row.
"""
import numpy as np
import pytest

from gpuexplore_gb300 import gen
from helpers import FLAGS, oracle, write_net

pytestmark = pytest.mark.gpu


def _gpu(lib, path, kw, **extra):
    args = dict(kw)
    args.update(extra)
    args.setdefault("q_words", 1 << 22)
    return lib.explore(path, check=False, **args)


def _same(o, g):
    assert g["rc"] == 0, g
    assert g["states"] == o["states"]
    assert g["levels"] == o["levels"]
    assert g["verdict"] == o["verdict"]
    assert g["stopped"] == o["stopped"]
    assert g["set_hash"] == o["set_hash"]


MODELS = {
    "ring1": lambda: gen.ring(1),
    "ring2": lambda: gen.ring(2),
    "ring7": lambda: gen.ring(7),
    "rand6": lambda: gen.random_network(11, nprocs=6, states=(3, 6)),           # 32-bit keys
    "rand12": lambda: gen.random_network(12, nprocs=12, states=(4, 9)),         # 64-bit keys
    "rand24": lambda: gen.random_network(13, nprocs=24, states=(4, 9), outdeg=(1, 2)),  # 128-bit keys
    "dead9": lambda: gen.random_network(16, nprocs=9, states=(3, 6), outdeg=(1, 2), sync_frac=0.7),
    "clus10": lambda: gen.clustered(14, nprocs=10, nclusters=(3, 3)),
    "clus16": lambda: gen.clustered(15, nprocs=16, nclusters=(4, 5), states=(3, 5)),
}


@pytest.mark.parametrize("model", sorted(MODELS))
@pytest.mark.parametrize("flags", sorted(FLAGS))
def test_parity(gpu, tmp_path, model, flags):
    net = MODELS[model]()
    path = write_net(net, tmp_path, model)
    cli, kw = FLAGS[flags]
    budget = 300_000
    o = oracle(path, cli, max_states=budget)
    g = _gpu(gpu, path, kw, max_states=budget, q_words=1 << 24)
    _same(o, g)


@pytest.mark.parametrize("launch", [dict(blocks=1, threads=32), dict(kernel_iters=1), dict(kernel_iters=3),
                                    dict(blocks=7, threads=96)])
def test_launch_shapes(gpu, tmp_path, launch):
    net = gen.random_network(21, nprocs=9, states=(3, 7))
    path = write_net(net, tmp_path, "shape")
    for flags in ("deadlock", "por_proviso"):
        cli, kw = FLAGS[flags]
        o = oracle(path, cli, max_states=100_000)
        g = _gpu(gpu, path, kw, max_states=100_000, **launch)
        _same(o, g)
        if launch.get("kernel_iters"):
            assert g["launches"] >= (len(g["levels"]) - 1) // launch["kernel_iters"]  # one level per expansion


def test_full_set_rows(gpu, tmp_path):
    """The visited set row by row (sorted), not only its hash."""
    net = gen.random_network(31, nprocs=10, states=(3, 6))
    path = write_net(net, tmp_path, "rows")
    dump = str(tmp_path / "oracle.bin")
    o = oracle(path, [], dump=dump)
    g = _gpu(gpu, path, {}, collect_states=1)
    _same(o, g)
    ref = np.fromfile(dump, dtype=np.uint32).reshape(-1, g["key_words"])
    got = g["states_words"]
    assert got.shape == ref.shape
    srt = lambda a: a[np.lexsort(a.T[::-1])]  # noqa: E731
    assert np.array_equal(srt(got), srt(ref))
    # the store holds each state once, and the table holds exactly the stored states
    assert len(np.unique(got, axis=0)) == len(got)
    assert g["table_count"] == g["states"]
    # BFS order: level boundaries of the store match the per-level counts
    assert got.shape[0] == sum(g["levels"])


@pytest.mark.parametrize("flags", ["por_proviso", "stubborn_proviso", "ample_safety", "safety"])
def test_high_load_eviction_with_reductions(gpu, tmp_path, flags):
    """Bounded eviction under the cycle proviso (whose decide pass looks keys up
    after level-close eviction has moved some) with cample, stubborn and ample
    clusters over thousands of levels, and under the safety check with pruning."""
    net = gen.random_network(42, nprocs=28, states=(3, 6), outdeg=(1, 2))
    assert net.firstbit()[-1] > 63
    path = write_net(net, tmp_path, "dense")
    cli, kw = FLAGS[flags]
    o = oracle(path, cli, max_states=150_000)
    q_words = (int(o["states"] * 1.08) * 16) // 4
    g = _gpu(gpu, path, kw, max_states=150_000, q_words=q_words, store_states=o["states"] + 64, collect_states=1)
    _same(o, g)
    assert g["table_count"] == g["states"]


@pytest.mark.parametrize("slots_per_state", [1.03, 1.06, 1.15])
def test_high_load_bounded_eviction(gpu, tmp_path, slots_per_state):
    """A table barely larger than the state space (97% load at 1.03 slots per
    state): inserts whose probe sequence is full are placed after their level,
    by every warp at once, displacing occupants along chains of at most four
    moves; the visited set stays exact and every state is stored once."""
    net = gen.random_network(41, nprocs=28, states=(3, 6), outdeg=(1, 2), safety=False)
    assert net.firstbit()[-1] > 63  # 128-bit slots: 2 per bucket, the tightest case
    path = write_net(net, tmp_path, "dense")
    o = oracle(path, [], max_states=200_000)
    slots = int(o["states"] * slots_per_state)
    q_words = (slots * 16) // 4
    g = _gpu(gpu, path, {}, max_states=200_000, q_words=q_words, store_states=o["states"] + 64,
             collect_states=1)
    _same(o, g)
    assert g["table_count"] == g["states"]  # every state stored exactly once
    if slots_per_state < 1.1:
        assert g["evictions"] > 0
        assert g["overflowed"] > 0 and g["evict_ms"] > 0  # the placement phases ran and were timed


# exact key-width boundaries: 31/32 bits (32- vs 64-bit slots), 63/64 (64- vs
# 128-bit), 112/113 (generation-tagged vs untagged 128-bit slots), and 126 bits
# over 31 processes (the widest vector and the process limit)
WIDTHS = {31: [15] * 7 + [7], 32: [15] * 8, 63: [15] * 15 + [7], 64: [15] * 16, 112: [15] * 28,
          113: [31] + [15] * 27, 126: [31, 31] + [15] * 29}


@pytest.mark.parametrize("bits", sorted(WIDTHS))
@pytest.mark.parametrize("flags", ["deadlock", "por_proviso", "stubborn_deadlock"])
def test_width_boundaries(gpu, tmp_path, bits, flags):
    net = gen.random_network(7, nstates=WIDTHS[bits], outdeg=(1, 2), safety=False)
    assert net.firstbit()[-1] == bits
    path = write_net(net, tmp_path, f"w{bits}")
    cli, kw = FLAGS[flags]
    o = oracle(path, cli, max_states=60_000)
    g = _gpu(gpu, path, kw, max_states=60_000)
    _same(o, g)
    assert g["slot_bytes"] == (4 if bits <= 31 else (8 if bits <= 63 else 16))
    assert g["table_generation"] == (1 if 64 <= bits <= 112 else 0)


@pytest.mark.parametrize("seed,nprocs,width,slots_per_state", [(45, 11, 4, 1.01), (43, 14, 8, 1.02)])
def test_high_load_eviction_narrow_slots(gpu, tmp_path, seed, nprocs, width, slots_per_state):
    """Placement with eviction on 32- and 64-bit slots (8 and 4 per bucket, so
    longer probe sequences: 98-99% load to make them overflow): parity with the
    oracle, every state stored once."""
    net = gen.random_network(seed, nprocs=nprocs, states=(3, 6), outdeg=(1, 2), safety=False)
    bits = net.firstbit()[-1]
    assert (4 if bits <= 31 else (8 if bits <= 63 else 16)) == width
    path = write_net(net, tmp_path, f"narrow{width}")
    o = oracle(path, [], max_states=150_000)
    assert o["states"] > 20_000
    q_words = (int(o["states"] * slots_per_state) * width + 63) // 4
    g = _gpu(gpu, path, {}, max_states=150_000, q_words=q_words, store_states=o["states"] + 64, collect_states=1)
    _same(o, g)
    assert g["table_count"] == g["states"]
    assert g["slot_bytes"] == width and g["overflowed"] > 0
