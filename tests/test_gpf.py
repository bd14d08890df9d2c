"""gpf format and generators (CPU)."""
import random

import pytest

from gpuexplore_gb300 import gen, gpf
from gpuexplore_gb300.gpf import Network
import abstract_explorer as ax


def _canon(net):
    return (net.nstates, [[sorted(t) for t in p] for p in net.local],
            [[{a: sorted(t) for a, t in d.items()} for d in p] for p in net.sync],
            {a: sorted(r) for a, r in net.rules.items() if r})


@pytest.mark.parametrize("seed", range(8))
def test_roundtrip(seed):
    for net in (gen.ring(seed), gen.random_network(seed, nprocs=7, states=(3, 9)),
                gen.clustered(seed, nprocs=11)):
        words = gpf.encode(net)
        back = gpf.decode(words)
        assert _canon(back) == _canon(net)
        assert gpf.encode(back) == words


def test_write_read(tmp_path):
    net = gen.random_network(3)
    p = tmp_path / "m.gpf"
    gpf.write(net, str(p))
    assert gpf.read_words(str(p)) == gpf.encode(net)
    h = gpf.header(gpf.encode(net))
    assert h.nr_procs == net.nprocs and h.firstbit == net.firstbit()
    assert h.bits_statevector == net.firstbit()[-1] + 1


def test_generators_deterministic():
    assert gpf.encode(gen.random_network(42)) == gpf.encode(gen.random_network(42))
    assert gpf.encode(gen.ring(5)) == gpf.encode(gen.ring(5))
    assert gpf.encode(gen.clustered(5)) != gpf.encode(gen.clustered(6))


def test_generator_invariants():
    """Rules have >= 2 participants, <= 2 entries per (p, s, a), no repeated targets."""
    for seed in range(20):
        net = gen.random_network(seed, nprocs=10, states=(4, 20))
        words = gpf.encode(net)
        assert gpf.header(words).max_buf_ints <= 2
        for rs in net.rules.values():
            assert all(bin(r).count("1") >= 2 for r in rs)


def test_monitor_tracks_error_pair():
    """Every reachable state's monitor equals f(s_i == a, s_j == b); the count is unchanged."""
    for seed in range(6):
        base = gen.random_network(seed, nprocs=5, states=(3, 5), safety=False)
        rng = random.Random(seed)
        i, j = rng.sample(range(5), 2)
        a, b = rng.randrange(1, base.nstates[i]), rng.randrange(1, base.nstates[j])
        # sync transitions crossing the error states are not allowed; make them local
        for p, e in ((i, a), (j, b)):
            for s in range(base.nstates[p]):
                for act in list(base.sync[p][s]):
                    ts = base.sync[p][s][act]
                    cross = [t for t in ts if (s == e) != (t == e)]
                    for t in cross:
                        ts.remove(t)
                        if t not in base.local[p][s]:
                            base.local[p][s].append(t)
                    if not ts:
                        del base.sync[p][s][act]
        mon = gen.add_safety_monitor(base, i, a, j, b)
        r0 = ax.explore(base)
        r1 = ax.explore(mon)
        assert r1["states"] == r0["states"]
        for s in r1["visited"]:
            A, B = s[i] == a, s[j] == b
            assert s[-1] == {(False, False): 0, (True, True): 1, (True, False): 2, (False, True): 3}[(A, B)]


def test_validate_rejects():
    bad = Network(nstates=[2], local=[[[1, 1], []]], sync=[[{}, {}]])
    with pytest.raises(ValueError):
        gpf.encode(bad)
    bad = Network(nstates=[2], local=[[[5], []]], sync=[[{}, {}]])
    with pytest.raises(ValueError):
        gpf.encode(bad)
    bad = Network(nstates=[2, 2], local=[[[], []], [[], []]], sync=[[{0: []}, {}], [{}, {}]], rules={0: [3]})
    with pytest.raises(ValueError):
        gpf.encode(bad)
