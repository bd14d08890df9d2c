"""Ample and stubborn POR variants in the oracle: exact agreement (states, levels,
verdict, visited set) with the abstract explorer's independent restatement,
and the verdict of unreduced BFS preserved on seeded networks."""
import pytest

import abstract_explorer as ax
from gpuexplore_gb300 import gen
from helpers import oracle, write_net

KINDS = {"ample": "--ample", "stubborn": "--stubborn"}


def _nets(seed):
    return (gen.ring(seed, nprocs=5, nstates=4),
            gen.random_network(seed, nprocs=6, states=(3, 5)),
            gen.random_network(seed + 100, nprocs=7, states=(3, 5), parties=(2, 4), sync_frac=0.5, safety=False),
            gen.clustered(seed, nprocs=8, nclusters=(2, 3), states=(2, 4), outdeg=(1, 2)))


@pytest.mark.parametrize("kind", sorted(KINDS))
@pytest.mark.parametrize("seed", range(20, 25))
def test_against_abstract_explorer(built, tmp_path, seed, kind):
    flags = {("-d",): {"prop": "deadlock"}, ("-p",): {"prop": "safety", "proviso": True},
             (): {}, ("--cycle-proviso",): {"proviso": True}}
    for k, net in enumerate(_nets(seed)):
        path = write_net(net, tmp_path, f"m{k}")
        for fl, kw in flags.items():
            a = ax.explore(net, por=True, kind=kind, **kw)
            o = oracle(path, [KINDS[kind]] + list(fl), threads=2)
            assert o["states"] == a["states"] and o["levels"] == a["levels"], (k, fl)
            assert o["verdict"] == a["verdict"] and o["set_hash"] == ax.set_hash(net, a["visited"]), (k, fl)


@pytest.mark.parametrize("seed", range(40))
def test_verdicts_preserved(built, tmp_path, seed):
    """Deadlocks (-d, no proviso needed) and safety violations (-p, cycle proviso)
    are found by every reduction exactly when unreduced BFS finds them."""
    net = (gen.random_network(seed, nprocs=7, states=(3, 6), outdeg=(1, 3), parties=(2, 4)) if seed % 2
           else gen.clustered(seed, nprocs=10, nclusters=(3, 4)))
    path = write_net(net, tmp_path, "n")
    for prop in ("-d", "-p"):
        ref = oracle(path, [prop], threads=2)
        for flag in ("--por", "--ample", "--stubborn"):
            o = oracle(path, [prop, flag], threads=2)
            assert o["verdict"] == ref["verdict"], (prop, flag)
            if ref["verdict"] == "none":
                assert o["states"] <= ref["states"]


def test_stubborn_clusters_within_static(built):
    """Necessary-enabling clusters are subsets of the static clusters, state by state."""
    smaller = 0
    for seed in range(6):
        net = gen.random_network(seed, nprocs=7, states=(3, 5), parties=(2, 4), sync_frac=0.6)
        for s in ax.explore(net)["visited"]:
            st, sb = ax.static_clusters(net, s), ax.stubborn_clusters(net, s)
            assert all(b & ~a == 0 for a, b in zip(st, sb))
            smaller += sum(a != b for a, b in zip(st, sb))
    assert smaller > 0  # 3- and 4-party rules with a member lacking the action
