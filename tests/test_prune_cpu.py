"""Commuting-move pruning, checked on the CPU against unpruned BFS: the same
per-level counts and visited set whatever order decides which predecessor
inserts a state first (the order is shuffled, as races shuffle it on the GPU),
on networks with local moves only, with many multi-party synchronisations, and
with clusters."""
import random

import pytest

import abstract_explorer as ax
from gpuexplore_gb300 import gen


def _nets(seed):
    return (gen.ring(seed, nprocs=6, nstates=4),
            gen.random_network(seed, nprocs=7, states=(3, 5), safety=False),
            gen.random_network(seed + 50, nprocs=7, states=(2, 5), parties=(2, 4), sync_frac=0.7, safety=False),
            gen.random_network(seed + 90, nprocs=6, states=(3, 5), sync_frac=0.0, safety=False),
            gen.clustered(seed, nprocs=8, nclusters=(2, 3), states=(2, 4), outdeg=(1, 2)))


@pytest.mark.parametrize("seed", range(12))
def test_same_levels_and_set(seed):
    for k, net in enumerate(_nets(seed)):
        ref = ax.explore(net)
        total = None
        for order in range(3):
            got = ax.explore_pruned(net, random.Random(1000 * seed + 10 * k + order))
            assert got["levels"] == ref["levels"], (k, order)
            assert got["visited"] == ref["visited"], (k, order)
            # every successor of every state is either generated or pruned
            if total is None:
                total = got["generated"] + got["pruned"]
            assert got["generated"] + got["pruned"] == total


def test_prunes_most_diamonds():
    """Independent local moves: most successors follow from another order."""
    net = gen.random_network(3, nprocs=6, states=(3, 5), sync_frac=0.0, safety=False)
    got = ax.explore_pruned(net, random.Random(0), max_states=20_000)
    assert got["pruned"] > 2 * got["generated"]
