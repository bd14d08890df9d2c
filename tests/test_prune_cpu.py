"""Commuting-move pruning, checked on the CPU against unpruned BFS: the same
per-level counts and visited set whatever order decides which predecessor
inserts a state first (the order is shuffled, as races shuffle it on the GPU),
on networks with local moves only, with many multi-party synchronisations, and
with clusters."""
import functools
import operator
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


def _por_pruned_states(net):
    """Cluster POR (no proviso) with the pruning rule applied on top: the
    combination the kernels do not make."""
    n = net.nprocs
    init = tuple([0] * n)
    label = {init: 0}
    frontier = [init]
    while frontier:
        sel = {s: ax.select_cluster(n, ax.static_clusters(net, s),
                                    functools.reduce(operator.or_, (m for _, m in ax.successors(net, s)), 0))
               for s in frontier}
        nxt = []
        for s in frontier:
            lab = label[s]
            low = (lab & -lab).bit_length() - 1
            for t, mask in ax.successors(net, s):
                lead = (mask & -mask).bit_length() - 1
                if mask & sel[s] != mask or (lab and lead < low and mask & lab == 0):
                    continue
                if t not in label:
                    label[t] = mask
                    nxt.append(t)
        frontier = nxt
    return set(label)


def test_unsound_under_por():
    """Why only plain exploration prunes: a reduced expansion need not contain
    the commuted path the argument relies on, so pruning inside cluster POR can
    lose states (here one of four)."""
    net = gen.random_network(182, nprocs=5, states=(2, 4), outdeg=(1, 2), safety=False)
    ref = ax.explore(net, por=True)["visited"]
    got = _por_pruned_states(net)
    assert got < ref
