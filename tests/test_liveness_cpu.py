"""Liveness (accepting-cycle) check of the oracle, pinned against an independent
check: networkx strongly connected components over the generators' abstract
model (tests/abstract_explorer.py), and hand-derived answers on tiny networks.

The gpf liveness flag means here: the last process is a Buchi automaton whose
local state 1 is accepting; the property is violated iff a reachable cycle
passes through an accepting state.
"""
import subprocess

import pytest

from abstract_explorer import accepting_cycle
from gpuexplore_gb300 import gen, gpf
from gpuexplore_gb300.build import ORACLE
from helpers import oracle, write_net


def _net(nstates, local, sync=None, rules=None):
    sync = sync or [[{} for _ in range(n)] for n in nstates]
    return gpf.Network(nstates=nstates, local=local, sync=sync, rules=rules or {}, liveness=1)


KNOWN = {
    # the property process alone: 0 -> 1 -> 1 (self-loop in the accepting state)
    "accepting_self_loop": (_net([2], [[[1], [1]]]), "liveness"),
    # 0 -> 1 and stuck: no cycle at all (a deadlock, not an infinite run)
    "no_cycle": (_net([2], [[[1], []]]), "none"),
    # a cycle 0 -> 1 -> 0 through the accepting state
    "accepting_two_cycle": (_net([2], [[[1], [0]]]), "liveness"),
    # process 0 cycles forever, the property process never leaves 0
    "cycle_never_accepting": (_net([2, 2], [[[1], [0]], [[], []]]), "none"),
    # the property process passes through 1 on a one-way path, nothing else cycles
    "accepting_transient": (_net([2, 3], [[[1], []], [[1], [2], []]]), "none"),
    # ... unless process 0 keeps cycling while it sits in 1: violation
    "accepting_with_other_cycle": (_net([2, 2], [[[1], [0]], [[1], []]]), "liveness"),
}


@pytest.mark.parametrize("name", sorted(KNOWN))
def test_known_answers(built, tmp_path, name):
    net, want = KNOWN[name]
    n, acc = accepting_cycle(net)
    assert ("liveness" if acc else "none") == want
    o = oracle(write_net(net, tmp_path, name), ["-p"])
    assert o["verdict"] == want
    assert o["stopped"] == ("violation" if want != "none" else "done")
    assert o["states"] == n


@pytest.mark.parametrize("seed", range(8))
def test_oracle_matches_networkx_random(built, tmp_path, seed):
    net = gen.liveness_network(seed)
    n, acc = accepting_cycle(net)
    o = oracle(write_net(net, tmp_path, "l"), ["-p"], threads=2)
    assert o["states"] == n
    assert o["verdict"] == ("liveness" if acc else "none")
    assert (o["live_states"] > 0) == acc


@pytest.mark.parametrize("cyclic", [False, True])
@pytest.mark.parametrize("seed", range(5))
def test_oracle_matches_networkx_progress(built, tmp_path, seed, cyclic):
    net = gen.progress_network(seed, cyclic=cyclic)
    n, acc = accepting_cycle(net)
    assert acc == cyclic  # the verdict the construction promises
    o = oracle(write_net(net, tmp_path, "p"), ["-p"], threads=2)
    assert o["states"] == n and o["verdict"] == ("liveness" if acc else "none")


def test_liveness_flag_without_p_checks_nothing(built, tmp_path):
    """As in the reference, -d (or no property flag) ignores the liveness flag."""
    net = gen.progress_network(0, cyclic=True)
    path = write_net(net, tmp_path, "p")
    assert oracle(path, [])["verdict"] == "none"
    assert oracle(path, ["-d"])["verdict"] in ("none", "deadlock")


def test_oracle_rejects_por_with_liveness(built, tmp_path):
    path = write_net(gen.progress_network(1), tmp_path, "p")
    out = subprocess.run([ORACLE, path, "-p", "--por"], capture_output=True, text=True)
    assert out.returncode == 1 and "liveness" in out.stderr


def test_liveness_generator_monitor_never_blocks():
    """The monitor enables every transition it observes: projected on the other
    processes, the monitored network reaches exactly the states of the network
    without it (the observed synchronisations turned back into local moves)."""
    from abstract_explorer import successors

    net = gen.progress_network(3)
    E = max(net.rules)  # the observed action, shared by process 0 and the monitor only
    n = net.nprocs - 1
    base = gpf.Network(nstates=net.nstates[:n], local=[[list(ts) for ts in net.local[p]] for p in range(n)],
                       sync=[[dict((a, ts) for a, ts in d.items() if a != E) for d in net.sync[p]] for p in range(n)],
                       rules=dict((a, r) for a, r in net.rules.items() if a != E))
    for s in range(net.nstates[0]):
        base.local[0][s] += net.sync[0][s].get(E, [])

    def reach(nw):
        init = tuple([0] * nw.nprocs)
        seen, stack = {init}, [init]
        while stack:
            for v, _ in successors(nw, stack.pop()):
                if v not in seen:
                    seen.add(v)
                    stack.append(v)
        return seen

    assert {s[:n] for s in reach(net)} == reach(base)
