"""Generate the golden fixtures for the exploration path.

The reference ships no tests, fixtures or example models, and has no CPU path,
so its own outputs cannot be recorded here.  The fixtures pin the oracle (and
the GPU path) instead against answers obtained without the oracle:

known_answers.json  tiny networks whose reachable sets, per-level counts and
                    verdicts were derived by hand (the reasoning is in each
                    case's "why"); the script re-checks each one with the
                    independent abstract explorer before writing it.
generated.json      seeded networks from the generators, with the gpf words
                    and the results of the abstract explorer (tests/
                    abstract_explorer.py), which works on tuples of local
                    states and never touches the gpf bit encoding.

Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from gpuexplore_gb300 import gen, gpf  # noqa: E402
from gpuexplore_gb300.gpf import Network  # noqa: E402
import abstract_explorer as ax  # noqa: E402

FLAGSETS = {
    "plain": ([], {}),
    "deadlock": (["-d"], {"prop": "deadlock"}),
    "safety": (["-p"], {"prop": "safety", "proviso": True}),
    "por": (["--por"], {"por": True}),
    "por_proviso": (["--por", "--cycle-proviso"], {"por": True, "proviso": True}),
    "por_safety": (["--por", "-p"], {"por": True, "proviso": True, "prop": "safety"}),
}


def hand_cases():
    """(name, network, {flagset: (states, levels, verdict, stopped)}, why)."""
    cases = []

    # A: two independent processes, local 0 -> 1 each.
    a = Network(nstates=[2, 2], local=[[[1], []], [[1], []]], sync=[[{}, {}], [{}, {}]], rules={})
    cases.append(("two_independent", a, {
        "plain": (4, [1, 2, 1], "none", "done"),
        "deadlock": (4, [1, 2, 1], "deadlock", "violation"),
        "safety": (3, [1, 2], "safety", "violation"),
        "por": (3, [1, 1, 1], "none", "done"),
        "por_proviso": (3, [1, 1, 1], "none", "done"),
    }, "Reachable: (0,0); (1,0),(0,1); (1,1).  (1,1) has no transition -> deadlock found while "
       "expanding level 2, all 4 states visited.  Safety: process 1 (the last) enters local state 1 "
       "from the initial state -> stop after level 1 with 3 states.  POR: at (0,0) both singleton "
       "clusters are valid, the lowest index {0} wins -> (1,0); at (1,0) process 0 is disabled (its "
       "cluster loses its own bit and is invalid), {1} -> (1,1): 3 states, one per level; with the cycle "
       "proviso every successor is unvisited, so the same choice."))

    # B: one handshake with two targets on one side.
    b = Network(nstates=[2, 3], local=[[[], []], [[], [], []]],
                sync=[[{0: [1]}, {}], [{0: [1, 2]}, {}, {}]], rules={0: [0b11]})
    cases.append(("handshake_product", b, {
        "plain": (3, [1, 2], "none", "done"),
        "deadlock": (3, [1, 2], "deadlock", "violation"),
        "safety": (3, [1, 2], "safety", "violation"),
        "por": (3, [1, 2], "none", "done"),
    }, "Rule {0,1} on action 0 gives the product {1} x {1,2}: (1,1),(1,2) at level 1; both are dead. "
       "Safety: the successor (1,1) puts the last process in local state 1 while level 0 is expanded; "
       "exploration stops at the end of that level, so level 1 is still added (3 states)."))

    # C: three-process ring of handshakes, each process 2 states, every state offers
    # both handshakes back to its other state: a_i moves processes i and i+1 together.
    n = 3
    c = Network(nstates=[2] * n, local=[[[], []] for _ in range(n)],
                sync=[[{i: [1 - s], (i - 1) % n: [1 - s]} for s in range(2)] for i in range(n)],
                rules={i: [(1 << i) | (1 << ((i + 1) % n))] for i in range(n)})
    cases.append(("ring3_flip", c, {
        "plain": (4, [1, 3], "none", "done"),
        "deadlock": (4, [1, 3], "none", "done"),
    }, "Each handshake flips two of three bits, so only even-parity vectors are reachable: "
       "000; 110, 011, 101 -> 4 states in 2 levels; every state enables all three handshakes."))

    # D: a 2-process rule with a 3-party rule that can never fire (process 2 never has the action).
    d = Network(nstates=[2, 2, 1], local=[[[], []], [[], []], [[]]],
                sync=[[{0: [1]}, {}], [{0: [1]}, {}], [{}]], rules={0: [0b111, 0b011]})
    cases.append(("partial_rules", d, {
        "plain": (2, [1, 1], "none", "done"),
        "deadlock": (2, [1, 1], "deadlock", "violation"),
    }, "Action 0 has rules {0,1,2} and {0,1}; process 2 never offers action 0, so only {0,1} fires: "
       "(0,0,0) -> (1,1,0), which is dead."))
    return cases


def main():
    hand = []
    for name, net, expect, why in hand_cases():
        words = gpf.encode(net)
        for fs, (states, levels, verdict, stopped) in expect.items():
            got = ax.explore(net, **FLAGSETS[fs][1])
            assert (got["states"], got["levels"], got["verdict"], got["stopped"]) == \
                (states, levels, verdict, stopped), (name, fs, got)
        hand.append({"name": name, "gpf": words, "why": why,
                     "expect": {fs: {"flags": FLAGSETS[fs][0], "states": v[0], "levels": v[1],
                                     "verdict": v[2], "stopped": v[3]} for fs, v in expect.items()}})
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(hand, f, indent=1)

    generated = []
    specs = [("ring", s, {}) for s in (1, 4, 9)] + \
            [("random_network", s, {"nprocs": 6, "states": [3, 5], "outdeg": [1, 3]}) for s in (5, 6)] + \
            [("random_network", 16, {"nprocs": 9, "states": [3, 6], "outdeg": [1, 2], "sync_frac": 0.7})] + \
            [("clustered", s, {"nprocs": 9, "nclusters": [2, 3], "states": [2, 4], "outdeg": [1, 2]}) for s in (7, 8)]
    for fam, seed, kw in specs:
        net = getattr(gen, fam)(seed, **{k: tuple(v) if isinstance(v, list) else v for k, v in kw.items()})
        entry = {"family": fam, "seed": seed, "params": kw, "gpf": gpf.encode(net), "expect": {}}
        for fs, (flags, akw) in FLAGSETS.items():
            got = ax.explore(net, **akw)
            entry["expect"][fs] = {"flags": flags, "states": got["states"], "levels": got["levels"],
                                   "verdict": got["verdict"], "stopped": got["stopped"],
                                   "set_hash": ax.set_hash(net, got["visited"])}
        generated.append(entry)
    with open(os.path.join(HERE, "generated.json"), "w") as f:
        json.dump(generated, f)
    print(f"wrote {len(hand)} hand cases, {len(generated)} generated cases")


if __name__ == "__main__":
    main()
