"""An independent BFS over the generators' abstract networks (test helper).

It works on :class:`gpuexplore_gb300.gpf.Network` objects directly -- tuples of
local states, Python dicts -- and never touches the gpf encoding, so agreement
with the C oracle (which decodes gpf bit fields) pins the encoder, the oracle's
decoder and its successor relation at once.  It restates the same semantics as
the oracle (GPUexplore.cu:904-1122 successors, 1134-1151 deadlock, 927-935 and
1063-1069 safety, 1345-1675 cluster POR with the cycle proviso evaluated
against the visited set at the start of the level).  Small models only.
"""
from __future__ import annotations

from itertools import product
from typing import Dict, List, Optional, Set, Tuple

from gpuexplore_gb300.gpf import Network

State = Tuple[int, ...]


def successors(net: Network, s: State) -> List[Tuple[State, int]]:
    """All successors of s with their origin mask (1<<p for a local move of p,
    the rule mask for a synchronisation)."""
    n = net.nprocs
    out: List[Tuple[State, int]] = []
    for p in range(n):
        for t in net.local[p][s[p]]:
            v = list(s)
            v[p] = t
            out.append((tuple(v), 1 << p))
    actions = set()
    for p in range(n):
        actions.update(net.sync[p][s[p]])
    for a in sorted(actions):
        enabled = {p for p in range(n) if a in net.sync[p][s[p]]}
        for r in net.rules.get(a, []):
            parts = [p for p in range(n) if r >> p & 1]
            if not set(parts) <= enabled:
                continue
            for combo in product(*[net.sync[p][s[p]][a] for p in parts]):
                v = list(s)
                for p, t in zip(parts, combo):
                    v[p] = t
                out.append((tuple(v), r))
    return out


def static_clusters(net: Network, s: State) -> List[int]:
    n = net.nprocs
    cl = []
    for p in range(n):
        c = 1 << p
        for a in net.sync[p][s[p]]:
            for r in net.rules.get(a, []):
                if r >> p & 1:
                    c |= r
        cl.append(c)
    return cl


def stubborn_clusters(net: Network, s: State) -> List[int]:
    """Per process: itself, and for each rule containing it of an action it has
    enabled, the rule's members if all have the action, else the rule's lowest
    member without it (a necessary enabling process)."""
    n = net.nprocs
    cl = []
    for p in range(n):
        c = 1 << p
        for a in net.sync[p][s[p]]:
            for r in net.rules.get(a, []):
                if not r >> p & 1:
                    continue
                lack = [q for q in range(n) if r >> q & 1 and a not in net.sync[q][s[q]]]
                c |= (1 << lack[0]) if lack else r
        cl.append(c)
    return cl


def select_cluster(n: int, cl: List[int], prov: int, ample: bool = False) -> int:
    c = [cl[p] if prov >> p & 1 else cl[p] & ~(1 << p) for p in range(n)]
    best, bestc = (1 << n) - 1, n
    for p in range(n):
        closure = c[p]
        stack = [i for i in range(n) if c[p] >> i & 1]
        seen = set(stack)
        while stack:
            i = stack.pop()
            closure |= c[i]
            for j in range(n):
                if c[i] >> j & 1 and j not in seen:
                    seen.add(j)
                    stack.append(j)
        valid = any(c[i] >> i & 1 for i in range(n) if closure >> i & 1)
        if valid and closure and (not ample or bin(closure).count("1") == 1) and bin(closure).count("1") < bestc:
            bestc, best = bin(closure).count("1"), closure
    return best


def explore(net: Network, prop: str = "none", por: bool = False, proviso: bool = False,
            max_states: int = 0, kind: str = "cample") -> Dict:
    """BFS; with `por`, the cluster reduction of `kind`: "cample" (static
    clusters), "ample" (single-process clusters only) or "stubborn"
    (necessary-enabling clusters)."""
    n = net.nprocs
    init: State = tuple([0] * n)
    visited: Set[State] = {init}
    frontier = [init]
    levels = [1]
    verdict = "none"
    stopped = "done"
    while frontier:
        violation = False
        nxt: List[State] = []
        decisions: Dict[State, int] = {}
        for s in frontier:
            succ = successors(net, s)
            if prop == "deadlock" and not succ:
                violation = True
            if prop == "safety" and any(t[n - 1] == 1 for t, _ in succ):
                violation = True
            sel = (1 << n) - 1
            if por:
                prov = 0
                for t, mask in succ:
                    if not proviso or t not in visited:
                        prov |= mask
                cl = stubborn_clusters(net, s) if kind == "stubborn" else static_clusters(net, s)
                sel = select_cluster(n, cl, prov, ample=kind == "ample")
            decisions[s] = sel
        for s in frontier:
            sel = decisions[s]
            for t, mask in successors(net, s):
                if mask & sel == mask and t not in visited:
                    visited.add(t)
                    nxt.append(t)
        if nxt:
            levels.append(len(nxt))
        frontier = nxt
        if violation:
            verdict = prop
            stopped = "violation"
            break
        if max_states and len(visited) >= max_states and frontier:
            stopped = "budget"
            break
    return {"states": len(visited), "levels": levels, "verdict": verdict, "stopped": stopped,
            "visited": visited}


def explore_pruned(net: Network, rng, max_states: int = 0) -> Dict:
    """Plain BFS with commuting-move pruning, restated independently of the
    kernel: every new state is labelled with the participants of the move that
    first inserted it; a state does not generate a move led by a process below
    its label's lowest participant that is disjoint from the label.  Expansion
    and successor order are shuffled with `rng`, so the labels -- which
    predecessor inserts a state first -- vary as they do between GPU runs."""
    n = net.nprocs
    init: State = tuple([0] * n)
    label: Dict[State, int] = {init: 0}
    frontier = [init]
    levels = [1]
    generated = pruned = 0
    while frontier:
        rng.shuffle(frontier)
        nxt: List[State] = []
        for s in frontier:
            lab = label[s]
            low = (lab & -lab).bit_length() - 1
            succ = successors(net, s)
            rng.shuffle(succ)
            for t, mask in succ:
                lead = (mask & -mask).bit_length() - 1
                if lab and lead < low and mask & lab == 0:
                    pruned += 1
                    continue
                generated += 1
                if t not in label:
                    label[t] = mask
                    nxt.append(t)
        if nxt:
            levels.append(len(nxt))
        frontier = nxt
        if max_states and len(label) >= max_states and frontier:
            break
    return {"states": len(label), "levels": levels, "visited": set(label), "generated": generated,
            "pruned": pruned}


def pack(net: Network, s: State) -> List[int]:
    """Pack a state tuple into gpf state-vector words (firstbit layout)."""
    fb = net.firstbit()
    W = max(1, (fb[-1] + 31) // 32)
    x = 0
    for p, v in enumerate(s):
        x |= v << fb[p]
    return [(x >> (32 * i)) & 0xFFFFFFFF for i in range(W)]


MASK64 = (1 << 64) - 1


def _mix64(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def key_hash(words: List[int]) -> int:
    h = 0x9E3779B97F4A7C15
    for j in range(0, len(words), 2):
        c = words[j] | ((words[j + 1] << 32) if j + 1 < len(words) else 0)
        h = _mix64(h ^ c)
    return h


def set_hash(net: Network, states: Optional[Set[State]]) -> str:
    total = 0
    for s in states or ():
        total = (total + key_hash(pack(net, s))) & MASK64
    return f"{total:016x}"


def accepting_cycle(net: Network, max_states: int = 200_000) -> Tuple[int, bool]:
    """(reachable states, whether a reachable cycle passes through a state whose
    last process is in local state 1) -- the liveness check, by networkx's
    strongly connected components over the explicit graph."""
    import networkx as nx

    init = tuple([0] * net.nprocs)
    g = nx.DiGraph()
    g.add_node(init)
    seen = {init}
    stack = [init]
    while stack:
        s = stack.pop()
        for v, _ in successors(net, s):
            g.add_edge(s, v)
            if v not in seen:
                seen.add(v)
                if len(seen) > max_states:
                    raise ValueError("state space too large for the networkx check")
                stack.append(v)
    acc = False
    for comp in nx.strongly_connected_components(g):
        if not any(s[-1] == 1 for s in comp):
            continue
        if len(comp) > 1:
            acc = True
            break
        (s,) = tuple(comp)
        if g.has_edge(s, s):
            acc = True
            break
    return len(seen), acc
