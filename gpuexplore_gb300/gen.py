"""Seeded generators of gpf networks (the reference's model generator and model
set are not available, so the benchmark and test networks are built here).

Every generator is a pure function of its seed (Python's `random.Random`, so the
same file is produced on any host).  The generated networks keep by default to
the subset of the gpf semantics on which the reference's two successor kernels
agree (GPUexplore.cu:756-1189 vs 1191-1733): every synchronisation rule has at
least two participants, one (process, state, action) never needs more than two
transition entries (max_buf_ints <= 2), and targets are never repeated.
:func:`corner_network` (with gpf.encode's max_slots / repeat_seed) leaves that
subset on purpose.

Families
--------
ring            ring of n processes, each an m-state LTS with one local tau edge
                and two handshake actions with its neighbours (rule {i, i+1})
random_network  n processes with U[lo, hi] states, out-degree U[1, 4], a share of
                the transitions synchronising 2-3 processes, and optionally an
                embedded safety monitor over a seeded pair of error local states
clustered       processes in seeded clusters, transitions mostly inside the
                cluster (tau or intra-cluster sync) and a share of
                cross-cluster synchronisations
corner_network  random networks with single-party synchronisation rules and
                few actions per process (many targets per action)
batch           many random networks of uneven sizes
"""
from __future__ import annotations

import random
from typing import Dict, List, Optional, Tuple

from .gpf import Network


def _empty(nstates: List[int]) -> Network:
    return Network(
        nstates=list(nstates),
        local=[[[] for _ in range(ns)] for ns in nstates],
        sync=[[{} for _ in range(ns)] for ns in nstates],
        rules={},
    )


def _add_sync(net: Network, p: int, s: int, a: int, t: int) -> bool:
    ts = net.sync[p][s].setdefault(a, [])
    if t in ts:
        return False
    ts.append(t)
    return True


def _add_local(net: Network, p: int, s: int, t: int) -> bool:
    if t in net.local[p][s]:
        return False
    net.local[p][s].append(t)
    return True


def ring(seed: int, nprocs: int = 8, nstates: int = 5, p_sync: float = 0.9) -> Network:
    """Ring of `nprocs` processes with `nstates` local states each.

    Process i has one local tau edge (a seeded state to a seeded other state) and
    takes part in two handshake actions: h_i with its right neighbour (rule
    {i, i+1 mod n}) and h_{i-1} with its left neighbour.  Each state offers each
    handshake with probability `p_sync`, to a seeded target.  The seed also picks
    each process's initial local state; states are relabelled so that it is 0
    (the reference's initial state is the all-zero vector, GPUexplore.cu:673-676).
    """
    rng = random.Random(seed)
    net = _empty([nstates] * nprocs)
    for a in range(nprocs):
        net.rules[a] = [(1 << a) | (1 << ((a + 1) % nprocs))]
    for i in range(nprocs):
        init = rng.randrange(nstates)
        perm = list(range(nstates))
        perm[0], perm[init] = perm[init], perm[0]  # relabel: seeded initial state -> 0
        src = rng.randrange(nstates)
        tgt = rng.choice([x for x in range(nstates) if x != src])
        _add_local(net, i, perm[src], perm[tgt])
        for s in range(nstates):
            for a in (i, (i - 1) % nprocs):
                if rng.random() < p_sync:
                    _add_sync(net, i, perm[s], a, perm[rng.randrange(nstates)])
    return net


def add_safety_monitor(net: Network, i: int, a: int, j: int, b: int) -> Network:
    """Embed the safety property "never process i in local state a while process j
    is in local state b" as a monitor process appended last.

    The reference checks a safety property as "the last process reaches local
    state 1" (GPUexplore.cu:927-935, 1063-1069).  Every local transition of i that
    enters or leaves a (and of j for b) becomes a two-party synchronisation with the
    monitor, whose four states track (i in a, j in b): 0 = neither, 1 = both (the
    error state), 2 = only i in a, 3 = only j in b.  The monitor enables every
    action it observes in every state where it can occur, so it never blocks and
    the reachable state count equals that of the unmonitored network.
    Requires a != 0, b != 0 (the initial state maps to monitor state 0) and that
    no synchronising transition of i (j) enters or leaves a (b).
    """
    if i == j or a == 0 or b == 0:
        raise ValueError("need two distinct processes and nonzero error states")
    n = net.nprocs
    M = n
    base = net.nactions()
    E_i, L_i, E_j, L_j = base, base + 1, base + 2, base + 3
    out = Network(
        nstates=net.nstates + [4],
        local=[[list(ts) for ts in net.local[p]] for p in range(n)] + [[[] for _ in range(4)]],
        sync=[[dict((k, list(v)) for k, v in d.items()) for d in net.sync[p]] for p in range(n)]
        + [[{} for _ in range(4)]],
        rules=dict((k, list(v)) for k, v in net.rules.items()),
        liveness=net.liveness,
    )
    for proc, err, enter, leave in ((i, a, E_i, L_i), (j, b, E_j, L_j)):
        for s in range(out.nstates[proc]):
            for aa, ts in out.sync[proc][s].items():
                for t in ts:
                    if (s == err) != (t == err):
                        raise ValueError("a synchronising transition crosses an error state")
            keep = []
            for t in out.local[proc][s]:
                if s != err and t == err:
                    _add_sync(out, proc, s, enter, t)
                elif s == err and t != err:
                    _add_sync(out, proc, s, leave, t)
                else:
                    keep.append(t)
            out.local[proc][s] = keep
        out.rules[enter] = [(1 << proc) | (1 << M)]
        out.rules[leave] = [(1 << proc) | (1 << M)]
    # monitor transitions: states 0=(-A,-B) 1=(A,B) 2=(A,-B) 3=(-A,B)
    for act, moves in ((E_i, ((0, 2), (3, 1))), (L_i, ((2, 0), (1, 3))),
                       (E_j, ((0, 3), (2, 1))), (L_j, ((3, 0), (1, 2)))):
        for s, t in moves:
            _add_sync(out, M, s, act, t)
    return out


def add_liveness_monitor(net: Network, i: int, a: int) -> Network:
    """Embed the liveness property "process i takes a transition into local state
    a infinitely often" as a Buchi monitor for its negation, appended last, and
    set the gpf liveness flag.

    Accepting state 1 (the convention the safety monitor uses for its error
    state): monitor state 0 may guess, by a local tau, that no such transition
    follows any more and move to 1; in 1 a transition of i into a traps the
    monitor in state 2.  Every local transition of i into a becomes a two-party
    synchronisation with the monitor, enabled in all three monitor states, so
    the monitor never blocks the network.  A violation is a reachable cycle
    through a state with the monitor in 1: a run on which i eventually never
    enters a again.  Requires that no synchronising transition of i targets a.
    """
    n = net.nprocs
    M = n
    E = net.nactions()
    for s in range(net.nstates[i]):
        for ts in net.sync[i][s].values():
            if a in ts:
                raise ValueError("a synchronising transition of i targets a")
    out = Network(
        nstates=net.nstates + [3],
        local=[[list(ts) for ts in net.local[p]] for p in range(n)] + [[[1], [], []]],
        sync=[[dict((k, list(v)) for k, v in d.items()) for d in net.sync[p]] for p in range(n)]
        + [[{} for _ in range(3)]],
        rules=dict((k, list(v)) for k, v in net.rules.items()),
        liveness=1,
    )
    for s in range(out.nstates[i]):
        keep = []
        for t in out.local[i][s]:
            if t == a:
                _add_sync(out, i, s, E, t)
            else:
                keep.append(t)
        out.local[i][s] = keep
    out.rules[E] = [(1 << i) | (1 << M)]
    for s, t in ((0, 0), (1, 2), (2, 2)):
        _add_sync(out, M, s, E, t)
    return out


def liveness_network(seed: int, nprocs: int = 6, states: Tuple[int, int] = (3, 6),
                     outdeg: Tuple[int, int] = (1, 2), sync_frac: float = 0.3) -> Network:
    """A random network (no safety monitor) with a liveness monitor over a seeded
    (process, local state) pair that no synchronising transition targets."""
    rng = random.Random(seed * 7919 + 13)
    for attempt in range(64):
        net = random_network(seed * 1000 + attempt, nprocs=nprocs, states=states, outdeg=outdeg,
                             sync_frac=sync_frac, safety=False)
        pairs = [(i, a) for i in range(nprocs) for a in range(net.nstates[i])
                 if not any(a in ts for st in net.sync[i] for ts in st.values())
                 and any(a in ts for ts in net.local[i])]
        if pairs:
            i, a = rng.choice(pairs)
            return add_liveness_monitor(net, i, a)
    raise ValueError("no eligible (process, state) pair")


def progress_network(seed: int, nprocs: int = 5, states: Tuple[int, int] = (3, 6), cyclic: bool = False,
                     sync_frac: float = 0.4) -> Network:
    """A network whose liveness verdict is known by construction, with the
    monitor of :func:`add_liveness_monitor` for "process 0 takes a transition
    into local state 0 infinitely often".  Process 0 moves forward (s -> t > s)
    plus one closing edge back to 0; processes 1.. move forward only, locally or
    synchronising in pairs.  Every cycle then runs through process 0's closing
    edge: the property holds.  With `cyclic`, process 1 gets a backward edge,
    so a cycle avoiding process 0 exists: a violation (when reachable)."""
    rng = random.Random(seed)
    nst = [rng.randint(states[0], states[1]) for _ in range(nprocs)]
    net = _empty(nst)
    k = nst[0]
    for s in range(k - 1):
        for t in sorted(set(rng.sample(range(s + 1, k), min(2, k - 1 - s)))):
            _add_local(net, 0, s, t)
    _add_local(net, 0, k - 1, 0)
    others = list(range(1, nprocs))
    rules, acts_of = _sync_pool(rng, others, 2 * len(others), (2, 2))
    net.rules = rules
    for p in others:
        for s in range(nst[p] - 1):
            for _ in range(rng.randint(1, 2)):
                t = rng.randrange(s + 1, nst[p])
                if acts_of[p - 1] and rng.random() < sync_frac:
                    _add_sync(net, p, s, rng.choice(acts_of[p - 1]), t)
                else:
                    _add_local(net, p, s, t)
    if cyclic:
        _add_local(net, 1, nst[1] - 1, 0)
        _add_local(net, 1, 0, nst[1] - 1)
    _prune_unused_rules(net)
    return add_liveness_monitor(net, 0, 0)


def _sync_pool(rng: random.Random, procs: List[int], nactions: int,
               parties: Tuple[int, int], groups: Optional[List[List[int]]] = None,
               p_subrule: float = 0.25, single: float = 0.0) -> Tuple[Dict[int, List[int]], List[List[int]]]:
    """Create `nactions` synchronising actions over `procs`; return (rules, per-process action lists).
    With `single` > 0 an action is, with that probability, a one-party rule of
    a seeded process, and a multi-party action gets, with that probability, a
    one-party rule of one member beside its full rule."""
    rules: Dict[int, List[int]] = {}
    acts_of: Dict[int, List[int]] = {p: [] for p in procs}
    for a in range(nactions):
        pool = procs if groups is None else rng.choice(groups)
        if single and rng.random() < single:
            p = rng.choice(pool)
            rules[a] = [1 << p]
            acts_of[p].append(a)
            continue
        k = min(len(pool), rng.randint(parties[0], parties[1]))
        if k < 2:
            continue
        members = sorted(rng.sample(pool, k))
        mask = 0
        for p in members:
            mask |= 1 << p
        rs = [mask]
        if k >= 3 and rng.random() < p_subrule:
            sub = sorted(rng.sample(members, 2))
            rs.append((1 << sub[0]) | (1 << sub[1]))
        if single and rng.random() < single:
            rs.append(1 << rng.choice(members))
        rules[a] = rs
        for p in members:
            acts_of[p].append(a)
    return rules, [acts_of[p] for p in sorted(acts_of)]


def random_network(seed: int, nprocs: int = 16, states: Tuple[int, int] = (8, 32),
                   outdeg: Tuple[int, int] = (1, 4), sync_frac: float = 0.2,
                   parties: Tuple[int, int] = (2, 3), safety: bool = True,
                   nactions: Optional[int] = None, nstates: Optional[List[int]] = None,
                   single: float = 0.0) -> Network:
    """Random network: `nprocs` processes with U[states] local states (or exactly
    `nstates`), out-degree U[outdeg] per state, each transition synchronising with
    probability `sync_frac` (an action shared by 2-3 seeded processes), otherwise
    local.  With `safety`, a monitor over a seeded pair of error local states is
    appended (see :func:`add_safety_monitor`), giving nprocs+1 processes.
    `single` adds one-party synchronisation rules (see :func:`_sync_pool`)."""
    rng = random.Random(seed)
    nst = [rng.randint(states[0], states[1]) for _ in range(nprocs)]
    if nstates is not None:
        nst = list(nstates)
        nprocs = len(nst)
    net = _empty(nst)
    na = nactions if nactions is not None else 2 * nprocs
    rules, acts_of = _sync_pool(rng, list(range(nprocs)), na, parties, single=single)
    net.rules = rules
    err = None
    if safety:
        i, j = rng.sample(range(nprocs), 2)
        err = {i: rng.randrange(1, nst[i]), j: rng.randrange(1, nst[j])}
    for p in range(nprocs):
        for s in range(nst[p]):
            for _ in range(rng.randint(outdeg[0], outdeg[1])):
                t = rng.randrange(nst[p])
                crosses = err is not None and p in err and ((s == err[p]) != (t == err[p]))
                if acts_of[p] and rng.random() < sync_frac and not crosses:
                    _add_sync(net, p, s, rng.choice(acts_of[p]), t)
                else:
                    _add_local(net, p, s, t)
    _prune_unused_rules(net)
    if safety:
        (i, a), (j, b) = sorted(err.items())
        net = add_safety_monitor(net, i, a, j, b)
    return net


def corner_network(seed: int, nprocs: int = 8, states: Tuple[int, int] = (3, 6),
                   outdeg: Tuple[int, int] = (2, 5), sync_frac: float = 0.6, single: float = 0.3,
                   safety: bool = True) -> Network:
    """A random network outside the subset both reference kernels agree on:
    single-party synchronisation rules (alone, or beside a multi-party rule of
    the same action), and only about one action per process, so a state often
    has three or more targets for one action.  Encoded with gpf.encode's
    max_slots=1 those targets take one entry each (max_buf_ints >= 3, entries
    with empty slots); repeat_seed repeats targets."""
    return random_network(seed, nprocs=nprocs, states=states, outdeg=outdeg, sync_frac=sync_frac,
                          nactions=nprocs, single=single, safety=safety)


def clustered(seed: int, nprocs: int = 24, nclusters: Tuple[int, int] = (4, 6),
              states: Tuple[int, int] = (3, 6), outdeg: Tuple[int, int] = (1, 3),
              p_tau: float = 0.5, p_intra: float = 0.3) -> Network:
    """Processes in U[nclusters] seeded clusters: a transition is a local tau with
    probability p_tau, an intra-cluster synchronisation with probability p_intra and
    a cross-cluster synchronisation otherwise (the default mix is 80% inside the
    cluster, 20% across)."""
    rng = random.Random(seed)
    k = rng.randint(nclusters[0], nclusters[1])
    procs = list(range(nprocs))
    rng.shuffle(procs)
    groups = [sorted(procs[c::k]) for c in range(k)]
    cluster_of = {p: c for c, g in enumerate(groups) for p in g}
    nst = [rng.randint(states[0], states[1]) for _ in range(nprocs)]
    net = _empty(nst)
    intra_rules, intra_acts = _sync_pool(rng, list(range(nprocs)), 2 * nprocs, (2, 2),
                                         groups=[g for g in groups if len(g) >= 2], p_subrule=0.0)
    cross_rules: Dict[int, List[int]] = {}
    cross_acts: Dict[int, List[int]] = {p: [] for p in range(nprocs)}
    base = 2 * nprocs
    for a in range(nprocs):
        c1, c2 = rng.sample(range(k), 2)
        p1, p2 = rng.choice(groups[c1]), rng.choice(groups[c2])
        cross_rules[base + a] = [(1 << p1) | (1 << p2)]
        cross_acts[p1].append(base + a)
        cross_acts[p2].append(base + a)
    net.rules = dict(intra_rules)
    net.rules.update(cross_rules)
    for p in range(nprocs):
        for s in range(nst[p]):
            for _ in range(rng.randint(outdeg[0], outdeg[1])):
                t = rng.randrange(nst[p])
                x = rng.random()
                if x < p_tau or (x < p_tau + p_intra and not intra_acts[p]) or \
                        (x >= p_tau + p_intra and not cross_acts[p]):
                    _add_local(net, p, s, t)
                elif x < p_tau + p_intra:
                    _add_sync(net, p, s, rng.choice(intra_acts[p]), t)
                else:
                    _add_sync(net, p, s, rng.choice(cross_acts[p]), t)
    del cluster_of
    _prune_unused_rules(net)
    return net


def batch(seed: int, count: int = 512, procs: Tuple[int, int] = (4, 24),
          states: Tuple[int, int] = (4, 32), max_bits: int = 126) -> List[Network]:
    """`count` random networks of uneven sizes: per network a process count in
    `procs` and an upper bound on local states in `states`; networks whose state
    vector would exceed `max_bits` are redrawn with fewer states per process.
    Every network carries the safety monitor, so the same network can be checked
    for deadlocks or for the embedded safety property."""
    rng = random.Random(seed)
    nets = []
    for _ in range(count):
        n = rng.randint(procs[0], procs[1])
        hi = rng.randint(states[0], states[1])
        while True:
            net = random_network(rng.randrange(1 << 30), nprocs=n, states=(states[0], hi), outdeg=(1, 3))
            if net.firstbit()[-1] <= max_bits or hi <= states[0]:
                break
            hi = max(states[0], hi // 2)
        nets.append(net)
    return nets


def _prune_unused_rules(net: Network) -> None:
    used = set()
    for p in range(net.nprocs):
        for d in net.sync[p]:
            used.update(d)
    net.rules = {a: rs for a, rs in net.rules.items() if a in used}
    # compact action ids so bits_act stays small
    order = sorted(used | set(net.rules))
    remap = {a: i for i, a in enumerate(order)}
    net.rules = {remap[a]: rs for a, rs in net.rules.items()}
    for p in range(net.nprocs):
        net.sync[p] = [{remap[a]: ts for a, ts in d.items()} for d in net.sync[p]]
