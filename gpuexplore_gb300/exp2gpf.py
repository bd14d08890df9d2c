"""Convert a network of LTSs -- Aldebaran `.aut` files composed by an EXP
`par using <synchronisation vectors> in <LTS> || ... end par` expression -- to
the gpf format, so models written for CADP-style tools can be explored.

The reference names a converter (GPUnetltsgen.py, README.md:22) that is not in
its tree; this one is written from the formats themselves:

.aut (Aldebaran)   first line ``des (initial, nr_transitions, nr_states)``, then one
                   transition per line ``(from, "label", to)`` (the label may be
                   unquoted; ``i`` / ``tau`` is the internal action).
EXP sync vectors   ``"a" * "b" * _ -> "c"``: one label (or ``_`` = does not take
                   part) per LTS in the order of the ``||`` list; the result label
                   after ``->`` is informational.  Only vectors fire: an LTS
                   transition whose label is in no vector for that LTS is blocked,
                   except the internal action, which stays local.

Mapping to gpf: a vector with one participant turns that LTS's transitions on
its label into local transitions; a vector with two or more participants
becomes one synchronising action whose single rule is the participant set, and
every participant's transitions on its vector label become entries of that
action.  States are relabelled so that each LTS's initial state is 0 (gpf
explores from the all-zero vector).
"""
from __future__ import annotations

import os
import re
import sys
from typing import Dict, List, Optional, Sequence, Tuple

from .gpf import Network, write

INTERNAL = ("i", "tau")


class Aut:
    def __init__(self, initial: int, nstates: int, trans: List[Tuple[int, str, int]]):
        self.initial, self.nstates, self.trans = initial, nstates, trans


_DES = re.compile(r"^\s*des\s*\(\s*(\d+)\s*,\s*(\d+)\s*,\s*(\d+)\s*\)\s*$")
_TR = re.compile(r'^\s*\(\s*(\d+)\s*,\s*("(?:[^"\\]|\\.)*"|[^,]+?)\s*,\s*(\d+)\s*\)\s*$')


def parse_aut(text: str) -> Aut:
    lines = [ln for ln in text.splitlines() if ln.strip()]
    if not lines:
        raise ValueError("empty .aut")
    m = _DES.match(lines[0])
    if not m:
        raise ValueError(f"bad .aut header: {lines[0]!r}")
    initial, ntr, nst = map(int, m.groups())
    trans = []
    for ln in lines[1:]:
        t = _TR.match(ln)
        if not t:
            raise ValueError(f"bad .aut transition: {ln!r}")
        src, lab, dst = t.groups()
        lab = lab.strip()
        if lab.startswith('"') and lab.endswith('"'):
            lab = lab[1:-1]
        trans.append((int(src), lab, int(dst)))
    if len(trans) != ntr:
        raise ValueError(f".aut declares {ntr} transitions, has {len(trans)}")
    for s, _, d in trans:
        if not (0 <= s < nst and 0 <= d < nst):
            raise ValueError("transition state out of range")
    return Aut(initial, nst, trans)


_LBL = r'"(?:[^"\\]|\\.)*"|_|[A-Za-z0-9_.!?:-]+'


def parse_exp(text: str) -> Tuple[List[List[Optional[str]]], List[str]]:
    """Return (vectors, lts file names) of a `par using ... in ... end par` expression."""
    body = re.sub(r"\(\*.*?\*\)", " ", text, flags=re.S)  # comments
    m = re.search(r"\bpar\s+using\b(.*?)\bin\b(.*?)\bend\s+par\b", body, flags=re.S)
    if not m:
        raise ValueError("expected: par using <vectors> in <lts> || ... end par")
    vec_text, lts_text = m.groups()
    names = [re.sub(r'^"|"$', "", x.strip()) for x in lts_text.split("||")]
    names = [n for n in names if n]
    vectors: List[List[Optional[str]]] = []
    for item in re.split(r",(?=(?:[^\"]*\"[^\"]*\")*[^\"]*$)", vec_text):
        item = item.strip()
        if not item:
            continue
        left = item.split("->")[0]
        parts = [p.strip() for p in left.split("*")]
        vec = []
        for p in parts:
            if not re.fullmatch(_LBL, p):
                raise ValueError(f"bad vector element {p!r}")
            vec.append(None if p == "_" else p.strip('"'))
        if len(vec) != len(names):
            raise ValueError(f"vector {item!r} has {len(vec)} elements for {len(names)} LTSs")
        vectors.append(vec)
    return vectors, names


def to_network(auts: Sequence[Aut], vectors: Sequence[Sequence[Optional[str]]]) -> Network:
    n = len(auts)
    # relabel so each initial state is 0
    relabel = []
    for a in auts:
        perm = list(range(a.nstates))
        perm[0], perm[a.initial] = perm[a.initial], perm[0]
        relabel.append(perm)
    local = [[[] for _ in range(a.nstates)] for a in auts]
    sync: List[List[Dict[int, List[int]]]] = [[{} for _ in range(a.nstates)] for a in auts]
    rules: Dict[int, List[int]] = {}
    local_labels = [set(INTERNAL) for _ in range(n)]
    multi = []
    for vec in vectors:
        parts = [k for k in range(n) if vec[k] is not None]
        if len(parts) == 1:
            local_labels[parts[0]].add(vec[parts[0]])
        elif len(parts) >= 2:
            multi.append(vec)
    for k, a in enumerate(auts):
        for s, lab, d in a.trans:
            if lab in local_labels[k]:
                ts = local[k][relabel[k][s]]
                if relabel[k][d] not in ts:
                    ts.append(relabel[k][d])
    for act, vec in enumerate(multi):
        mask = 0
        for k in range(n):
            if vec[k] is None:
                continue
            mask |= 1 << k
            for s, lab, d in auts[k].trans:
                if lab == vec[k]:
                    ts = sync[k][relabel[k][s]].setdefault(act, [])
                    if relabel[k][d] not in ts:
                        ts.append(relabel[k][d])
        rules[act] = [mask]
    return Network(nstates=[a.nstates for a in auts], local=local, sync=sync, rules=rules)


def convert(exp_path: str, out_path: str) -> Network:
    with open(exp_path) as f:
        vectors, names = parse_exp(f.read())
    base = os.path.dirname(os.path.abspath(exp_path))
    auts = []
    for nm in names:
        with open(os.path.join(base, nm)) as f:
            auts.append(parse_aut(f.read()))
    net = to_network(auts, vectors)
    write(net, out_path)
    return net


def main(argv: Sequence[str]) -> int:
    if len(argv) != 3:
        print("usage: python -m gpuexplore_gb300.exp2gpf <network.exp> <out.gpf>", file=sys.stderr)
        return 1
    net = convert(argv[1], argv[2])
    print(f"{argv[2]}: {net.nprocs} LTSs, state vector of {net.firstbit()[-1]} bits")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
