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

EXP operators     an operand of the composition may be wrapped in
                   ``hide L1, ... in <operand> end hide`` (those labels become the
                   internal action), ``hide all but L1, ... in ... end hide`` (every
                   other label does) or ``rename L1 -> M1, ... in ... end rename``;
                   the innermost wrapper applies first.  Hiding or renaming around
                   the whole ``par`` only relabels the composed transitions, which
                   leaves the state space and the verdicts unchanged, so such outer
                   wrappers are accepted as they are.  A ``par`` nested inside an
                   operand is not supported.

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


# an operand: (.aut file name, [(operator, argument)] innermost first)
Operand = Tuple[str, List[Tuple[str, object]]]


def _label_list(text: str) -> List[str]:
    labs = [x.strip() for x in text.split(",") if x.strip()]
    for x in labs:
        if not re.fullmatch(_LBL, x) or x == "_":
            raise ValueError(f"bad label {x!r}")
    return [x.strip('"') for x in labs]


def parse_operand(text: str) -> Operand:
    """An operand of the parallel composition: an .aut file name, possibly under
    hide / rename wrappers."""
    t = text.strip()
    m = re.fullmatch(r"hide\s+(all\s+but\s+)?(.*?)\s+in\s+(.*)\s+end\s+hide", t, flags=re.S)
    if m:
        name, ops = parse_operand(m.group(3))
        return name, ops + [("hide_all_but" if m.group(1) else "hide", _label_list(m.group(2)))]
    m = re.fullmatch(r"rename\s+(.*?)\s+in\s+(.*)\s+end\s+rename", t, flags=re.S)
    if m:
        pairs = {}
        for item in m.group(1).split(","):
            if not item.strip():
                continue
            if "->" not in item:
                raise ValueError(f"bad renaming {item!r}")
            a, b = (x.strip() for x in item.split("->", 1))
            (a,), (b,) = _label_list(a), _label_list(b)
            pairs[a] = b
        name, ops = parse_operand(m.group(2))
        return name, ops + [("rename", pairs)]
    if re.search(r"\b(par|hide|rename)\b", t):
        raise ValueError(f"unsupported operand {t!r} (a nested par, or a malformed hide / rename)")
    return t.strip('"'), []


def apply_ops(aut: Aut, ops: Sequence[Tuple[str, object]]) -> Aut:
    """The LTS with the operand's hide / rename wrappers applied, innermost first."""
    trans = list(aut.trans)
    for op, arg in ops:
        if op == "hide":
            trans = [(s, INTERNAL[0] if lab in arg else lab, d) for s, lab, d in trans]
        elif op == "hide_all_but":
            trans = [(s, lab if (lab in arg or lab in INTERNAL) else INTERNAL[0], d) for s, lab, d in trans]
        else:
            trans = [(s, arg.get(lab, lab), d) for s, lab, d in trans]
    return Aut(aut.initial, aut.nstates, trans)


def parse_exp(text: str) -> Tuple[List[List[Optional[str]]], List[str]]:
    """Return (vectors, lts file names) of a `par using ... in ... end par` expression."""
    vectors, ops = parse_exp_operands(text)
    return vectors, [name for name, _ in ops]


def parse_exp_operands(text: str) -> Tuple[List[List[Optional[str]]], List[Operand]]:
    """Return (vectors, operands) of a `par using ... in ... end par` expression."""
    body = re.sub(r"\(\*.*?\*\)", " ", text, flags=re.S)  # comments
    m = re.search(r"\bpar\s+using\b(.*?)\bin\b(.*?)\bend\s+par\b", body, flags=re.S)
    if not m:
        raise ValueError("expected: par using <vectors> in <lts> || ... end par")
    vec_text, lts_text = m.groups()
    operands = [parse_operand(x) for x in lts_text.split("||") if x.strip()]
    names = [name for name, _ in operands]
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
    return vectors, operands


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
        vectors, operands = parse_exp_operands(f.read())
    base = os.path.dirname(os.path.abspath(exp_path))
    auts = []
    for nm, ops in operands:
        with open(os.path.join(base, nm)) as f:
            auts.append(apply_ops(parse_aut(f.read()), ops))
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
