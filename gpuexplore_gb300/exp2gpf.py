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
                   operand is flattened onto its leaf LTSs: an outer vector element
                   naming an inner result label (``-> b``) stands for every inner
                   vector with that result; inner vectors whose result is internal
                   fire without outer partners.

Mapping to gpf: a vector with one participant turns that LTS's transitions on
its label into local transitions; a vector with two or more participants
becomes one synchronising action whose single rule is the participant set, and
every participant's transitions on its vector label become entries of that
action.  States are relabelled so that each LTS's initial state is 0 (gpf
explores from the all-zero vector).
"""
from __future__ import annotations

import itertools
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

_TOKEN = re.compile(r'\s*(\|\||->|\*|,|"(?:[^"\\]|\\.)*"|[A-Za-z0-9_.!?:-]+)')
_KEYWORDS = {"par", "using", "in", "end", "hide", "all", "but", "rename"}


def _tokens(text: str) -> List[str]:
    body = re.sub(r"\(\*.*?\*\)", " ", text, flags=re.S)  # comments
    out, pos = [], 0
    while pos < len(body):
        if body[pos:].strip() == "":
            break
        m = _TOKEN.match(body, pos)
        if not m:
            raise ValueError(f"unexpected text near {body[pos:pos + 20]!r}")
        out.append(m.group(1))
        pos = m.end()
    return out


class _Parser:
    """Recursive descent over the EXP subset: par using / hide / rename / .aut leaves."""

    def __init__(self, text: str):
        self.t, self.k = _tokens(text), 0

    def peek(self, off: int = 0) -> Optional[str]:
        return self.t[self.k + off] if self.k + off < len(self.t) else None

    def take(self, want: Optional[str] = None) -> str:
        tok = self.peek()
        if tok is None or (want is not None and tok != want):
            raise ValueError(f"expected {want or 'more input'}, found {tok!r}")
        self.k += 1
        return tok

    def label(self) -> str:
        tok = self.take()
        if tok in _KEYWORDS or tok in ("||", "->", "*", ",", "_"):
            raise ValueError(f"expected a label, found {tok!r}")
        return tok.strip('"')

    def labels(self) -> List[str]:
        out = [self.label()]
        while self.peek() == ",":
            self.take(",")
            out.append(self.label())
        return out

    def expr(self):
        tok = self.peek()
        if tok == "par":
            self.take("par")
            self.take("using")
            vectors = [self.vector()]
            while self.peek() == ",":
                self.take(",")
                vectors.append(self.vector())
            self.take("in")
            ops = [self.expr()]
            while self.peek() == "||":
                self.take("||")
                ops.append(self.expr())
            self.take("end")
            self.take("par")
            for elems, _ in vectors:
                if len(elems) != len(ops):
                    raise ValueError(f"a vector has {len(elems)} elements for {len(ops)} operands")
            return ("par", vectors, ops)
        if tok == "hide":
            self.take("hide")
            all_but = self.peek() == "all" and self.peek(1) == "but"
            if all_but:
                self.take("all")
                self.take("but")
            labs = self.labels()
            self.take("in")
            e = self.expr()
            self.take("end")
            self.take("hide")
            return ("hide_all_but" if all_but else "hide", labs, e)
        if tok == "rename":
            self.take("rename")
            pairs = {}
            while True:
                a = self.label()
                self.take("->")
                pairs[a] = self.label()
                if self.peek() != ",":
                    break
                self.take(",")
            self.take("in")
            e = self.expr()
            self.take("end")
            self.take("rename")
            return ("rename", pairs, e)
        return ("leaf", self.label())

    def vector(self):
        elems = [self.elem()]
        while self.peek() == "*":
            self.take("*")
            elems.append(self.elem())
        result = None
        if self.peek() == "->":
            self.take("->")
            result = self.label()
        return elems, result

    def elem(self) -> Optional[str]:
        if self.peek() == "_":
            self.take("_")
            return None
        return self.label()


def _relabel(lab: str, op: str, arg) -> str:
    if lab in INTERNAL:
        return lab
    if op == "hide":
        return INTERNAL[0] if lab in arg else lab
    if op == "hide_all_but":
        return lab if lab in arg else INTERNAL[0]
    return arg.get(lab, lab)


def _flatten(node, ops=()):
    """(leaves, moves) of an expression: leaves are (file, wrappers) operands;
    moves are None for a leaf (it offers its own labels), else the composite's
    transitions as (one label or None per leaf, result label).  Wrappers on a
    composite act on its result labels; on a leaf they are applied to its LTS."""
    kind = node[0]
    if kind == "leaf":  # `ops` lists the wrappers outermost first; a leaf applies the innermost first
        return [(node[1], list(reversed(ops)))], None
    if kind in ("hide", "hide_all_but", "rename"):
        leaves, moves = _flatten(node[2], ops + ((kind, node[1]),))
        if moves is None:
            return leaves, None
        return leaves, [(el, _relabel(r, kind, node[1])) for el, r in moves]
    _, vectors, operands = node
    parts = [_flatten(o) for o in operands]
    offs, n = [], 0
    for leaves, _ in parts:
        offs.append(n)
        n += len(leaves)
    leaves_all = [lf for leaves, _ in parts for lf in leaves]
    moves: List[Tuple[List[Optional[str]], str]] = []
    for elems, result in vectors:
        options = []
        for i, e in enumerate(elems):
            if e is None:
                continue
            leaves, sub = parts[i]
            if sub is None:
                options.append([{offs[i]: e}])
            else:  # a composite operand: any of its moves with that result label
                options.append([{offs[i] + k: x for k, x in enumerate(el) if x is not None} for el, r in sub if r == e])
        if not options:
            continue
        present = [e for e in elems if e is not None]
        res = result if result is not None else (present[0] if len(set(present)) == 1 else "_".join(present))
        for combo in itertools.product(*options):
            vec: List[Optional[str]] = [None] * n
            for part in combo:
                for k, x in part.items():
                    vec[k] = x
            moves.append((vec, res))
    for i, (leaves, sub) in enumerate(parts):  # an operand's internal moves need no partner
        if sub is None:
            continue
        for el, r in sub:
            if r in INTERNAL:
                vec = [None] * n
                for k, x in enumerate(el):
                    vec[offs[i] + k] = x
                moves.append((vec, r))
    return leaves_all, moves


def parse_operand(text: str) -> Operand:
    """One .aut operand, possibly under hide / rename wrappers."""
    leaves, moves = _flatten(_Parser(text).expr())
    if moves is not None or len(leaves) != 1:
        raise ValueError("expected a single .aut operand")
    return leaves[0]


def apply_ops(aut: Aut, ops: Sequence[Tuple[str, object]]) -> Aut:
    """The LTS with the operand's hide / rename wrappers applied, innermost first."""
    trans = list(aut.trans)
    for op, arg in ops:
        trans = [(s, _relabel(lab, op, arg), d) for s, lab, d in trans]
    return Aut(aut.initial, aut.nstates, trans)


def parse_exp(text: str) -> Tuple[List[List[Optional[str]]], List[str]]:
    """Return (vectors, lts file names) of an EXP network."""
    vectors, ops = parse_exp_operands(text)
    return vectors, [name for name, _ in ops]


def parse_exp_operands(text: str) -> Tuple[List[List[Optional[str]]], List[Operand]]:
    """Return (vectors over the leaf LTSs, leaf operands) of an EXP network:
    nested compositions are flattened -- an outer vector element naming an inner
    result label stands for every inner vector with that result -- and inner
    vectors whose result is internal fire without outer partners."""
    p = _Parser(text)
    root = p.expr()
    if p.peek() is not None:
        raise ValueError(f"unexpected {p.peek()!r} after the expression")
    leaves, moves = _flatten(root)
    if moves is None:
        raise ValueError("expected: par using <vectors> in <operand> || ... end par")
    return [el for el, _ in moves], leaves


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
