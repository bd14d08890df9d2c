"""EXP/.aut -> gpf conversion against an independent product explorer that
reads the .aut files and synchronisation vectors directly."""
import os

import pytest

from gpuexplore_gb300 import exp2gpf
from helpers import oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "philosophers")
EXP = os.path.join(HERE, "philosophers.exp")


def product_explore(exp_path):
    """BFS over tuples of .aut states: internal actions and 1-party vectors move one
    LTS; a multi-party vector moves all its participants (EXP par-using semantics)."""
    vectors, names = exp2gpf.parse_exp(open(exp_path).read())
    auts = [exp2gpf.parse_aut(open(os.path.join(os.path.dirname(exp_path), n)).read()) for n in names]
    n = len(auts)
    out = [{} for _ in range(n)]
    for k, a in enumerate(auts):
        for s, lab, d in a.trans:
            out[k].setdefault(s, []).append((lab, d))
    init = tuple(a.initial for a in auts)
    seen, frontier, levels, dead = {init}, [init], [1], 0
    while frontier:
        nxt = []
        for st in frontier:
            succ = []
            for k in range(n):
                for lab, d in out[k].get(st[k], []):
                    if lab in exp2gpf.INTERNAL or any(v[k] == lab and sum(x is not None for x in v) == 1 for v in vectors):
                        t = list(st)
                        t[k] = d
                        succ.append(tuple(t))
            for v in vectors:
                parts = [k for k in range(n) if v[k] is not None]
                if len(parts) < 2:
                    continue
                choices = [[d for lab, d in out[k].get(st[k], []) if lab == v[k]] for k in parts]
                if all(choices):
                    import itertools
                    for combo in itertools.product(*choices):
                        t = list(st)
                        for k, d in zip(parts, combo):
                            t[k] = d
                        succ.append(tuple(t))
            if not succ:
                dead += 1
            for t in succ:
                if t not in seen:
                    seen.add(t)
                    nxt.append(t)
        if nxt:
            levels.append(len(nxt))
        frontier = nxt
    return len(seen), levels, dead


def test_philosophers_convert_and_explore(built, tmp_path):
    out = str(tmp_path / "phil.gpf")
    net = exp2gpf.convert(EXP, out)
    assert net.nprocs == 6
    states, levels, dead = product_explore(EXP)
    o = oracle(out, [])
    assert (o["states"], o["levels"]) == (states, levels)
    d = oracle(out, ["-d"])
    assert dead > 0 and d["verdict"] == "deadlock"


def test_aut_parsing_errors():
    with pytest.raises(ValueError):
        exp2gpf.parse_aut("des (0, 2, 2)\n(0, a, 1)\n")      # declares 2 transitions, has 1
    with pytest.raises(ValueError):
        exp2gpf.parse_aut("des (0, 1, 2)\n(0, a, 5)\n")      # state out of range
    with pytest.raises(ValueError):
        exp2gpf.parse_exp('par using "a" * _ -> "a" in "x.aut" end par')  # vector length


P_AUT = 'des (0, 3, 3)\n(0, "u", 1)\n(1, "w", 2)\n(2, i, 0)\n'
Q_AUT = 'des (0, 3, 3)\n(0, "a", 1)\n(1, "v", 2)\n(2, "v", 0)\n'
VEC = '"a" * "a" -> s, _ * "v" -> v'

# (EXP text, the test's own reading: per operand, a relabelling applied to its labels)
OPERAND_CASES = [
    (f'par using {VEC} in "p.aut" || "q.aut" end par', [{}, {}]),
    (f'par using {VEC} in rename "u" -> "a" in "p.aut" end rename || "q.aut" end par', [{"u": "a"}, {}]),
    (f'par using {VEC} in hide "w" in rename "u" -> "a" in "p.aut" end rename end hide || "q.aut" end par',
     [{"u": "a", "w": "i"}, {}]),
    (f'par using {VEC} in rename "u" -> "a" in hide all but "u" in "p.aut" end hide end rename || "q.aut" end par',
     [{"u": "a", "w": "i"}, {}]),
    (f'par using {VEC} in "p.aut" || hide "v" in "q.aut" end hide end par', [{}, {"v": "i"}]),
    # around the whole composition: relabels the composed transitions only
    (f'hide s, v in par using {VEC} in rename "u" -> "a" in "p.aut" end rename || "q.aut" end par end hide',
     [{"u": "a"}, {}]),
]


def _product(auts, vectors):
    """BFS over tuples of states, the EXP par-using semantics (as product_explore)."""
    import itertools
    n = len(auts)
    out = [{} for _ in range(n)]
    for k, a in enumerate(auts):
        for src, lab, dst in a.trans:
            out[k].setdefault(src, []).append((lab, dst))
    init = tuple(a.initial for a in auts)
    seen, frontier, levels = {init}, [init], [1]
    while frontier:
        nxt = []
        for st in frontier:
            succ = []
            for k in range(n):
                for lab, dst in out[k].get(st[k], []):
                    if lab in exp2gpf.INTERNAL or any(v[k] == lab and sum(x is not None for x in v) == 1 for v in vectors):
                        succ.append(st[:k] + (dst,) + st[k + 1:])
            for v in vectors:
                parts = [k for k in range(n) if v[k] is not None]
                if len(parts) < 2:
                    continue
                choices = [[dst for lab, dst in out[k].get(st[k], []) if lab == v[k]] for k in parts]
                for combo in itertools.product(*choices):
                    t = list(st)
                    for k, dst in zip(parts, combo):
                        t[k] = dst
                    succ.append(tuple(t))
            for t in succ:
                if t not in seen:
                    seen.add(t)
                    nxt.append(t)
        if nxt:
            levels.append(len(nxt))
        frontier = nxt
    return len(seen), levels


@pytest.mark.parametrize("case", range(len(OPERAND_CASES)))
def test_hide_and_rename_operands(built, tmp_path, case):
    """Operands under hide / rename, and wrappers around the whole composition:
    the converted network against a product explorer that applies the same
    relabellings by itself."""
    text, relabel = OPERAND_CASES[case]
    (tmp_path / "p.aut").write_text(P_AUT)
    (tmp_path / "q.aut").write_text(Q_AUT)
    (tmp_path / "n.exp").write_text(text)
    out = str(tmp_path / "n.gpf")
    exp2gpf.convert(str(tmp_path / "n.exp"), out)
    vectors = [["a", "a"], [None, "v"]]
    auts = []
    for raw, rl in zip((P_AUT, Q_AUT), relabel):
        a = exp2gpf.parse_aut(raw)
        a.trans = [(src, rl.get(lab, lab), dst) for src, lab, dst in a.trans]
        auts.append(a)
    states, levels = _product(auts, vectors)
    o = oracle(out, [])
    assert (o["states"], o["levels"]) == (states, levels), text


P3 = 'des (0, 2, 2)\n(0, "a", 1)\n(1, "u", 0)\n'
Q3 = 'des (0, 3, 3)\n(0, "a", 1)\n(1, "v", 2)\n(2, i, 0)\n'
R3 = 'des (0, 2, 2)\n(0, "b", 1)\n(1, "v", 0)\n'
INNER = 'par using "a" * "b" -> x, "v" * "v" -> {v} in "q.aut" || "r.aut" end par'
FLAT = 'par using {vecs} in "p.aut" || "q.aut" || "r.aut" end par'

# (a nested network, the same network written flat over p, q, r)
NESTED_CASES = [
    ('par using "a" * "x" -> s, "u" * _ -> u, _ * "v" -> w in "p.aut" || ' + INNER.format(v="v") + ' end par',
     FLAT.format(vecs='"a" * "a" * "b" -> s, "u" * _ * _ -> u, _ * "v" * "v" -> w')),
    # an inner vector with the internal result fires without an outer partner
    ('par using "a" * "x" -> s, "u" * _ -> u in "p.aut" || ' + INNER.format(v="i") + ' end par',
     FLAT.format(vecs='"a" * "a" * "b" -> s, "u" * _ * _ -> u, _ * "v" * "v" -> i')),
    # hiding an inner result: the inner move becomes internal, the outer vector on it never fires
    ('par using "a" * "x" -> s, "u" * _ -> u, _ * "v" -> w in "p.aut" || hide x in ' + INNER.format(v="v") +
     ' end hide end par',
     FLAT.format(vecs='"u" * _ * _ -> u, _ * "v" * "v" -> w, _ * "a" * "b" -> i')),
    # renaming an inner result
    ('par using "a" * "y" -> s, "u" * _ -> u, _ * "v" -> w in "p.aut" || rename x -> y in ' + INNER.format(v="v") +
     ' end rename end par',
     FLAT.format(vecs='"a" * "a" * "b" -> s, "u" * _ * _ -> u, _ * "v" * "v" -> w')),
]


@pytest.mark.parametrize("case", range(len(NESTED_CASES)))
def test_nested_par_equals_flat(built, tmp_path, case):
    """A par nested inside an operand is flattened onto its leaf LTSs: an outer
    vector element naming an inner result label stands for the inner vectors
    with that result.  Each nested network explores exactly like its flat form."""
    nested, flat = NESTED_CASES[case]
    for name, text in (("p.aut", P3), ("q.aut", Q3), ("r.aut", R3), ("nested.exp", nested), ("flat.exp", flat)):
        (tmp_path / name).write_text(text)
    exp2gpf.convert(str(tmp_path / "nested.exp"), str(tmp_path / "nested.gpf"))
    exp2gpf.convert(str(tmp_path / "flat.exp"), str(tmp_path / "flat.gpf"))
    a, b = oracle(str(tmp_path / "nested.gpf"), []), oracle(str(tmp_path / "flat.gpf"), [])
    assert (a["states"], a["levels"], a["set_hash"]) == (b["states"], b["levels"], b["set_hash"])
    vectors, _ = exp2gpf.parse_exp(flat)
    auts = [exp2gpf.parse_aut(t) for t in (P3, Q3, R3)]
    assert (a["states"], a["levels"]) == _product(auts, vectors)


def test_exp_syntax_errors():
    for bad in ('par using "a" * "a" in "p.aut" end par',             # two elements, one operand
                'par using "a" in "p.aut" || end par',                # missing operand
                'hide in "p.aut" end hide',                           # no label
                '"p.aut"'):                                           # no composition
        with pytest.raises(ValueError):
            exp2gpf.parse_exp(bad)


@pytest.mark.gpu
def test_philosophers_on_gpu(gpu, tmp_path):
    out = str(tmp_path / "phil.gpf")
    exp2gpf.convert(EXP, out)
    states, levels, dead = product_explore(EXP)
    r = gpu.explore(out, property="deadlock", q_words=1 << 20)
    assert r["verdict"] == "deadlock"
    r = gpu.explore(out, q_words=1 << 20)
    assert (r["states"], r["levels"]) == (states, levels)
