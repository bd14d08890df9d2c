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


@pytest.mark.gpu
def test_philosophers_on_gpu(gpu, tmp_path):
    out = str(tmp_path / "phil.gpf")
    exp2gpf.convert(EXP, out)
    states, levels, dead = product_explore(EXP)
    r = gpu.explore(out, property="deadlock", q_words=1 << 20)
    assert r["verdict"] == "deadlock"
    r = gpu.explore(out, q_words=1 << 20)
    assert (r["states"], r["levels"]) == (states, levels)
