"""The CPU oracle, pinned against hand-derived answers and the independent
abstract explorer (CPU only)."""
import json
import os
import subprocess

import pytest

from gpuexplore_gb300 import gen, gpf
import abstract_explorer as ax
from helpers import oracle, write_net

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def _write_words(words, tmp_path, name):
    p = tmp_path / (name + ".gpf")
    p.write_text("\n".join(str(w) for w in words) + "\n")
    return str(p)


@pytest.mark.parametrize("threads", [1, 3])
def test_known_answers(built, tmp_path, threads):
    for case in _load("known_answers.json"):
        path = _write_words(case["gpf"], tmp_path, case["name"])
        for fs, e in case["expect"].items():
            o = oracle(path, e["flags"], threads=threads)
            assert (o["states"], o["levels"], o["verdict"], o["stopped"]) == \
                (e["states"], e["levels"], e["verdict"], e["stopped"]), (case["name"], fs)


@pytest.mark.parametrize("threads", [1, 4])
def test_generated_fixtures(built, tmp_path, threads):
    for i, case in enumerate(_load("generated.json")):
        path = _write_words(case["gpf"], tmp_path, f"g{i}")
        for fs, e in case["expect"].items():
            o = oracle(path, e["flags"], threads=threads)
            for k in ("states", "levels", "verdict", "stopped", "set_hash"):
                assert o[k] == e[k], (case["family"], case["seed"], fs, k)


@pytest.mark.parametrize("seed", range(10, 16))
def test_against_abstract_explorer(built, tmp_path, seed):
    flags = {(): {}, ("-d",): {"prop": "deadlock"}, ("-p",): {"prop": "safety", "proviso": True},
             ("--por",): {"por": True}, ("--por", "--cycle-proviso"): {"por": True, "proviso": True}}
    for k, net in enumerate((gen.ring(seed, nprocs=5, nstates=4),
                             gen.random_network(seed, nprocs=6, states=(3, 5)),
                             gen.clustered(seed, nprocs=8, nclusters=(2, 3), states=(2, 4), outdeg=(1, 2)))):
        path = write_net(net, tmp_path, f"m{k}")
        for fl, kw in flags.items():
            a = ax.explore(net, **kw)
            o = oracle(path, list(fl), threads=2)
            assert o["states"] == a["states"] and o["levels"] == a["levels"]
            assert o["verdict"] == a["verdict"] and o["set_hash"] == ax.set_hash(net, a["visited"])


def test_thread_count_invariance(built, tmp_path):
    path = write_net(gen.random_network(2024, nprocs=10, states=(4, 10)), tmp_path, "c2small")
    ref = oracle(path, ["-d"], threads=1, max_states=200_000)
    for t in (2, 5, 8):
        o = oracle(path, ["-d"], threads=t, max_states=200_000)
        assert (o["states"], o["levels"], o["set_hash"]) == (ref["states"], ref["levels"], ref["set_hash"])
    assert ref["stopped"] == "budget" and ref["states"] >= 200_000


def test_budget_is_level_aligned(built, tmp_path):
    path = write_net(gen.ring(2), tmp_path, "ring")
    full = oracle(path, [])
    for budget in (1, 10, 1000, 20000):
        o = oracle(path, [], max_states=budget)
        L = len(o["levels"])
        assert o["levels"] == full["levels"][:L]
        assert o["states"] >= budget or o["stopped"] == "done"
        assert L <= 2 or sum(o["levels"][:-1]) < budget  # checked after each expansion


def test_flag_semantics(built, tmp_path):
    """-d turns the cycle proviso off; -p turns it on; --cycle-proviso counts only before -d/-p."""
    path = write_net(gen.random_network(12, nprocs=8, states=(3, 6)), tmp_path, "f")
    prov = oracle(path, ["--por", "--cycle-proviso"])
    nopr = oracle(path, ["--por"])
    assert prov["states"] != nopr["states"]
    assert oracle(path, ["--por", "--cycle-proviso", "-d"])["levels"] == nopr["levels"]
    assert oracle(path, ["--por", "-d", "--cycle-proviso"])["levels"] == nopr["levels"]
    assert oracle(path, ["--por", "-p"])["set_hash"] == oracle(path, ["--por", "--cycle-proviso", "-p"])["set_hash"]


def test_oracle_errors(built, tmp_path):
    from gpuexplore_gb300.build import ORACLE
    r = subprocess.run([ORACLE, str(tmp_path / "missing")], capture_output=True, text=True)
    assert r.returncode == 1 and "input network does not exist" in r.stderr
    r = subprocess.run([ORACLE, str(tmp_path / "missing"), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "unrecognized option --bogus" in r.stderr
    bad = tmp_path / "bad.gpf"
    bad.write_text("0\n3\n")
    r = subprocess.run([ORACLE, str(bad)], capture_output=True, text=True)
    assert r.returncode == 1


def test_dump_is_bfs_order(built, tmp_path):
    import numpy as np
    net = gen.ring(4)
    path = write_net(net, tmp_path, "r")
    dump = str(tmp_path / "s.bin")
    o = oracle(path, [], dump=dump)
    rows = np.fromfile(dump, dtype=np.uint32).reshape(-1, o["words"])
    assert rows.shape[0] == o["states"] and rows[0].sum() == 0
    assert len({tuple(r) for r in rows}) == o["states"]
    a = ax.explore(net)
    assert {tuple(ax.pack(net, s)) for s in a["visited"]} == {tuple(int(x) for x in r) for r in rows}
