"""The gpuexplore command-line tool on a GPU: result lines, verdicts, --dump
and -v output against the oracle."""
import re
import subprocess

import numpy as np
import pytest

from gpuexplore_gb300 import gen
from helpers import oracle, write_net

pytestmark = pytest.mark.gpu


def _run(built, path, *args):
    base = path[:-4]
    out = subprocess.run([built.CLI, base] + list(args), capture_output=True, text=True, timeout=300)
    return out


def _count(stdout):
    return int(re.search(r"^nr\. of states in hash table: (\d+)$", stdout, re.M).group(1))


@pytest.mark.parametrize("flags,expect", [([], None), (["-d"], "deadlock"), (["-p"], "safety"),
                                          (["--por", "--cycle-proviso"], None),
                                          (["--stubborn", "-d"], "deadlock"), (["--ample", "-p"], "safety")])
def test_cli_matches_oracle(gpu, built, tmp_path, flags, expect):
    net = gen.random_network(16, nprocs=9, states=(3, 6), outdeg=(1, 2), sync_frac=0.7) if expect == "deadlock" \
        else gen.ring(2)
    path = write_net(net, tmp_path, "m")
    o = oracle(path, flags)
    r = _run(built, path, "-q", str(1 << 22), *flags)
    assert r.returncode == 0, r.stderr
    assert _count(r.stdout) == o["states"]
    assert ("deadlock detected!" in r.stdout) == (o["verdict"] == "deadlock")
    assert ("safety property violation detected!" in r.stdout) == (o["verdict"] == "safety")
    assert re.search(r"^Exploration time [0-9.]+$", r.stdout, re.M)
    assert re.search(r"^Run time: [0-9.]+$", r.stdout, re.M)


@pytest.mark.parametrize("prop", ["-d", "-p"])
def test_cli_no_prune(gpu, built, tmp_path, prop):
    """--no-prune (every successor looked up) prints the same result lines."""
    net = gen.random_network(16, nprocs=9, states=(3, 6), outdeg=(1, 2), sync_frac=0.7)
    path = write_net(net, tmp_path, "m")
    o = oracle(path, [prop])
    for extra in ([], ["--no-prune"]):
        r = _run(built, path, "-q", str(1 << 22), prop, *extra)
        assert r.returncode == 0, r.stderr
        assert _count(r.stdout) == o["states"]
        assert ("deadlock detected!" in r.stdout) == (o["verdict"] == "deadlock")
        assert ("safety property violation detected!" in r.stdout) == (o["verdict"] == "safety")


def test_cli_dump_is_the_visited_set(gpu, built, tmp_path):
    net = gen.random_network(31, nprocs=10, states=(3, 6))
    path = write_net(net, tmp_path, "m")
    dump = tmp_path / "space.txt"
    r = _run(built, path, "-q", str(1 << 22), "--dump", str(dump))
    assert r.returncode == 0 and "Dumping state space to file..." in r.stdout
    lines = dump.read_text().splitlines()
    assert re.match(r"nr\. of states in hash table: \d+ \(0 unexplored states\)", lines[-1])
    got = {tuple(int(x) for x in ln.split(" ")[0].split(",")) for ln in lines[:-1]}
    raw = tmp_path / "o.bin"
    o = oracle(path, [], dump=str(raw))
    words = np.fromfile(raw, dtype=np.uint32).reshape(-1, o["words"])
    fb = net.firstbit()
    want = set()
    for row in words:
        x = 0
        for j, w in enumerate(row):
            x |= int(w) << (32 * j)
        want.add(tuple((x >> fb[p]) & ((1 << (fb[p + 1] - fb[p])) - 1) for p in range(net.nprocs)))
    assert got == want and len(lines) - 1 == o["states"]


def test_cli_verbosity_and_relaunch(gpu, built, tmp_path):
    path = write_net(gen.ring(2), tmp_path, "m")
    o = oracle(path, [])
    r = _run(built, path, "-q", str(1 << 22), "-k", "2", "-v", "2")
    counts = [int(m) for m in re.findall(r"^nr\. of states in hash table: (\d+) \(", r.stdout, re.M)]
    # one line per launch of 2 levels; cumulative counts along the BFS levels
    cum = np.cumsum(o["levels"]).tolist()
    assert counts[-1] == o["states"] and len(counts) == (len(o["levels"]) + 1) // 2
    assert all(c in cum for c in counts)
    r1 = _run(built, path, "-q", str(1 << 22), "-k", "1", "-v", "1")
    seq = re.findall(r"^(\d+)$", r1.stdout, re.M)
    assert seq == [str(i) for i in range(len(seq))] and len(seq) >= len(o["levels"]) - 1
    r3 = _run(built, path, "-q", str(1 << 22), "-k", "100", "-v", "3")
    assert r3.stdout.count("\n") > o["states"]
