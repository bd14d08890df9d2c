"""Batched exploration (many networks, one persistent launch) against the
oracle, instance by instance."""
import random

import pytest

from gpuexplore_gb300 import gen
from helpers import FLAGS, oracle, write_net

pytestmark = pytest.mark.gpu

FLAGSET = ["plain", "deadlock", "safety", "por", "por_proviso", "por_safety", "ample_safety", "stubborn_deadlock",
           "stubborn_safety"]


def _batch_cases(n, seed):
    rng = random.Random(seed)
    cases = []
    for k in range(n):
        fam = rng.choice(["ring", "rand", "rand", "clus"])
        if fam == "ring":
            net = gen.ring(rng.randrange(100))
        elif fam == "rand":
            net = gen.random_network(rng.randrange(1000), nprocs=rng.randint(4, 14), states=(3, rng.randint(4, 9)),
                                     outdeg=(1, rng.randint(2, 3)))
        else:
            net = gen.clustered(rng.randrange(1000), nprocs=rng.randint(6, 16), nclusters=(2, 4))
        fs = rng.choice(FLAGSET)
        budget = rng.choice([0, 2000, 50_000])
        cases.append((net, fs, budget))
    return cases


def _check(lib, tmp_path, cases, **opts):
    models, jobs, want = [], [], []
    for k, (net, fs, budget) in enumerate(cases):
        path = write_net(net, tmp_path, f"b{k}")
        cli, kw = FLAGS[fs]
        job = {"property": kw.get("property", "none"), "por": kw.get("por", 0),
               "cycle_proviso": kw.get("cycle_proviso", 0), "max_states": budget or 400_000}
        want.append(oracle(path, cli, max_states=job["max_states"]))
        models.append(lib.Model.from_file(path))
        jobs.append(job)
    items, stats = lib.batch_explore(models, jobs, level_capacity=4096, **opts)
    for k, (it, w) in enumerate(zip(items, want)):
        assert it["status"] == 0, (k, it)
        bits = cases[k][0].firstbit()[-1]  # narrow slots: the narrowest slot its vector fits; else 128-bit
        narrow = 4 if bits <= 31 else (8 if bits <= 63 else 16)
        assert it["slot_bytes"] == (narrow if stats["narrow_slots"] else 16), (k, bits)  # the policy that ran
        assert it["nlevels"] == len(w["levels"]), k
        for key in ("states", "levels", "verdict", "stopped", "set_hash"):
            assert it[key] == w[key], (k, cases[k][1], key, it[key], w[key])
    assert stats["states"] == sum(w["states"] for w in want)
    return items, stats


@pytest.mark.parametrize("narrow_slots", [0, 1])
def test_batch_matches_oracle(gpu, tmp_path, narrow_slots):
    _check(gpu, tmp_path, _batch_cases(40, 1), narrow_slots=narrow_slots)


def test_batch_readmission(gpu, tmp_path):
    """Partitions admitted too small overflow and are re-admitted with 4x capacity."""
    cases = _batch_cases(12, 2)
    lib = gpu
    models = []
    for k, (net, fs, budget) in enumerate(cases):
        models.append(lib.Model.from_file(write_net(net, tmp_path, f"r{k}")))
    jobs = [{"max_states": 20_000, "capacity": 64} for _ in cases]
    items, stats = lib.batch_explore(models, jobs, max_admissions=6)
    for k, it in enumerate(items):
        w = oracle(str(tmp_path / f"r{k}.gpf"), [], max_states=20_000)
        assert it["status"] == 0 and it["states"] == w["states"] and it["set_hash"] == w["set_hash"]
    assert max(it["admissions"] for it in items) > 1


def test_batch_launch_shapes_and_autotune(gpu, tmp_path):
    cases = _batch_cases(16, 3)
    _check(gpu, tmp_path, cases, claim=32, threads=128, kernel_iters=8)
    # 8 warps with a budget of 2 claims per launch: the captured loop relaunches on the device
    items, stats = _check(gpu, tmp_path, cases, claim=8, threads=64, blocks=4, kernel_iters=2)
    assert stats["launches"] > 10
    items, stats = _check(gpu, tmp_path, cases, autotune=1)
    assert stats["kernel_iters"] in (0, 64, 512) and stats["narrow_slots"] in (0, 1)
    assert stats["claim"] in (4, 8, 16, 32, 64, 256) and stats["tune_ms"] > 0
    assert stats["p99_ms"] >= stats["p50_ms"] > 0


def test_batch_autotune_whole_batch_stage(gpu, tmp_path):
    """A batch larger than the autotuner's 64-instance sample: after the sample
    stages the claim size is chosen again on the whole batch (the sample's
    choice, twice and four times it).  Every instance equals the oracle."""
    cases = _batch_cases(72, 13)
    items, stats = _check(gpu, tmp_path, cases, autotune=1)
    assert stats["tune_ms"] > 0
    assert stats["claim"] in (4, 8, 16, 32, 64, 128, 256, 512, 1024)


def test_batch_pruning_on_and_off(gpu, tmp_path):
    """Plain instances prune commuting moves by default (the label array is the
    per-state array cycle-proviso instances use for clusters); with pruning off
    every successor is looked up.  Both equal the oracle."""
    cases = [c for c in _batch_cases(40, 5) if c[1] in ("plain", "deadlock", "safety")][:12]
    assert len(cases) >= 6
    _check(gpu, tmp_path, cases)
    _check(gpu, tmp_path, cases, prune_commuting=0)


def test_batch_eviction_instead_of_readmission(gpu, tmp_path):
    """Partitions at a 0.95 load factor: inserts whose probe sequence is full are
    placed with eviction by the warp that closes the level, so the instances
    finish in their first admission with results equal to the oracle's."""
    cases = []
    for k in range(6):
        net = gen.random_network(300 + k, nprocs=20, states=(3, 5), outdeg=(1, 2), safety=False)
        cases.append((net, ["plain", "deadlock", "por_proviso"][k % 3], 0))
    models, jobs, want = [], [], []
    for k, (net, fs, _) in enumerate(cases):
        path = write_net(net, tmp_path, f"e{k}")
        cli, kw = FLAGS[fs]
        w = oracle(path, cli, max_states=60_000)
        want.append(w)
        jobs.append({"property": kw.get("property", "none"), "por": kw.get("por", 0),
                     "cycle_proviso": kw.get("cycle_proviso", 0), "max_states": 60_000,
                     "capacity": w["states"] + 16})
        models.append(gpu.Model.from_file(path))
    items, stats = gpu.batch_explore(models, jobs, level_capacity=4096, load_factor=0.95)
    for k, (it, w) in enumerate(zip(items, want)):
        assert it["status"] == 0 and it["admissions"] == 1, (k, it)
        for key in ("states", "levels", "verdict", "stopped", "set_hash"):
            assert it[key] == w[key], (k, key)


def test_batch_eviction_narrow_slots(gpu, tmp_path):
    """The closing warp's placement on 32- and 64-bit slots (narrow_slots) at a
    0.95 load factor: first admission, oracle results."""
    cases = []
    for k, (seed, n) in enumerate(((50, 10), (53, 10), (45, 11), (43, 14))):  # 21K-78K states each
        net = gen.random_network(seed, nprocs=n, states=(3, 6), outdeg=(1, 2), safety=False)
        cases.append((net, ["plain", "deadlock"][k % 2], 0))
    models, jobs, want = [], [], []
    for k, (net, fs, _) in enumerate(cases):
        path = write_net(net, tmp_path, f"n{k}")
        cli, kw = FLAGS[fs]
        w = oracle(path, cli, max_states=100_000)
        want.append(w)
        jobs.append({"property": kw.get("property", "none"), "max_states": 100_000, "capacity": w["states"] + 16})
        models.append(gpu.Model.from_file(path))
    items, stats = gpu.batch_explore(models, jobs, level_capacity=4096, load_factor=0.95, narrow_slots=1)
    assert stats["narrow_slots"] == 1 and set(it["slot_bytes"] for it in items) <= {4, 8}
    for k, (it, w) in enumerate(zip(items, want)):
        assert it["status"] == 0 and it["admissions"] == 1, (k, it)
        for key in ("states", "levels", "verdict", "stopped", "set_hash"):
            assert it[key] == w[key], (k, key)
