"""Liveness on the GPU: the accepting-cycle check (One-Way-Catch-Them-Young over
the explored table) against the oracle's Tarjan check, for 32-, 64- and 128-bit
state vectors, violating and non-violating networks; and the paths that refuse
it (POR, the batch and no-allocation entry points) do so loudly."""
import subprocess

import pytest

from gpuexplore_gb300 import gen
from helpers import oracle, write_net

pytestmark = pytest.mark.gpu

CASES = {
    "random6": lambda: gen.liveness_network(3),                                               # 32-bit, violation
    "random18": lambda: gen.liveness_network(1, nprocs=18, states=(3, 4), outdeg=(1, 1), sync_frac=0.5),  # 64-bit
    "random30": lambda: gen.liveness_network(2, nprocs=30, states=(3, 4), outdeg=(1, 1), sync_frac=0.6),  # 128-bit
    "progress12": lambda: gen.progress_network(1, nprocs=12, states=(2, 3)),                  # 32-bit, holds
    "progress16": lambda: gen.progress_network(2, nprocs=16, states=(4, 5), sync_frac=0.9),   # 64-bit, holds
    "progress22": lambda: gen.progress_network(1, nprocs=22, states=(4, 5), sync_frac=0.9),   # 128-bit, holds
    "progress22c": lambda: gen.progress_network(1, nprocs=22, states=(4, 5), sync_frac=0.9, cyclic=True),
    "progress8c": lambda: gen.progress_network(4, nprocs=8, states=(3, 5), cyclic=True),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_liveness_matches_oracle(gpu, tmp_path, name):
    path = write_net(CASES[name](), tmp_path, name)
    o = oracle(path, ["-p"])
    for graph in (1, 0):
        g = gpu.explore(path, check=False, property="safety", cycle_proviso=1, q_words=1 << 22, launch_graph=graph)
        assert g["rc"] == 0, g
        assert g["states"] == o["states"] and g["levels"] == o["levels"] and g["set_hash"] == o["set_hash"]
        assert g["verdict"] == o["verdict"] and g["stopped"] == o["stopped"]
        assert (g["live_states"] > 0) == (o["verdict"] == "liveness")
        assert g["live_ms"] > 0


@pytest.mark.parametrize("name", ["random30", "progress22c"])
def test_liveness_on_a_full_table(gpu, tmp_path, name):
    """A table barely larger than the state space: level-close eviction moves
    keys along their probe sequences, and the check still finds every
    successor's slot; replays reuse the table by generation."""
    path = write_net(CASES[name](), tmp_path, name)
    o = oracle(path, ["-p"])
    q_words = (int(o["states"] * 1.08) * 16) // 4
    ex = gpu.Explorer(gpu.Model.from_file(path), gpu.options(property="safety", cycle_proviso=1, q_words=q_words,
                                                             store_states=o["states"] + 64))
    try:
        for _ in range(2):
            g = ex.run(check=False)
            assert g["rc"] == 0, g
            assert g["states"] == o["states"] and g["set_hash"] == o["set_hash"]
            assert g["verdict"] == o["verdict"] and (g["live_states"] > 0) == (o["verdict"] == "liveness")
    finally:
        ex.close()


def test_liveness_replay_and_model_switch(gpu, tmp_path):
    """One explorer, alternating violating and non-violating models."""
    nets = [gen.progress_network(5, cyclic=True), gen.progress_network(5), gen.progress_network(6, cyclic=True)]
    paths = [write_net(n, tmp_path, f"m{i}") for i, n in enumerate(nets)]
    refs = [oracle(p, ["-p"]) for p in paths]
    models = [gpu.Model.from_file(p) for p in paths]
    ex = gpu.Explorer(models[0], gpu.options(property="safety", cycle_proviso=1, q_words=1 << 20))
    try:
        for _ in range(2):
            for m, ref in zip(models, refs):
                ex.set_model(m)
                r = ex.run(check=False)
                assert r["verdict"] == ref["verdict"] and r["states"] == ref["states"]
    finally:
        ex.close()


def test_liveness_budget_is_inconclusive(gpu, tmp_path):
    """A run stopped by the state budget has not seen every cycle: no verdict."""
    path = write_net(gen.progress_network(1, nprocs=12, states=(2, 3), cyclic=True), tmp_path, "b")
    g = gpu.explore(path, check=False, property="safety", cycle_proviso=1, q_words=1 << 20, max_states=100)
    assert g["rc"] == 0 and g["stopped"] == "budget" and g["verdict"] == "none" and g["live_states"] == 0


def test_liveness_refused_where_unsupported(gpu, tmp_path):
    path = write_net(gen.progress_network(2, cyclic=True), tmp_path, "u")
    # with POR the reduced graph is not the state graph the check needs
    g = gpu.explore(path, check=False, property="safety", por=1, cycle_proviso=1, q_words=1 << 20)
    assert g["rc"] == gpu.GPX_ERR_UNSUPPORTED
    m = gpu.Model.from_file(path)
    n = gpu.explore_noalloc(m, check=False, property="safety", q_words=1 << 18, store_states=1 << 14)
    assert n["rc"] == gpu.GPX_ERR_UNSUPPORTED
    items, _ = gpu.batch_explore([m], [{"property": "safety"}], check=False)
    assert items[0]["status"] == gpu.GPX_ERR_UNSUPPORTED


def test_cli_reports_liveness_violation(gpu, built, tmp_path):
    path = write_net(gen.progress_network(3, cyclic=True), tmp_path, "cli")
    out = subprocess.run([built.CLI, path[:-4], "-p", "-q", str(1 << 20)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert "Property to check is a liveness property" in out.stdout
    assert "liveness property violation detected!" in out.stdout
    ok = write_net(gen.progress_network(3), tmp_path, "ok")
    out = subprocess.run([built.CLI, ok[:-4], "-p", "-q", str(1 << 20)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and "violation" not in out.stdout
