"""Failure detection without a GPU fault: bounded device waits end with a
status, and table/store overflow are reported statuses; the context stays
usable after each."""
import pytest

from gpuexplore_gb300 import gen
from helpers import oracle, write_net

pytestmark = pytest.mark.gpu


def _still_works(lib, tmp_path):
    path = write_net(gen.ring(1), tmp_path, "after")
    r = lib.explore(path, q_words=1 << 22)
    assert r["states"] == oracle(path, [])["states"]


def test_bounded_wait_times_out(gpu, tmp_path):
    rc, waited = gpu.selftest_bounded_wait(50_000_000)  # 50 ms on a flag nothing sets
    assert rc == 5  # GPX_ERR_TIMEOUT
    assert 50_000_000 <= waited < 2_000_000_000
    _still_works(gpu, tmp_path)


def test_table_full_is_a_status(gpu, tmp_path):
    path = write_net(gen.random_network(12, nprocs=12, states=(4, 9)), tmp_path, "big")
    r = gpu.explore(path, check=False, q_words=1 << 12, store_states=1 << 20)  # 16 KB table
    assert r["rc"] == 4 and r["stopped"] == "error"  # GPX_ERR_TABLE_FULL
    _still_works(gpu, tmp_path)


def test_store_full_is_a_status(gpu, tmp_path):
    path = write_net(gen.random_network(12, nprocs=12, states=(4, 9)), tmp_path, "big")
    r = gpu.explore(path, check=False, q_words=1 << 24, store_states=5000)
    assert r["rc"] == 8 and r["stopped"] == "error"  # GPX_ERR_STORE_FULL
    _still_works(gpu, tmp_path)


def test_invalid_launch_shape(gpu, tmp_path):
    path = write_net(gen.ring(1), tmp_path, "r")
    r = gpu.explore(path, check=False, threads=48)  # not a multiple of 32
    assert r["rc"] == 6
    _still_works(gpu, tmp_path)


def test_random_access_probes(gpu):
    """The two random-access ceilings the bench reports: gathers of random
    32-byte sectors, and insert-like read + CAS accesses (slower: each dirties
    a sector that is written back)."""
    g = gpu.random_gather_rate(0, 1 << 30)
    i = gpu.random_insert_rate(0, 1 << 30)
    assert 1e9 < g < 1e12 and 1e9 < i < 1e12
    assert i < 1.5 * g
