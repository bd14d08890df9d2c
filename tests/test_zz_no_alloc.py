"""gpx_explore_noalloc: the exploration for callers that cannot allocate device
memory (e.g. a process whose framework allocator owns the GPU's memory, or a
loop that cannot afford cudaMalloc's device synchronisation).  Its scratch is
the library's static device array; its results must equal gpx_explore's
bit for bit, on consecutive calls that reuse the array."""
import os
import subprocess
import sys

import pytest

from gpuexplore_gb300 import gen, gpf

pytestmark = pytest.mark.gpu

KEYS = ("states", "levels", "verdict", "stopped", "set_hash")


def _model(lib, net):
    return lib.Model.from_words(gpf.encode(net))


@pytest.mark.parametrize("case", ["ring_deadlock", "rand_por_proviso", "rand24_budget"])
def test_noalloc_matches_explore(gpu, case):
    lib = gpu
    if case == "ring_deadlock":
        net, kw = gen.ring(2), dict(property="deadlock")
    elif case == "rand_por_proviso":
        net, kw = gen.random_network(12, nprocs=12, states=(4, 9)), dict(por=1, cycle_proviso=1, max_states=200_000)
    else:
        net, kw = gen.random_network(13, nprocs=24, states=(4, 9), outdeg=(1, 2)), dict(max_states=300_000)
    m = _model(lib, net)
    ref = lib.explore(m, q_words=1 << 22, prune_commuting=0, **kw)  # the no-allocation path does not prune
    # two calls in a row: the second reuses the array the first left behind
    for _ in range(2):
        got = lib.explore_noalloc(m, **kw)
        for k in KEYS:
            assert got[k] == ref[k], (case, k)
        assert got["lookups"] == ref["lookups"] and got["inserts"] == ref["inserts"]


def test_noalloc_alternating_models(gpu):
    """Consecutive calls with different models and key widths leave no trace in each other's results."""
    lib = gpu
    nets = [gen.ring(4), gen.random_network(5, nprocs=12, states=(4, 9)), gen.ring(4)]
    for net in nets:
        m = _model(lib, net)
        ref = lib.explore(m, q_words=1 << 24, property="deadlock", max_states=200_000)
        got = lib.explore_noalloc(m, property="deadlock", max_states=200_000)
        assert [got[k] for k in KEYS] == [ref[k] for k in KEYS]


def test_noalloc_rejects_oversize(gpu):
    lib = gpu
    m = _model(lib, gen.ring(1))
    limit_words = (64 << 20) // 4
    r = lib.explore_noalloc(m, check=False, q_words=limit_words)      # table alone as big as the array
    assert r["rc"] == 6
    r = lib.explore_noalloc(m, check=False, q_words=1 << 20, store_states=1 << 30)
    assert r["rc"] == 6
    # sizes whose byte counts would wrap 64 bits are refused, not truncated
    for huge in (dict(store_states=1 << 62), dict(q_words=1 << 62), dict(q_words=1 << 20, store_states=(1 << 58))):
        r = lib.explore_noalloc(m, check=False, **huge)
        assert r["rc"] == 6, huge
    ok = lib.explore_noalloc(m, q_words=1 << 20, store_states=1 << 20)
    assert ok["states"] > 0


def test_noalloc_level_capacity(gpu):
    """A short caller array receives the first levels; nlevels reports the full count."""
    lib = gpu
    m = _model(lib, gen.ring(2))
    ref = lib.explore(m, q_words=1 << 22)
    import ctypes as C
    L = lib.load()
    o = lib.options()
    levels = (C.c_uint64 * 3)()
    r = lib.Result()
    rc = L.gpx_explore_noalloc(m.handle, C.byref(o), levels, 3, C.byref(r))
    assert rc == 0 and r.nlevels == len(ref["levels"])
    assert list(levels) == ref["levels"][:3]
    d = lib.explore_noalloc(m, level_capacity=3)
    assert d["levels"] == ref["levels"][:3] and d["nlevels"] == len(ref["levels"])


_FIRST_CALL = r"""
import sys
sys.path.insert(0, sys.argv[1])
from gpuexplore_gb300 import gen, gpf, lib
m = lib.Model.from_words(gpf.encode(gen.ring(5)))
first = lib.explore_noalloc(m, property="deadlock", set_hash=1)   # the first libgpx call on the device
second = lib.explore_noalloc(m, property="deadlock", set_hash=1)
ref = lib.explore(m, property="deadlock", q_words=1 << 22, set_hash=1)
for k in ("states", "levels", "verdict", "stopped", "set_hash"):
    assert first[k] == ref[k] == second[k], (k, first[k], second[k], ref[k])
print("ok", first["states"])
"""


def test_noalloc_first_call_in_fresh_process(gpu):
    """With lazy module loading (CUDA's default), the first use of the library
    on a device loads its kernels and reserves the static array.  When the
    no-allocation call is that first use, it still succeeds and matches
    gpx_explore."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    out = subprocess.run([sys.executable, "-c", _FIRST_CALL, root], capture_output=True, text=True, env=env,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("ok ")
