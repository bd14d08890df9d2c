"""GPU parity on the gpf forms the default generators avoid: single-party
synchronisation rules, an action's targets spread over three or more entries
with empty slots (max_buf_ints >= 3), and repeated targets, across every flag
set (plain, deadlock, safety, the three POR variants with and without the
cycle proviso) and all three slot widths.

libgpx decodes each (process, local state) once into its local targets and,
per action, the targets of all its entries; a rule fires when every member has
the action (G:1457-1464, gather_por's reading; gather additionally needs a
second enabled process, G:980-997) and yields the product of the members'
targets over every entry (gather drops entries past its doubled buffer index,
G:964-977; both reference kernels stop at an entry's first empty slot and find
the current target by value, G:1085-1112).  The oracle restates the same
intended semantics, pinned on these forms against the abstract explorer in
tests/test_corner_cases_cpu.py.
"""
import pytest

from gpuexplore_gb300 import gen, gpf
from helpers import FLAGS, oracle

FAMILIES = {
    # name: (network, encoding options)
    "c9_split": (lambda: gen.corner_network(1), dict(max_slots=1)),
    "c9_repeat": (lambda: gen.corner_network(5), dict(repeat_seed=5)),
    "c9_both": (lambda: gen.corner_network(7), dict(max_slots=1, repeat_seed=7)),
    "c14_both": (lambda: gen.corner_network(11, nprocs=14, states=(3, 6)), dict(max_slots=1, repeat_seed=11)),
    "c24_both": (lambda: gen.corner_network(13, nprocs=24, states=(3, 5)), dict(max_slots=1, repeat_seed=13)),
}


def _write(net, tmp_path, name, enc):
    words = gpf.encode(net, **enc)
    p = tmp_path / (name + ".gpf")
    p.write_text("\n".join(str(w) for w in words) + "\n")
    return str(p), gpf.header(words)


def test_families_cover_the_forms():
    widths = set()
    for name, (mk, enc) in FAMILIES.items():
        net = mk()
        words = gpf.encode(net, **enc)
        bits = net.firstbit()[-1]
        widths.add(4 if bits <= 31 else (8 if bits <= 63 else 16))
        assert any(bin(r).count("1") == 1 for rs in net.rules.values() for r in rs), name
        if "max_slots" in enc:
            assert gpf.header(words).max_buf_ints >= 3, name
    assert widths == {4, 8, 16}


@pytest.mark.gpu
@pytest.mark.parametrize("family", sorted(FAMILIES))
@pytest.mark.parametrize("flags", sorted(FLAGS))
def test_corner_parity(gpu, tmp_path, family, flags):
    mk, enc = FAMILIES[family]
    path, _ = _write(mk(), tmp_path, family, enc)
    cli, kw = FLAGS[flags]
    budget = 200_000
    o = oracle(path, cli, max_states=budget)
    g = gpu.explore(path, check=False, max_states=budget, q_words=1 << 24, **kw)
    assert g["rc"] == 0, g
    for k in ("states", "levels", "verdict", "stopped", "set_hash"):
        assert g[k] == o[k], (family, flags, k, g[k], o[k])


@pytest.mark.gpu
@pytest.mark.parametrize("family", ["c9_both", "c24_both"])
def test_corner_batch(gpu, tmp_path, family):
    """The many-network kernel on the same forms (its own rule evaluation path)."""
    mk, enc = FAMILIES[family]
    path, _ = _write(mk(), tmp_path, family, enc)
    models, jobs, want = [], [], []
    for fl in ("deadlock", "safety", "por_proviso", "stubborn_deadlock", "plain"):
        cli, kw = FLAGS[fl]
        jobs.append({"property": kw.get("property", "none"), "por": kw.get("por", 0),
                     "cycle_proviso": kw.get("cycle_proviso", 0), "max_states": 200_000})
        want.append(oracle(path, cli, max_states=200_000))
        models.append(gpu.Model.from_file(path))
    items, _ = gpu.batch_explore(models, jobs, level_capacity=4096)
    for it, w in zip(items, want):
        assert it["status"] == 0
        for k in ("states", "levels", "verdict", "stopped", "set_hash"):
            assert it[k] == w[k], (family, k)
