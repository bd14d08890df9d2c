"""The gpf forms the default generators avoid, on the CPU: single-party
synchronisation rules, an action's targets spread over three or more entries
(max_buf_ints >= 3) with empty slots in each, and repeated targets.

The reference's two kernels disagree on these forms (gather needs two enabled
processes per synchronisation round, G:980-997, where gather_por does not,
G:1457-1464; gather's buffer fill steps its index twice, G:964-977; the
odometer of both stops at the first empty slot and locates the current target
by value, G:1085-1112).  The oracle and libgpx implement the intended
semantics: a rule fires when every member has the action, with the product of
all the members' targets for it.  Here the oracle is pinned on these forms
against the abstract explorer, which never sees the gpf encoding.
"""
import pytest

from gpuexplore_gb300 import gen, gpf
import abstract_explorer as ax
from helpers import oracle

FLAGS = {(): {}, ("-d",): {"prop": "deadlock"}, ("-p",): {"prop": "safety", "proviso": True},
         ("--por",): {"por": True}, ("--por", "--cycle-proviso"): {"por": True, "proviso": True},
         ("--stubborn", "-d"): {"prop": "deadlock", "por": True, "kind": "stubborn"},
         ("--ample", "-p"): {"prop": "safety", "por": True, "proviso": True, "kind": "ample"}}

ENCODINGS = {"split": dict(max_slots=1), "repeat": dict(repeat_seed=7), "both": dict(max_slots=1, repeat_seed=3)}


def _write(net, tmp_path, name, **enc):
    words = gpf.encode(net, **enc)
    p = tmp_path / (name + ".gpf")
    p.write_text("\n".join(str(w) for w in words) + "\n")
    return str(p), gpf.header(words)


@pytest.mark.parametrize("enc", sorted(ENCODINGS))
@pytest.mark.parametrize("seed", [1, 5, 7])
def test_corner_forms_against_abstract_explorer(built, tmp_path, enc, seed):
    net = gen.corner_network(seed, nprocs=5, states=(3, 5))
    path, hdr = _write(net, tmp_path, f"c{seed}", **ENCODINGS[enc])
    if "max_slots" in ENCODINGS[enc]:
        assert hdr.max_buf_ints >= 3
    for fl, kw in FLAGS.items():
        a = ax.explore(net, **kw)
        o = oracle(path, list(fl), threads=2)
        assert o["states"] == a["states"] and o["levels"] == a["levels"], (enc, seed, fl)
        assert o["verdict"] == a["verdict"] and o["set_hash"] == ax.set_hash(net, a["visited"]), (enc, seed, fl)


def test_corner_networks_exercise_single_party_rules():
    """Not vacuous: the single-party rules change the level counts on these
    seeds (compared with the same networks without them), and some fire in
    states where no other process offers the action -- the case gather never
    fires."""
    changed = 0
    for seed in (1, 5, 7):
        net = gen.corner_network(seed, nprocs=5, states=(3, 5))
        singles = {a: [r for r in rs if bin(r).count("1") == 1] for a, rs in net.rules.items()}
        assert any(singles.values())
        stripped = gpf.Network(nstates=net.nstates, local=net.local, sync=net.sync,
                               rules={a: [r for r in rs if bin(r).count("1") > 1] for a, rs in net.rules.items()})
        full, less = ax.explore(net), ax.explore(stripped)
        changed += full["levels"] != less["levels"]
        lonely = False
        for s in full["visited"]:
            for a, rs in singles.items():
                offered = [p for p in range(net.nprocs) if a in net.sync[p][s[p]]]
                if len(offered) == 1 and any(r == 1 << offered[0] for r in rs):
                    lonely = True
        assert lonely, seed
    assert changed == 3
