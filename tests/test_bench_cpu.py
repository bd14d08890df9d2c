"""bench.py's host-side pieces on CPU: the workload object both arms print and
the oracle legs under each property of the headline network."""
import os
import sys

from gpuexplore_gb300 import gen, gpf

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_workload_config_names_the_property():
    d = bench.workload_config(100, 1 << 20, 42, 3)
    p = bench.workload_config(100, 1 << 20, 42, 3, "safety")
    assert d["property"] == "deadlock (-d)" and ", -d," in d["workload"]
    assert p["property"] == "safety (-p)" and ", -p," in p["workload"]
    # everything but the property is the same workload
    assert {k: v for k, v in d.items() if k not in ("property", "workload")} == \
           {k: v for k, v in p.items() if k not in ("property", "workload")}


def test_oracle_legs_follow_the_property(built, tmp_path):
    """The CPU legs pass the property's flag to the oracle: this ring never
    deadlocks, but its safety monitor reaches the error state, so only the -p
    leg reports a violation (and stops at that level)."""
    path = str(tmp_path / "r.gpf")
    gpf.write(gen.ring(3), path)
    d = bench.cpu_oracle_run(path, 2, 0, "deadlock")
    p = bench.cpu_oracle_run(path, 2, 0, "safety")
    assert (d["verdict"], d["stopped"]) == ("none", "done")
    assert (p["verdict"], p["stopped"]) == ("safety", "violation") and p["states"] <= d["states"]
    s = bench.cpu_single_thread(path, "safety")
    assert s["cores"] == 1 and s["value"] > 0
