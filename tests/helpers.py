"""Shared test helpers: write generated networks and run the oracle (the checker)."""
import json
import os
import subprocess

from gpuexplore_gb300 import gpf
from gpuexplore_gb300.build import ORACLE

FLAGS = {
    "plain": ([], {}),
    "deadlock": (["-d"], {"property": "deadlock"}),
    "safety": (["-p"], {"property": "safety", "cycle_proviso": 1}),
    "por": (["--por"], {"por": 1}),
    "por_proviso": (["--por", "--cycle-proviso"], {"por": 1, "cycle_proviso": 1}),
    "por_safety": (["--por", "-p"], {"por": 1, "cycle_proviso": 1, "property": "safety"}),
    "por_deadlock": (["--por", "-d"], {"por": 1, "property": "deadlock"}),
    "ample_deadlock": (["--ample", "-d"], {"por": 3, "property": "deadlock"}),
    "ample_safety": (["--ample", "-p"], {"por": 3, "cycle_proviso": 1, "property": "safety"}),
    "stubborn_proviso": (["--stubborn", "--cycle-proviso"], {"por": 4, "cycle_proviso": 1}),
    "stubborn_deadlock": (["--stubborn", "-d"], {"por": 4, "property": "deadlock"}),
    "stubborn_safety": (["--stubborn", "-p"], {"por": 4, "cycle_proviso": 1, "property": "safety"}),
}


def write_net(net, tmpdir, name):
    path = os.path.join(str(tmpdir), name + ".gpf")
    gpf.write(net, path)
    return path


def oracle(path, flags, threads=2, max_states=0, dump=None):
    cmd = [ORACLE, path, "--threads", str(threads)] + list(flags)
    if max_states:
        cmd += ["--max-states", str(max_states)]
    if dump:
        cmd += ["--dump-states", dump]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    return json.loads(out.stdout)
