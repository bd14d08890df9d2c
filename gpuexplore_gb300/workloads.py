"""The benchmark workloads: seeded synthetic gpf networks with the sizes and
settings each configuration is measured on.  bench.py times them and the GPU
parity tests compare the same networks, with the same options, against the
CPU oracle, so a benchmarked figure always belongs to a checked result.

The reference's own model set is not available (an external tarball); these
generators stand in for it with the shapes the measurement plan names.

config 1  rings of 8 processes x 5 local states, seeds 1-10, -d, 2^22-word table
config 2  one random network of 16 processes (8-32 states, out-degree 1-4, 20%
          synchronising actions over 2-3 processes) plus the embedded safety
          monitor: 17 processes, 82-bit state vectors; -d (headline) or -p;
          BFS to the end of the level that reaches 1e8 states; 5e9-word
          (20 GB) hash table
config 3  clustered networks of 24 processes in 4-6 clusters, seeds 1-3,
          --por --cycle-proviso, 2e7-state budget per network
"""
from __future__ import annotations

from typing import Dict, List, Tuple

from . import gen
from .gpf import Network

CONFIG2_SEED = 2024
CONFIG2_BUDGET = 100_000_000
CONFIG2_Q_WORDS = 5_000_000_000
# a bounded sample of the same network: the first 9 BFS levels (38.8M states)
CONFIG2_SAMPLE_BUDGET = 10_000_000

CONFIG3_SEEDS = (1, 2, 3)
CONFIG3_BUDGET = 20_000_000
CONFIG3_Q_WORDS = 2_500_000_000

CONFIG1_SEEDS = tuple(range(1, 11))
CONFIG1_Q_WORDS = 1 << 22

# (oracle flags, libgpx options) of each property setting used by the workloads
PROPERTY_FLAGS: Dict[str, Tuple[List[str], Dict]] = {
    "deadlock": (["-d"], {"property": "deadlock"}),
    "safety": (["-p"], {"property": "safety", "cycle_proviso": 1}),
    "por_proviso": (["--por", "--cycle-proviso"], {"por": 1, "cycle_proviso": 1}),
}


def config1_networks() -> List[Network]:
    return [gen.ring(s) for s in CONFIG1_SEEDS]


def config2_network() -> Network:
    return gen.random_network(CONFIG2_SEED)


def config3_networks() -> List[Network]:
    return [gen.clustered(s, nprocs=24) for s in CONFIG3_SEEDS]
