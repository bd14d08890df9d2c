"""Learned cluster proposal for partial-order reduction (config 4).

Pipeline, all on the GPU through libgpx:

1. log      explore seeded config-2 networks with cluster POR and the cycle
            proviso; the decide pass logs, for a sample of expanded states, every
            valid cluster closure: its features (gpx_por_log_row.x), the
            successors its members generate, and how many of those were not yet
            visited -- the outcome the exploration itself observes.
2. train    regress log(1 + new successors) of each candidate from its features
            with the library's own forward/backward kernels (gpx_por_train);
            the model is exported with int8 weights.
3. use      gpx_options.por = 2: each state expands the valid closure with the
            lowest predicted new-successor count; the proposal is re-checked
            (closed, a member's proviso holds) and plain cample is used otherwise.
4. evaluate on held-out seeds: states explored until the verdict with plain
            cample and with the learned proposal, and the verdicts against
            unreduced BFS.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Iterable, List, Optional

import numpy as np

from . import gen, gpf, lib


def network(seed: int):
    """A config-2 network (16 processes + the safety monitor)."""
    return gen.random_network(seed)


def random_model(seed: int) -> "lib.PorModel":
    """A seeded random model (parity tests: any weights must give identical GPU and oracle results)."""
    rng = np.random.default_rng(seed)
    m = lib.PorModel()
    w1 = rng.integers(-127, 128, size=(lib.POR_H, lib.POR_F), dtype=np.int8)
    C.memmove(C.addressof(m.w1), w1.tobytes(), w1.nbytes)
    for k in range(lib.POR_H):
        m.s1[k] = float(np.float32(rng.uniform(0.001, 0.02)))
        m.b1[k] = float(np.float32(rng.normal(0, 0.5)))
        m.w2[k] = int(rng.integers(-127, 128))
    m.s2 = float(np.float32(0.01))
    m.b2 = float(np.float32(0.1))
    return m


def save(model: "lib.PorModel", path: str) -> None:
    with open(path, "wb") as f:
        f.write(model.to_bytes())


def load_model(path: str) -> "lib.PorModel":
    with open(path, "rb") as f:
        return lib.PorModel.from_bytes(f.read())


def log_candidates(seeds: Iterable[int], budget: int = 20_000, sample_every: int = 128,
                   cap_per_run: int = 1 << 16, device: int = 0) -> np.ndarray:
    """Candidate rows logged by cycle-proviso POR explorations of the seeds' networks."""
    seeds = list(seeds)
    rows: List[np.ndarray] = []
    ex = None
    for s in seeds:
        m = lib.Model.from_words(gpf.encode(network(s)))
        if ex is None:
            ex = lib.Explorer(m, lib.options(por=1, cycle_proviso=1, max_states=budget, q_words=budget * 64,
                                             device=device))
            ex.set_por_log(cap_per_run, sample_every)
        else:
            ex.set_model(m)
        ex.run()
        r = ex.get_por_log()
        rows.append(r)
    if ex is not None:
        ex.close()
    if not rows:
        return np.zeros(0, dtype=lib.POR_LOG_DTYPE)
    out = np.concatenate(rows)
    # warps append rows in no fixed order: sort them by their bytes, so that the
    # (seeded) training sees the same sequence on every run
    order = np.argsort(out.view(np.dtype((np.void, out.dtype.itemsize))).ravel(), kind="stable")
    return out[order]


TARGETS = ("new", "succ", "mix")


def labels(rows: np.ndarray, target: str = "new") -> np.ndarray:
    """Training label of each logged candidate: log(1 + new successors) -- the
    states it adds to the next level --, log(1 + successors) -- the states the
    exploration must handle --, or the mean of the two."""
    new = np.log1p(rows["new_succ"].astype(np.float32))
    succ = np.log1p(rows["succ"].astype(np.float32))
    return {"new": new, "succ": succ, "mix": 0.5 * (new + succ)}[target]


def train(rows: np.ndarray, target: str = "new", **kw):
    return lib.por_train(rows["x"].reshape(len(rows), lib.POR_F), labels(rows, target), **kw)


def choose_target(rows: np.ndarray, val_seeds: Iterable[int], budget: int = 2_000_000, device: int = 0,
                  init_seeds: Iterable[int] = (7, 8, 9)):
    """Train one model per (target, initialisation seed) and keep the one with the
    fewest states to the verdict on validation seeds (decided by BFS).  Returns
    (model, target, loss, scores) with scores keyed "target/seed"."""
    val_seeds = list(val_seeds)
    best = None
    scores = {}
    for t in TARGETS:
        for sd in init_seeds:
            model, loss = train(rows, target=t, device=device, seed=sd)
            ev = evaluate(model, val_seeds, budget=budget, device=device)
            key = f"{t}/{sd}"
            scores[key] = ev["decided_states_learned"]
            if best is None or scores[key] < best[3]:
                best = (model, t, loss, scores[key], sd)
    return best[0], best[1], best[2], scores


def evaluate(model: "lib.PorModel", seeds: Iterable[int], budget: int = 2_000_000, device: int = 0) -> Dict:
    """Per seed: unreduced BFS, plain cample and learned proposal with -p (the
    cycle proviso on), until the verdict or the budget."""
    per: List[Dict] = []
    runs = {}
    q = budget * 64  # 16 slots per budgeted state: room for a last level that overshoots the budget
    for s in seeds:
        m = lib.Model.from_words(gpf.encode(network(s)))
        res = {}
        for name, kw in (("bfs", dict(property="safety")),
                         ("cample", dict(property="safety", por=1, cycle_proviso=1)),
                         ("learned", dict(property="safety", por=2, cycle_proviso=1))):
            if name not in runs:
                runs[name] = lib.Explorer(m, lib.options(max_states=budget, q_words=q, device=device, **kw))
                if name == "learned":
                    runs[name].set_por_model(model)
            else:
                runs[name].set_model(m)
            r = runs[name].run()
            res[name] = {"states": r["states"], "verdict": r["verdict"], "stopped": r["stopped"]}
        per.append({"seed": s, **res})
    for ex in runs.values():
        ex.close()
    done = [p for p in per if p["bfs"]["stopped"] != "budget"]
    out = {
        "decided_states_bfs": sum(p["bfs"]["states"] for p in done),
        "decided_states_cample": sum(p["cample"]["states"] for p in done),
        "decided_states_learned": sum(p["learned"]["states"] for p in done),
        "seeds": len(per),
        "verdict_mismatch_learned": sum(p["learned"]["verdict"] != p["bfs"]["verdict"] for p in per
                                        if p["bfs"]["stopped"] != "budget" and p["learned"]["stopped"] != "budget"),
        "verdict_mismatch_cample": sum(p["cample"]["verdict"] != p["bfs"]["verdict"] for p in per
                                       if p["bfs"]["stopped"] != "budget" and p["cample"]["stopped"] != "budget"),
        "states_cample": sum(p["cample"]["states"] for p in per),
        "states_learned": sum(p["learned"]["states"] for p in per),
        "states_bfs": sum(p["bfs"]["states"] for p in per),
        "learned_fewer": sum(p["learned"]["states"] < p["cample"]["states"] for p in per),
        "learned_more": sum(p["learned"]["states"] > p["cample"]["states"] for p in per),
        "violations_bfs": sum(p["bfs"]["verdict"] != "none" for p in per),
        "decided": len(done),
        "per_seed": per,
    }
    return out
