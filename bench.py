"""Benchmark: new states/s of on-the-fly exploration on one GB300 (per rank).

Workload (the config-2 network): a seeded random gpf network of 16 processes
with U[8, 32] local states, local out-degree U[1, 4], 20% of transitions
synchronising 2-3 processes, plus the embedded safety monitor (17 processes,
82-bit state vectors, 128-bit hash slots); deadlock check (-d); exploration to
the end of the BFS level that reaches 1e8 states; hash table of 5e9 32-bit
words (20 GB).  One step = one complete exploration: table reset, initial
state, all levels.  The reset is by generation: the 128-bit slots carry the
run's 8-bit tag and slots of older runs read as free, so the table is zeroed
once every 255 runs; that clear is charged to every step, amortised.  Inputs
are synthetic (seeded generator) -- the reference's model set is not available.

value    states / device time of the step (table reset + exploration kernels,
         CUDA events on the launching stream; the model is already resident)
e2e      the same metric through the C ABI with host buffers: every step parses
         the gpf words from host memory, copies the model to the device
         (gpx_explorer_set_model) and reads the results back (gpx_explorer_run;
         the visited-set hash, a check, is off as in the library's defaults)
roofline dominant kernel (explore_kernel): algorithmic bytes per launch --
         32 B per hash lookup, 32 B per insert, 2 x 4*sv_nints B per expanded
         state -- over its CUDA-event duration, against the measured HBM peak
cpu_baseline / --impl reference
         the CPU oracle (a port of the reference's semantics; the reference has
         no CPU path) with all host threads on the whole workload (all 10
         levels); its states, level counts and visited-set hash must equal the
         GPU run's (cpu_baseline.parity).  A single-thread figure on a named
         sample (the first 9 levels) is reported beside it.

Multi-GPU (torchrun): replicas -- each rank explores its own copy; the job
value is the sum of states over the max step time across ranks ("weak").
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from gpuexplore_gb300 import workloads as W  # noqa: E402

SEED = W.CONFIG2_SEED
BUDGET = W.CONFIG2_BUDGET
Q_WORDS = W.CONFIG2_Q_WORDS
CPU_SAMPLE_BUDGET = W.CONFIG2_SAMPLE_BUDGET  # the first 9 BFS levels (38.8M states)
WORKLOAD = "config-2 random gpf network (16 procs + monitor, seed 2024), -d, BFS to 1e8-state budget"
KERNEL_BUILD = "claim-rule-v2"  # names the kernel version a committed traffic capture belongs to


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def make_network_words():
    """The network and its gpf words as a host buffer (32-bit words)."""
    import numpy as np
    from gpuexplore_gb300 import gpf
    net = W.config2_network()
    return net, np.asarray(gpf.encode(net), dtype=np.uint32)


PROPERTY_FLAG = {"deadlock": "-d", "safety": "-p"}


def workload_config(budget, q_words, states, levels, prop="deadlock"):
    """The `config` object both arms print: the workload only (network,
    property, budget, table size) and the size of its result."""
    workload = WORKLOAD if prop == "deadlock" else WORKLOAD.replace(", -d,", ", -p,")
    return {"workload": workload, "property": f"{prop} ({PROPERTY_FLAG[prop]})", "budget": budget, "q_words": q_words,
            "table_gb": q_words * 4 / 1e9, "states": states, "levels": levels,
            "l2": "inputs larger than L2 (20 GB hash table, reset every step)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(r, sv_nints):
    """32 B per hash lookup (one DRAM sector), 32 B per insert (the sector written
    back), and the frontier write + read of each expanded state."""
    return 32 * r["lookups"] + 32 * r["inserts"] + 2 * 4 * sv_nints * r["expanded"]


def max_over_ranks(step_ms, e2e_s, dist):
    """Slowest replica's step time and end-to-end time (replicas run concurrently)."""
    if dist is None:
        return step_ms, e2e_s
    import torch
    t = torch.tensor([step_ms, e2e_s], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0]), float(t[1])


def job_value(states_per_rank, step_ms, world):
    """Whole-job states per second: every replica explores its own copy."""
    return states_per_rank * world / (step_ms / 1000.0)


def cpu_oracle_run(path, threads, budget, prop="deadlock"):
    from gpuexplore_gb300.build import ORACLE
    out = subprocess.run([ORACLE, path, PROPERTY_FLAG[prop], "--threads", str(threads), "--max-states", str(budget)],
                         capture_output=True, text=True, check=True)
    return json.loads(out.stdout)


def cpu_single_thread(path, prop="deadlock"):
    """The oracle on one thread over the named sample (the first 9 levels)."""
    o = cpu_oracle_run(path, 1, CPU_SAMPLE_BUDGET, prop)
    return {"value": o["states"] / o["seconds"], "unit": "states/s", "cores": 1, "seconds": o["seconds"],
            "sample": f"first {len(o['levels'])} BFS levels ({o['states']} states) of the same network"}


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores: the CPU oracle (the reference
    has no CPU path of its own) with every host thread, on the whole workload.
    Warm-up steps run the first 9 levels only (the CPU has nothing to warm
    beyond its caches and page tables); timed steps run all 10."""
    if rank != 0:
        return
    from gpuexplore_gb300 import build, gpf
    build.build_oracle()
    net, words = make_network_words()
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "c2.gpf")
        gpf.write(net, path)
        for _ in range(args.warmup):
            cpu_oracle_run(path, threads, CPU_SAMPLE_BUDGET, args.property)
        secs, results = [], []
        for _ in range(args.steps):
            o = cpu_oracle_run(path, threads, args.budget, args.property)
            secs.append(o["seconds"])
            results.append(o)
        single = cpu_single_thread(path, args.property)
    o = results[-1]
    for x in results:  # deterministic whatever the thread schedule
        assert (x["states"], x["levels"], x["set_hash"]) == (o["states"], o["levels"], o["set_hash"])
    v = o["states"] / (sum(secs) / len(secs))
    sample = (f"the whole workload: {len(o['levels'])} BFS levels, {o['states']} states, on {threads} host threads "
              f"(OpenMP); warm-up steps on the first 9 levels")
    line = {"impl": "reference", "metric": "new states/s", "value": v, "unit": "states/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(secs) / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": workload_config(args.budget, args.q_words, o["states"], len(o["levels"]), args.property),
            "cpu_baseline": {"value": v, "unit": "states/s", "cores": threads, "kind": "port", "sample": sample,
                             "set_hash": o["set_hash"], "single_thread": single},
            "e2e": {"value": v, "unit": "states/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# the batch options gpx_batch_explore's autotuner chooses
TUNED = ("claim", "threads", "load_factor", "kernel_iters", "narrow_slots")


def run_other_workload(args, local):
    """Configs 1, 3 and 5 (the headline is config 2): one JSON line each."""
    import random
    from gpuexplore_gb300 import build, gen, gpf, lib
    build.build_all()
    line = {"metric": "new states/s", "unit": "states/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded gpf generator)"}
    if args.workload == "config4":
        import time as _t
        from gpuexplore_gb300 import learned_por
        t0 = _t.time()
        rows = learned_por.log_candidates(range(1, args.train_seeds + 1), budget=20_000, sample_every=128,
                                          device=local)
        t1 = _t.time()
        # validation seeds (disjoint from training and evaluation) pick the training target
        val = range(500_001, 500_001 + args.val_seeds)
        model, target, loss, val_scores = learned_por.choose_target(rows, val, budget=args.eval_budget,
                                                                    device=local)
        t2 = _t.time()
        held = range(1_000_001, 1_000_001 + args.eval_seeds)
        ev = learned_por.evaluate(model, held, budget=args.eval_budget, device=local)
        t3 = _t.time()
        model_path = os.path.join(ROOT, "gpuexplore_gb300", "_lib", "por_model_config2.bin")
        learned_por.save(model, model_path)
        red = 1.0 - ev["decided_states_learned"] / max(1, ev["decided_states_cample"])
        # the chosen target trained from initialisations not seen in validation: how much
        # the gain depends on the seed without the validation-based choice
        spread = {}
        for sd in (11, 12, 13):
            m_sd, _ = learned_por.train(rows, target=target, device=local, seed=sd)
            e_sd = learned_por.evaluate(m_sd, held, budget=args.eval_budget, device=local)
            spread[str(sd)] = 1.0 - e_sd["decided_states_learned"] / max(1, e_sd["decided_states_cample"])
        line.update(metric="states-to-verdict reduction vs plain cample", value=red, unit="fraction",
                    higher_is_better=True, ms_per_step=1000 * (t3 - t0),
                    config={"workload": f"config-4 learned cluster proposal: trained on candidate logs of "
                                        f"{args.train_seeds} config-2 seeds, target chosen on {args.val_seeds} "
                                        f"validation seeds, evaluated on {args.eval_seeds} held-out seeds with -p "
                                        f"(cycle proviso), budget {args.eval_budget}; value = 1 - states to the "
                                        f"verdict (learned / plain cample) on the seeds BFS decides",
                            "rows": int(len(rows)), "target": target, "val_decided_states": val_scores,
                            "reduction_other_train_seeds": spread,
                            "train_loss": loss, "log_s": t1 - t0, "train_s": t2 - t1, "eval_s": t3 - t2,
                            **{k: v for k, v in ev.items() if k != "per_seed"}})
        print(json.dumps(line), flush=True)
        return
    if args.workload == "liveness":
        # accepting-cycle check: a 20-process network, 5.2M states, where the
        # property holds (the whole fixpoint runs), and its violating variant
        import time as _t
        nets = {"holds": gen.progress_network(7, nprocs=20, states=(3, 4), sync_frac=0.5),
                "violated": gen.progress_network(7, nprocs=20, states=(3, 4), sync_frac=0.5, cyclic=True)}
        per = {}
        for name, net in nets.items():
            m = lib.Model.from_words(gpf.encode(net))
            ex = lib.Explorer(m, lib.options(device=local, property="safety", cycle_proviso=1, q_words=1 << 29))
            for _ in range(args.warmup):
                ex.run()
            ker, live, r = [], [], None
            for _ in range(args.steps):
                r = ex.run()
                ker.append(r["kernel_ms"])
                live.append(r["live_ms"])
            ex.close()
            per[name] = {"states": r["states"], "verdict": r["verdict"], "explore_ms": statistics.median(ker),
                         "check_ms": statistics.median(live), "fixpoint_states": r["live_states"],
                         "check_rounds": r["live_rounds"]}
        h = per["holds"]
        value = h["states"] / ((h["explore_ms"] + h["check_ms"]) / 1000.0)
        line.update(metric="states checked/s (exploration + accepting-cycle check)", value=value,
                    ms_per_step=h["explore_ms"] + h["check_ms"],
                    config={"workload": "liveness: progress network (20 processes + Buchi monitor, seed 7), "
                                        "-p on a liveness gpf, full exploration + accepting-cycle check",
                            **{f"{k}_{kk}": vv for k, v in per.items() for kk, vv in v.items()}})
        if not args.no_cpu_baseline:
            from gpuexplore_gb300.build import ORACLE
            threads = os.cpu_count() or 1
            with tempfile.TemporaryDirectory() as d:
                path = os.path.join(d, "live.gpf")
                gpf.write(nets["holds"], path)
                t0 = _t.time()
                o = json.loads(subprocess.run([ORACLE, path, "-p", "--threads", str(threads)], capture_output=True,
                                              text=True, check=True).stdout)
                secs = _t.time() - t0
            line["cpu_baseline"] = {"value": o["states"] / secs, "unit": "states/s", "cores": threads, "kind": "port",
                                    "sample": f"the whole 'holds' network ({o['states']} states): OpenMP BFS, then "
                                              "a single-threaded Tarjan SCC check (verdict "
                                              f"{o['verdict']})"}
        print(json.dumps(line), flush=True)
        return
    if args.workload in ("config1", "config3"):
        if args.workload == "config1":
            nets = W.config1_networks()
            kw = dict(W.PROPERTY_FLAGS["deadlock"][1], q_words=W.CONFIG1_Q_WORDS)
            desc = "config-1 rings of 8 processes x 5 states, seeds 1-10, -d, 2^22-word table"
        else:
            nets = W.config3_networks()
            kw = dict(W.PROPERTY_FLAGS["por_proviso"][1], q_words=args.q_words or W.CONFIG3_Q_WORDS,
                      max_states=args.budget or W.CONFIG3_BUDGET)
            desc = "config-3 clustered networks (24 processes, 4-6 clusters), seeds 1-3, --por --cycle-proviso"
        models = [lib.Model.from_words(gpf.encode(n)) for n in nets]
        kw["launch_graph"] = 0 if args.no_graph else 1
        ex = lib.Explorer(models[0], lib.options(device=local, **kw))
        for _ in range(args.warmup):
            for m in models:
                ex.set_model(m)
                ex.run()
        ms, states, kms = 0.0, 0, 0.0
        probes = inserts = lookups = 0
        for _ in range(args.steps):
            for m in models:
                ex.set_model(m)
                r = ex.run()
                ms += r["setup_ms"] + r["kernel_ms"]
                kms += r["kernel_ms"]
                states += r["states"]
                probes += r["probes"]
                inserts += r["inserts"]
                lookups += r["lookups"]
        extra = {"lookups_per_step": lookups // args.steps, "probes_per_step": probes // args.steps,
                 "inserts_per_step": inserts // args.steps}
        if args.workload == "config3":
            # the table's random-access floor, as for the headline: every insert is a
            # read + CAS of a random bucket, every other probe (the decide pass's
            # lookups, mostly) a random 32-byte gather; the table is 10 GB
            gathers = lib.random_gather_rate(local, 20 << 30)
            rmw = lib.random_insert_rate(local, 20 << 30)
            floor = (inserts / rmw + max(0, probes - inserts) / gathers) * 1000.0 / args.steps
            extra["random_access"] = {"floor_ms": floor, "frac": floor / (kms / args.steps),
                                      "peak_gathers_per_s": gathers, "peak_inserts_per_s": rmw}
        if args.workload == "config1":
            # the same ten rings in one batched launch (gpx_batch_explore); the first
            # warm-up call autotunes, the timed calls reuse what it chose
            jobs = [{"property": "deadlock", "capacity": 1 << 18} for _ in nets]
            tuned = {}
            for w in range(max(1, args.warmup)):
                _, st = lib.batch_explore(models, jobs, autotune=1 if w == 0 else 0, **tuned)
                tuned = {k: st[k] for k in TUNED}
            bms, bst = 0.0, 0
            for _ in range(args.steps):
                items, st = lib.batch_explore(models, jobs, **tuned)
                bms += st["device_ms"]
                bst += st["states"]
            extra.update({"batched_states_per_s": bst / (bms / 1000.0), "batched_ms_per_step": bms / args.steps,
                          "batched_tuned": tuned})
        else:
            # the other reductions on the same networks: states kept and device time
            ex.close()
            for name, por in (("ample", 3), ("stubborn", 4), ("none", 0)):
                kwv = dict(kw, por=por)
                exv = lib.Explorer(models[0], lib.options(device=local, **kwv))
                vs, vms = 0, 0.0
                for m in models:
                    exv.set_model(m)
                    exv.run()
                    r = exv.run()
                    vs += r["states"]
                    vms += r["setup_ms"] + r["kernel_ms"]
                exv.close()
                extra[f"{name}_states"] = vs
                extra[f"{name}_ms"] = vms
            extra["note"] = "none_* = unreduced BFS to the same state budget"
        line.update(value=states / (ms / 1000.0), ms_per_step=ms / args.steps,
                    config={"workload": desc, "states_per_step": states // args.steps, "networks": len(nets),
                            "kernel_ms_per_step": kms / args.steps, **extra})
    else:
        from gpuexplore_gb300 import learned_por
        rng = random.Random(5)
        nets = gen.batch(5, count=args.batch_count)
        models = [lib.Model.from_words(gpf.encode(n)) for n in nets]
        # the learned cluster proposal for the POR half (outside the timed region):
        # candidate logs of 200 config-2 seeds, the label and initialisation config 4 selects
        rows = learned_por.log_candidates(range(1, 201), budget=20_000, sample_every=128, device=local)
        por_model, _ = learned_por.train(rows, target="succ", device=local, seed=8)
        jobs = []
        for k in range(len(nets)):
            jobs.append({"property": "deadlock" if k % 2 == 0 else "safety",
                         "por": 2 if (k // 2) % 2 else 0, "cycle_proviso": 1 if (k // 2) % 2 else 0,
                         "max_states": int(10 ** rng.uniform(3, 7))})
        # the warm-up call autotunes claim size, block size, load factor and claims per
        # launch; timed calls reuse them
        tuned = {}
        for w in range(max(1, args.warmup)):
            _, st = lib.batch_explore(models, jobs, autotune=1 if w == 0 else 0, por_model=por_model, **tuned)
            tuned = {k: st[k] for k in TUNED}
        dev, states, p50, p99 = 0.0, 0, [], []
        for _ in range(args.steps):
            items, st = lib.batch_explore(models, jobs, por_model=por_model, **tuned)
            dev += st["device_ms"]
            states += st["states"]
            p50.append(st["p50_ms"])
            p99.append(st["p99_ms"])
        line.update(value=states / (dev / 1000.0), ms_per_step=dev / args.steps,
                    config={"workload": f"config-5 batch of {len(nets)} random networks (4-24 procs x 4-32 states), "
                                        "state budgets log-uniform 1e3-1e7, half -d / half -p, half cluster POR with "
                                        "the learned proposal and the cycle proviso, one persistent launch",
                            "states_per_step": states // args.steps, "p50_ms": statistics.median(p50),
                            "p99_ms": statistics.median(p99), "claim": st["claim"], "threads": st["threads"],
                            "load_factor": st["load_factor"], "kernel_iters": st["kernel_iters"],
                            "narrow_slots": st["narrow_slots"], "instances_by_slot_32_64_128": st["instances_by_slot"],
                            "admissions_max": max(it["admissions"] for it in items),
                            "failed": sum(1 for it in items if it["status"] != 0)})
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpx", choices=["gpx", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch the exploration kernels from the host loop instead of one CUDA graph per run "
                         "(same kernels; used for the ncu captures)")
    ap.add_argument("--budget", type=int, default=None,
                    help="state budget (smaller values give the profiling cases of the same network)")
    ap.add_argument("--q-words", type=int, default=None,
                    help="hash table size in 32-bit words (default: the workload's own)")
    ap.add_argument("--store-states", type=int, default=0, help="state store capacity (0: table slots)")
    ap.add_argument("--property", default="deadlock", choices=["deadlock", "safety"],
                    help="the headline network's property: -d (default) or -p")
    ap.add_argument("--workload", default="config2",
                    choices=["config1", "config2", "config3", "config4", "config5", "liveness"],
                    help="config2 is the headline; the others print their own line")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--train-seeds", type=int, default=2000)
    ap.add_argument("--eval-seeds", type=int, default=200)
    ap.add_argument("--val-seeds", type=int, default=60)
    ap.add_argument("--eval-budget", type=int, default=2_000_000)
    args = ap.parse_args()
    if args.workload == "config2":
        args.budget = args.budget or BUDGET
        args.q_words = args.q_words or Q_WORDS
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload != "config2":
        if rank == 0:
            run_other_workload(args, local)
        if dist:
            dist.destroy_process_group()
        return

    from gpuexplore_gb300 import build, lib
    build.build_all()
    net, words = make_network_words()
    sv_nints = (net.firstbit()[-1] + 1 + 31) // 32  # the reference's words per vector
    model = lib.Model.from_words(words)
    base = dict(property=args.property, q_words=args.q_words, max_states=args.budget, store_states=args.store_states,
                device=local, launch_graph=0 if args.no_graph else 1)
    # Device-timed runs compute the visited-set hash after the timed interval, so
    # that every run can be checked against the others and against the oracle.
    ex = lib.Explorer(model, lib.options(set_hash=1, **base))

    def barrier():
        if dist:
            dist.barrier()

    warm = [ex.run() for _ in range(args.warmup)]
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms, ker_ms, results = [], [], []
    for _ in range(args.steps):
        r = ex.run()
        dev_ms.append(r["setup_ms"] + r["kernel_ms"])
        ker_ms.append(r["kernel_ms"])
        results.append(r)
    ex.close()
    # End to end through the C ABI from host buffers, with the library's defaults
    # (no set hash): parse the gpf words, upload the model, explore, read back.
    ex2 = lib.Explorer(model, lib.options(**base))
    for _ in range(args.warmup):
        ex2.run()
    e2e_s, e2e_runs = [], []
    h2d = len(words) * 4
    for _ in range(args.steps):
        t0 = time.perf_counter()
        m = lib.Model.from_words(words)
        ex2.set_model(m)
        r2 = ex2.run()
        e2e_s.append(time.perf_counter() - t0)
        e2e_runs.append(r2)
        m.close()
    ex2.close()
    barrier()
    clk = clocks.stop()
    r = results[-1]
    for x in results:
        assert x["states"] == r["states"] and x["levels"] == r["levels"] and x["set_hash"] == r["set_hash"]
    for x in e2e_runs:
        assert x["states"] == r["states"] and x["levels"] == r["levels"]
    # The table is reset by generation: each run's keys carry a new 8-bit tag and
    # older slots read as free, so one run in 255 zeroes the 20 GB table.  That
    # clear is charged to every step, amortised over the runs it serves.
    cleared = [x["setup_ms"] for x in warm + results if x["table_cleared"]]
    plain = [x["setup_ms"] for x in warm + results if not x["table_cleared"]]
    clear_ms = max(0.0, max(cleared) - (min(plain) if plain else 0.0)) if cleared else 0.0
    per_clear = 255 if r["table_generation"] else 1
    amortised = clear_ms / per_clear if any(not x["table_cleared"] for x in results) else 0.0
    step_ms, e2e_step = max_over_ranks(sum(dev_ms) / len(dev_ms) + amortised,
                                       sum(e2e_s) / len(e2e_s) + amortised / 1000.0, dist)
    value = job_value(r["states"], step_ms, world)
    e2e = job_value(r["states"], e2e_step * 1000.0, world)
    abytes = algorithmic_bytes(r, sv_nints)
    kms = sum(ker_ms) / len(ker_ms)
    peaks, peak_kind = measured_peaks()
    achieved = abytes / (kms / 1000.0) / 1e9
    # DRAM traffic per launch, from the committed ncu capture of the medium case of
    # the same network (first 9 levels, 2 GB table; dram__bytes_read.sum +
    # dram__bytes_write.sum of one launch), scaled to this launch by the ratio of
    # algorithmic bytes (traffic grows with lookups, inserts and expanded states)
    traffic, traffic_how, ncu_eff = None, None, None
    prof = os.path.join(ROOT, "profiles", "explore_kernel_config2_medium.json")
    if os.path.exists(prof):
        with open(prof) as f:
            pj = json.load(f)
        if pj.get("kernel_build") == KERNEL_BUILD:
            # L2 sector efficiency of the probes and warp-execution efficiency of
            # successor generation, from the same capture
            ncu_eff = {"l2_read_sectors_per_request": pj["lts_read_sectors"] / pj["lts_read_requests"],
                       "warp_execution_efficiency": pj["thread_instructions"] / (32.0 * pj["warp_instructions"]),
                       "source": "profiles/explore_kernel_config2_medium.json"}
            scale = abytes / pj["algorithmic_bytes"]
            traffic = (pj["dram_bytes_read"] + pj["dram_bytes_write"]) * scale
            traffic_how = (f"ncu capture of the medium case ({pj['states']} states, one launch), x{scale:.3f} "
                           f"by algorithmic bytes")
    # the random-access ceilings over 20 GB: 32-byte sectors gathered at random,
    # and insert-like accesses (read a random bucket, CAS a slot of it: the
    # sector is dirtied and written back).  Every insert is one of the latter,
    # the other bucket probes are gathers: their sum is the table's time floor.
    gathers = lib.random_gather_rate(local, 20 << 30)
    rmw = lib.random_insert_rate(local, 20 << 30)
    floor_ms = (r["inserts"] / rmw + max(0, r["probes"] - r["inserts"]) / gathers) * 1000.0
    line = {
        "metric": "new states/s", "value": value, "unit": "states/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded gpf generator)",
        "config": workload_config(args.budget, args.q_words, r["states"], len(r["levels"]), args.property),
        "parallelism": f"replicas x{world}",
        "launch": {"slot_bytes": r["slot_bytes"], "blocks": r["blocks"], "threads": r["threads"],
                   "table_reset": {"how": "generation tag in every slot" if r["table_generation"] else "clear",
                                   "clear_ms": clear_ms, "runs_per_clear": per_clear,
                                   "amortised_ms_per_step": amortised}},
        "e2e": {"value": e2e, "unit": "states/s", "h2d_bytes_per_step": h2d + r2["h2d_bytes"],
                "d2h_bytes_per_step": r2["d2h_bytes"], "set_hash": "off (library default)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "traffic_how": traffic_how,
                     "peak_source": f"{peak_kind} hbm_gbs", "kernel": "explore_kernel",
                     "kernel_ms": kms, "algorithmic_bytes": abytes,
                     "lookups": r["lookups"], "inserts": r["inserts"], "expanded": r["expanded"],
                     "probes": r["probes"],
                     "ncu": ncu_eff,
                     "random_access": {"probes_per_s": r["probes"] / (kms / 1000.0),
                                       # each probe reads a random sector; each insert also dirties
                                       # it, so DRAM writes it back later: a second random access
                                       "sector_accesses_per_s": (r["probes"] + r["inserts"]) / (kms / 1000.0),
                                       "sector_accesses_frac_of_gather": (r["probes"] + r["inserts"]) /
                                       (kms / 1000.0) / gathers,
                                       "peak_gathers_per_s": gathers, "peak_inserts_per_s": rmw,
                                       "floor_ms": floor_ms, "frac": floor_ms / kms,
                                       "how": "floor = inserts / insert-like rate + other probes / gather "
                                              "rate (gpx_random_insert_probe, gpx_random_gather_probe: "
                                              "random 32 B buckets over 20 GB); frac = floor / kernel time"}},
        "clocks": clk,
        # per device-timed run: init, then per exploration launch the launch itself, the placement
        # kernel (returns at once unless a level overflowed) and, in the graph, the relaunch test;
        # then the set hash
        "gpu_launches": sum((3 if not args.no_graph else 2) * x["launches"] + 2 for x in results),
        "hash_probe_gbs": 32 * r["probes"] / (kms / 1000.0) / 1e9,
    }
    parity_ok = True
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from gpuexplore_gb300 import gpf
        threads = os.cpu_count() or 1
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "c2.gpf")
            gpf.write(net, path)
            o = cpu_oracle_run(path, threads, args.budget, args.property)
            single = cpu_single_thread(path, args.property)
        # the oracle checks the GPU run: same states, per-level counts and visited set
        parity_ok = (o["states"], o["levels"], o["set_hash"]) == (r["states"], r["levels"], r["set_hash"])
        line["cpu_baseline"] = {"value": o["states"] / o["seconds"], "unit": "states/s", "cores": threads,
                                "kind": "port",
                                "sample": f"the whole workload: {len(o['levels'])} BFS levels, {o['states']} states "
                                          f"on {threads} host threads (OpenMP)",
                                "parity": parity_ok, "set_hash": o["set_hash"], "single_thread": single}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    if not parity_ok:
        sys.exit("bench: the GPU run's visited set differs from the oracle's")


if __name__ == "__main__":
    main()
