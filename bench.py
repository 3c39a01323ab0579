#!/usr/bin/env python3
"""Benchmark of the GPU simplify path: inprocessing clauses/s (SUB + BVE rounds).

One step = one full `Solver::simplify`-equivalent call (all rounds until the
reference's stop rule). The metric counts, per step, the live clauses entering
every SUB+BVE round (sum of C_in over rounds and instances).

Workloads: `batched` (the default) simplifies 512 seeded instances of uneven
size (log-uniform 1k..200k variables; random 3-SAT, Tseitin and scale-free
generators) in one batch per step, and times the plain path -- the same
instances one per simplify call -- beside it. The same line carries the
serving stream: 10,000 jobs with Poisson arrivals submitted to the native
request loop (throughput, p50/p99 latency). `tseitin`, `ksat` and
`scalefree` run one instance per step.

  value : clauses/s with the input resident in HBM when timing starts
          (CUDA events around the engine's rounds on its own stream);
  e2e   : the same metric through the C ABI with host buffers: upload (H2D),
          simplify and download (D2H) inside the timed region (the batch
          through simplify_batch(streams=4): four runs of instances on four
          contexts, so one run's copies overlap another's kernels).

`--impl reference` times the reference's own CPU simplifier (Solver::sigmify
of src/cpu, built by oracle/ref_build.py) on every instance of the same
workload on all host cores; where it is not built, the oracle port.
"""
import argparse
import gc
import concurrent.futures as cf
import json
import multiprocessing as mp
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # plain one-instance GPU path on a Tseitin circuit (the default single-instance line)
    "tseitin": dict(family=1, a=1_000_000, b=50_000, c=1_000, seed=1,
                    desc="Tseitin circuit: 1M 2-input gates (40% AND, 30% OR, 30% XOR) over 50k inputs, "
                         "1k outputs asserted and root-propagated"),
    # uniform random 3-SAT, 20k vars, 85.2k clauses (small enough for the CPU simplifier)
    "ksat": dict(family=0, a=20_000, b=85_200, c=3, seed=1,
                 desc="uniform random 3-SAT, 20,000 vars, 85,200 clauses"),
    # scale-free, 4M vars, 16M clauses, planted model so all 5 rounds run
    "scalefree": dict(family=2, a=4_000_000, b=16_000_000, c=1, seed=1,
                      desc="scale-free CNF, 4M vars, 16M clauses, power-law exponent 2.5, "
                           "geometric lengths on [2,50] mean 4, planted model"),
}

# batched workload: 512 instances per batch, sizes log-uniform on [1e3, 2e5] variables,
# generator per instance uniform over {3-SAT (ratio 4.26), Tseitin, scale-free
# (ratio 4.0, planted)}, per-instance seeds
BATCH = dict(n=512, vmin=1_000, vmax=200_000, seed=7,
             desc="512 instances per batch, log-uniform 1k..200k vars each, generator per instance uniform over "
                  "random 3-SAT (4.26 clauses/var), Tseitin (5% inputs) and scale-free (4 clauses/var, planted)")

# serving workload: Poisson stream of 10,000 jobs, clause counts log-uniform on [1e3, 1e6]
# from the three generators, admitted by a 120 GB device-arena budget, 3 rounds each.
# Jobs are drawn from a pool of seeded instances (with replacement).
SERVE = dict(jobs=10_000, cmin=1_000, cmax=1_000_000, pool=1024, rates=(800.0, 1600.0, 3200.0, 6400.0, 12800.0),
             budget=120_000_000_000, tight_budget=500_000_000, phases=3, slots=4, max_batch=512, clients=8,
             seed=11,
             desc="Poisson arrivals of 10,000 jobs at fixed offered rates, swept until the loop saturates; clause "
                  "counts log-uniform 1e3..1e6 from random 3-SAT / Tseitin / scale-free generators (pool of 1024 "
                  "seeded instances drawn with replacement) submitted by 8 client threads; admission by a 120 GB "
                  "device-arena budget, and once at saturation by a 0.5 GB budget that binds; 3 rounds per job")

METRIC = "inprocessing clauses/s (BVE+SUB)"
UNIT = "clauses/s"


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_cnf(w):
    import parafrost_gb300 as pg
    return pg.generate(w["family"], w["a"], w["b"], w["c"], w["seed"])


def batch_specs(rank=0):
    """(family, a, b, c, seed) of every instance of the batched workload."""
    import numpy as np
    rng = np.random.default_rng(BATCH["seed"] + 1000 * rank)
    specs = []
    for i in range(BATCH["n"]):
        v = int(np.exp(rng.uniform(np.log(BATCH["vmin"]), np.log(BATCH["vmax"]))))
        fam = int(rng.integers(0, 3))
        seed = int(rng.integers(1, 2**31))
        if fam == 0:
            specs.append((0, v, int(round(v * 4.26)), 3, seed))
        elif fam == 1:
            inputs = max(8, v // 20)
            gates = v - inputs
            specs.append((1, gates, inputs, max(1, gates // 1000), seed))
        else:
            specs.append((2, v, 4 * v, 1, seed))
    return specs


def serve_pool(rank=0):
    """Pool of instances with clause counts log-uniform on [cmin, cmax]."""
    import numpy as np
    import parafrost_gb300 as pg
    rng = np.random.default_rng(SERVE["seed"] + 1000 * rank)
    pool = []
    for _ in range(SERVE["pool"]):
        c = float(np.exp(rng.uniform(np.log(SERVE["cmin"]), np.log(SERVE["cmax"]))))
        fam = int(rng.integers(0, 3))
        seed = int(rng.integers(1, 2**31))
        if fam == 0:
            pool.append(pg.generate(0, max(10, int(c / 4.26)), int(c), 3, seed))
        elif fam == 1:
            gates = max(16, int(c / 3.3))
            pool.append(pg.generate(1, gates, max(8, gates // 20), max(1, gates // 1000), seed))
        else:
            pool.append(pg.generate(2, max(10, int(c / 4)), int(c), 1, seed))
    return pool


def serve_stream(pool, jobs, rate, rank=0, budget=None):
    """Submit `jobs` jobs drawn from `pool` with Poisson arrivals at `rate` jobs/s;
    returns throughput, latency percentiles and the server's counters. The
    stream is driven by SERVE["clients"] client threads: client t submits the
    jobs k = t mod clients at their arrival times and fetches their results in
    order, as independent clients of one service would."""
    import threading
    import numpy as np
    import parafrost_gb300 as pg
    rng = np.random.default_rng(SERVE["seed"] + 7 + 1000 * rank)
    picks = rng.integers(0, len(pool), jobs)
    gaps = rng.exponential(1.0 / rate, jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    infos = [None] * jobs
    tickets = [None] * jobs
    P = SERVE["clients"]
    have = [threading.Semaphore(0) for _ in range(P)]
    late = [0.0] * P
    with pg.Server(arena_bytes=budget or SERVE["budget"], slots=SERVE["slots"], max_batch=SERVE["max_batch"],
                   phases=SERVE["phases"]) as srv:
        def collect(t):
            for k in range(t, jobs, P):
                have[t].acquire()
                infos[k] = srv.wait(tickets[k])
                srv.fetch(tickets[k])

        def produce(t, t0):
            for k in range(t, jobs, P):
                dt = t0 + arrivals[k] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                else:
                    late[t] = max(late[t], -dt)
                tickets[k] = srv.submit(pool[picks[k]])
                have[t].release()

        cols = [threading.Thread(target=collect, args=(t,)) for t in range(P)]
        for th in cols:
            th.start()
        t0 = time.perf_counter()
        prods = [threading.Thread(target=produce, args=(t, t0)) for t in range(P)]
        for th in prods:
            th.start()
        for th in prods + cols:
            th.join()
        st = srv.stats()
    lat = np.array([i.latency_s for i in infos]) * 1e3
    qlat = np.array([i.queue_s for i in infos]) * 1e3
    span = (max(i.t_done_ns for i in infos) - min(i.t_submit_ns for i in infos)) * 1e-9
    proc = sum(int(i.clauses_processed) for i in infos)
    return {
        "value": proc / span, "unit": UNIT, "jobs": jobs, "offered_rate_jobs_s": rate,
        "achieved_rate_jobs_s": jobs / span, "span_s": span,
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "p50_queue_ms": float(np.percentile(qlat, 50)), "p99_queue_ms": float(np.percentile(qlat, 99)),
        "clauses_in": int(sum(int(pool[p].num_clauses) for p in picks)), "clauses_processed": proc,
        "errors": int(sum(1 for i in infos if i.rc != 0)),
        "mean_batch": float(np.mean([i.batch_size for i in infos])),
        "max_in_flight_batches": st["max_in_flight_batches"], "max_jobs_in_flight": st["max_jobs_in_flight"],
        "peak_admitted_gb": st["peak_est_bytes"] / 1e9, "budget_gb": st["budget_bytes"] / 1e9,
        "slots": SERVE["slots"], "max_batch": SERVE["max_batch"], "clients": P,
        "producer_max_lateness_s": max(late),
        "latency": "submit to result on the host (admission wait, upload, rounds, download)",
    }


def serve_sweep(pool, jobs, rank=0):
    """The serving stream at rising offered rates until the achieved rate
    falls clearly below the offered one (the loop is saturated), then once
    more at the saturating rate under a budget small enough to bind. The
    reported point is the one with the highest throughput."""
    points = []
    for rate in SERVE["rates"]:
        pt = serve_stream(pool, jobs, rate, rank)
        points.append(pt)
        if pt["achieved_rate_jobs_s"] < 0.9 * rate:
            break
    best = max(points, key=lambda p: p["value"])
    tight = serve_stream(pool, jobs, best["offered_rate_jobs_s"], rank, budget=SERVE["tight_budget"])
    out = dict(best)
    out["desc"] = SERVE["desc"]
    out["saturated"] = points[-1]["achieved_rate_jobs_s"] < 0.9 * points[-1]["offered_rate_jobs_s"]
    keys = ("offered_rate_jobs_s", "achieved_rate_jobs_s", "value", "p50_ms", "p99_ms", "mean_batch",
            "max_jobs_in_flight", "peak_admitted_gb", "budget_gb")
    out["sweep"] = [{k: p[k] for k in keys} for p in points]
    out["budget_bound"] = {k: tight[k] for k in keys + ("p50_queue_ms", "p99_queue_ms", "errors")}
    return out


def make_batch(rank=0, n=None):
    import parafrost_gb300 as pg
    return [pg.generate(*sp) for sp in batch_specs(rank)[:n]]


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(prefix="clocks", suffix=".csv")
        self.p = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx = max(mx, float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---- CPU side: the reference's own CPU simplifier (Solver::sigmify of src/cpu,
# built by oracle/ref_build.py with the timing harness oracle/refcpu/time_main.cpp)
# where it is built, else the oracle port (oracle/pfo.c). Inputs are generated and
# written before any timing; only the simplify calls are timed. ----

REF_CPU_BIN = os.path.join(ROOT, "oracle", "_ref", "pfref_cpu_time")


def _write_instance(args):
    """Generate one instance and write it as DIMACS (spawned worker; loads only
    the host-only generator library)."""
    spec, path = args
    sys.path.insert(0, ROOT)
    import parafrost_gb300 as pg
    cnf = pg.generate(*spec)
    pg.write_dimacs(cnf, path)
    return int(cnf.num_clauses)


def _spec_clauses(spec):
    """Clause count of a generated instance (spawned worker)."""
    sys.path.insert(0, ROOT)
    import parafrost_gb300 as pg
    return int(pg.generate(*spec).num_clauses)


def _port_group(specs):
    """The oracle port on a group of instances, one after another (spawned
    worker): returns (seconds of the simplify calls, clauses processed)."""
    sys.path.insert(0, ROOT)
    import parafrost_gb300 as pg
    from oracle import pyoracle as po
    secs, proc = 0.0, 0
    opts = pg.options_from()
    for sp in specs:
        cnf = pg.generate(*sp)
        t0 = time.perf_counter()
        r = po.simplify(cnf, opts)
        secs += time.perf_counter() - t0
        proc += sum(s["clauses_before"] for s in r.round_stats)
    return secs, proc


def lpt_groups(sizes, k):
    """Longest-processing-time assignment of items to k workers by size."""
    groups, loads = [[] for _ in range(k)], [0] * k
    for i in sorted(range(len(sizes)), key=lambda i: -sizes[i]):
        j = min(range(k), key=loads.__getitem__)
        groups[j].append(i)
        loads[j] += sizes[i]
    return [g for g in groups if g]


class CpuSimplifier:
    """A set of instances simplified on the host cores: `cores` workers, each
    running its share of the instances one after another (one reference
    process per instance). A step's time is the largest sum of simplify times
    over the workers, which run at the same time."""

    def __init__(self, specs, cores):
        self.specs = list(specs)
        self.cores = max(1, min(cores, len(self.specs)))
        self.kind = "reference" if os.path.exists(REF_CPU_BIN) else "port"
        ctx = mp.get_context("spawn")
        uniq = sorted(set(self.specs))
        with cf.ProcessPoolExecutor(min(self.cores, len(uniq)), mp_context=ctx) as pool:
            if self.kind == "reference":
                self.tmp = tempfile.mkdtemp(prefix="pfref_")
                paths = {sp: os.path.join(self.tmp, f"i{k}.cnf") for k, sp in enumerate(uniq)}
                sizes = dict(zip(uniq, pool.map(_write_instance, [(sp, paths[sp]) for sp in uniq])))
                self.paths = [paths[sp] for sp in self.specs]
            else:
                sizes = dict(zip(uniq, pool.map(_spec_clauses, uniq)))
        self.sizes = [sizes[sp] for sp in self.specs]
        self.groups = lpt_groups(self.sizes, self.cores)

    def _run_group(self, idx):
        secs, proc = 0.0, 0
        for i in idx:
            p = subprocess.run([REF_CPU_BIN, self.paths[i], "--verbose=0"], capture_output=True, text=True)
            line = next((x for x in p.stdout.splitlines() if x.startswith("pfref_cpu ")), None)
            if line is None:
                raise RuntimeError(f"reference CPU simplifier gave no result ({p.returncode}): {p.stderr[-500:]}")
            kv = dict(t.split("=") for t in line.split()[1:])
            secs += float(kv["seconds"])
            proc += int(kv["processed"])
        return secs, proc

    def step(self):
        """(seconds, clauses processed, wall seconds) of one pass over the set."""
        t0 = time.perf_counter()
        if self.kind == "reference":
            with cf.ThreadPoolExecutor(len(self.groups)) as ex:
                res = list(ex.map(self._run_group, self.groups))
        else:
            ctx = mp.get_context("spawn")
            with cf.ProcessPoolExecutor(len(self.groups), mp_context=ctx) as pool:
                res = list(pool.map(_port_group, [[self.specs[i] for i in g] for g in self.groups]))
        wall = time.perf_counter() - t0
        return max(r[0] for r in res), sum(r[1] for r in res), wall

    def what(self):
        if self.kind == "reference":
            return "the reference's CPU simplifier (Solver::sigmify of src/cpu, oracle/_ref/pfref_cpu_time)"
        return "the oracle port (oracle/pfo.c)"

    def close(self):
        if self.kind == "reference":
            shutil.rmtree(self.tmp, ignore_errors=True)


def batch_sample(specs, every):
    """Bounded sample of the batched workload: every `every`-th instance."""
    return [sp for i, sp in enumerate(specs) if i % every == 0]


def batch_config():
    """The batched workload as both arms report it."""
    specs = batch_specs(0)
    return {"workload": "batched", "desc": BATCH["desc"], "instances": len(specs),
            "generator_seed": BATCH["seed"], "options": "reference defaults (phases=5, ERE on)",
            "l2": L2_NOTE + "; the batch's clause store is also larger than L2"}


def single_config(wname):
    return {"workload": wname, "desc": WORKLOADS[wname]["desc"], "options": "reference defaults (phases=5, ERE on)",
            "l2": L2_NOTE}


# how the device-timed calls keep the 129 MB L2 from carrying data between steps
L2_NOTE = "GPU arm: a 256 MB buffer is written, and the device synchronized, before every device-timed call"


def run_reference(a, world, rank):
    """The reference's own CPU implementation of the path on all host cores,
    on the same workload as the GPU arm (every instance of the batch, or one
    replica of the single instance per core), each step one full pass."""
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    if a.workload == "batched":
        specs = batch_specs(0)[:a.batch_n]
        config = batch_config()
        if a.batch_n:
            config["instances"] = len(specs)
        sample = f"all {len(specs)} instances of the batch per step"
    else:
        w = WORKLOADS[a.workload]
        specs = [(w["family"], w["a"], w["b"], w["c"], w["seed"])] * cores
        config = single_config(a.workload)
        sample = f"{cores} concurrent replicas of the instance per step"
    cpu = CpuSimplifier(specs, cores)
    for _ in range(a.warmup):
        cpu.step()
    total, proc, walls = 0.0, 0, []
    for _ in range(a.steps):
        secs, p, wall = cpu.step()
        total += secs
        proc += p
        walls.append(wall)
    cpu.close()
    value = proc / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1000.0 * total / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generators)", "config": config,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu.cores, "kind": cpu.kind,
                         "sample": f"{sample}: {cpu.what()}, {len(cpu.groups)} workers on {cores} host cores, each "
                                   f"running its share one instance at a time; a step's time is the largest "
                                   f"per-worker sum of simplify times (parsing and process start excluded)",
                         "wall_ms_per_step": round(1000.0 * statistics.mean(walls), 1)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_line(specs, cores, sample):
    cpu = CpuSimplifier(specs, cores)
    secs, proc, wall = cpu.step()
    cpu.close()
    return {"value": proc / secs, "unit": UNIT, "cores": cpu.cores, "kind": cpu.kind,
            "sample": f"{sample}: {cpu.what()}, {len(cpu.groups)} workers, one pass",
            "wall_ms": round(1000.0 * wall, 1)}


def run_gpu(a, world, rank, local):
    import numpy as np
    import torch
    import parafrost_gb300 as pg

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    from parafrost_gb300.dist import allreduce_max, allreduce_sum

    def max_over_ranks(x):
        return allreduce_max(x, device="cuda")

    def sum_over_ranks(x):
        return allreduce_sum(x, device="cuda")

    w = WORKLOADS[a.workload]
    cnf = make_cnf(w)
    sim = pg.Simplifier()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    for _ in range(a.warmup):
        sim.upload(cnf)
        sim.run()
        sim.download()
    # ---- device-timed region: HBM-resident input, rounds timed with CUDA events ----
    sim.profile(True)
    sim.profile_reset()
    clocks = Clocks(local)
    barrier()
    clocks.start()
    dev_ms, processed, launches, alg = 0.0, 0, 0, 0
    last = None
    t0 = time.perf_counter()
    for _ in range(a.steps):
        sim.upload(cnf)
        flush.fill_(1.0)
        torch.cuda.synchronize()    # the engine's stream does not wait on torch's
        st = sim.run()
        dev_ms += st.device_ms
        processed += st.clauses_processed
        launches += st.kernel_launches
        alg += st.alg_bytes
        last = st
    barrier()
    wall_ms = (time.perf_counter() - t0) * 1000
    clk = clocks.stop()
    prof = sim.profile_report()
    sim.profile(False)
    # ---- end-to-end through the C ABI with host buffers ----
    barrier()
    e2e_s, e2e_proc, h2d, d2h = 0.0, 0, 0, 0
    pcnf = cnf.pinned()     # inputs and results in page-locked host memory, as for the batch
    from parafrost_gb300 import pinned
    rbuf = pinned.ResultBuffers()
    sim.upload(pcnf)
    sim.run()
    sim.download(into=rbuf)  # sizes the result buffers (untimed)
    gc.collect()
    gc.disable()
    for _ in range(a.steps):
        t1 = time.perf_counter()
        sim.upload(pcnf)
        st = sim.run()
        res = sim.download(into=rbuf)
        e2e_s += time.perf_counter() - t1
        e2e_proc += st.clauses_processed
        h2d = cnf.lits.nbytes + cnf.off.nbytes
        d2h = (res.cnf.lits.nbytes + res.cnf.off.nbytes + res.cnf.learnt.nbytes + res.cnf.lbd.nbytes +
               res.cnf.usage.nbytes + res.eliminated.nbytes + res.units.nbytes + res.pending_units.nbytes +
               res.stack.nbytes)
    gc.enable()
    barrier()
    dev_ms_max = max_over_ranks(dev_ms)
    total_proc = sum_over_ranks(processed)
    e2e_max = max_over_ranks(e2e_s)
    e2e_total = sum_over_ranks(e2e_proc)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    value = total_proc / (dev_ms_max / 1000.0)
    # roofline of the dominant kernel group (most device time in the timed region)
    peak, peak_kind = load_peaks()
    # the dominant kernel group of the rounds (the upload's kernels run before them)
    dom_name, dom = max(((k, v) for k, v in prof.items() if v["ms"] > 0 and k not in ("upload", "download")),
                        key=lambda kv: kv[1]["ms"])
    achieved = (dom["alg_bytes"] / 1e9) / (dom["ms"] / 1e3) if dom["ms"] > 0 else 0.0
    roofline = {
        "bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_kind, "traffic": TRAFFIC.get((a.workload, dom_name)),
        "launches": dom["launches"], "ms_per_launch": dom["ms"] / max(1, dom["launches"]),
        "alg_bytes_per_launch": dom["alg_bytes"] / max(1, dom["launches"]),
        "share": dom["ms"] / sum(v["ms"] for v in prof.values()),
        "all_alg_bytes_gbs": (alg / 1e9) / (dev_ms / 1e3),
    }
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": dev_ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded generator)",
        "config": single_config(a.workload),
        "run": {"clauses_in": int(cnf.num_clauses), "literals_in": int(cnf.num_literals),
                "clauses_out": int(last.clauses_out), "rounds": int(last.rounds),
                "l2": "256 MB buffer written between steps; instance working set > L2",
                "parallelism": "replicas only" if world > 1 else "single GPU",
                "wall_ms_per_step_incl_upload": wall_ms / a.steps},
        "e2e": {"value": e2e_total / e2e_max, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000 * e2e_max / a.steps},
        "roofline": roofline,
        "gpu_launches": int(launches),
        "kernel_ms": {k: round(v["ms"] / a.steps, 4) for k, v in prof.items() if v["launches"]},
        "clocks": clk,
    }
    if not a.no_cpu_baseline:
        spec = (w["family"], w["a"], w["b"], w["c"], w["seed"])
        line["cpu_baseline"] = cpu_baseline_line([spec], 1, "the full instance once on one core")
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def result_bytes(res):
    return (res.cnf.lits.nbytes + res.cnf.off.nbytes + res.cnf.learnt.nbytes + res.cnf.lbd.nbytes +
            res.cnf.usage.nbytes + res.eliminated.nbytes + res.units.nbytes + res.pending_units.nbytes +
            res.stack.nbytes)


def run_gpu_batch(a, world, rank, local):
    import torch
    import parafrost_gb300 as pg

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    from parafrost_gb300.dist import allreduce_max, allreduce_sum
    cnfs = make_batch(rank)               # every rank its own batch (weak scaling)
    n = len(cnfs)
    cls_in = sum(int(c.num_clauses) for c in cnfs)
    sim = pg.Simplifier()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    # launch shapes picked by the engine's autotuner on this batch (untimed)
    tuning = sim.autotune(cnfs) if not a.no_autotune else sim.tuning
    for _ in range(a.warmup):
        sim.upload_batch(cnfs)
        sim.run()
    # ---- batched, device-timed: the batch resident in HBM, rounds timed with CUDA events ----
    sim.profile(True)
    sim.profile_reset()
    clocks = Clocks(local)
    barrier()
    clocks.start()
    dev_ms, processed, launches, alg = 0.0, 0, 0, 0
    last = None
    for _ in range(a.steps):
        sim.upload_batch(cnfs)
        flush.fill_(1.0)
        torch.cuda.synchronize()    # the engine's stream does not wait on torch's
        st = sim.run()
        dev_ms += st.device_ms
        processed += st.clauses_processed
        launches += st.kernel_launches
        alg += st.alg_bytes
        last = st
    barrier()
    prof = sim.profile_report()
    sim.profile(False)
    # ---- the same batch as k runs of consecutive instances on k contexts,
    # simplified at once (pfg_simplify_many; device time from one start event
    # every stream waits on to the last context's end) ----
    from parafrost_gb300.simplifier import split_runs
    runs = split_runs([c.num_clauses for c in cnfs], a.streams)
    sims = [sim] + sim.peers(len(runs) - 1)
    for _ in range(2):
        for s_, (b, e) in zip(sims, runs):
            s_.upload_batch(cnfs[b:e])
        pg.run_many(sims)
    barrier()
    mdev_ms, mprocessed, mlaunches = 0.0, 0, 0
    for _ in range(a.steps):
        for s_, (b, e) in zip(sims, runs):
            s_.upload_batch(cnfs[b:e])
        flush.fill_(1.0)
        torch.cuda.synchronize()
        sts, ms = pg.run_many(sims)
        mdev_ms += ms
        mprocessed += sum(st.clauses_processed for st in sts)
        mlaunches += sum(st.kernel_launches for st in sts)
    barrier()
    clk = clocks.stop()
    # ---- plain path on the same instances: one simplify call per instance ----
    for cnf in cnfs[:8]:
        sim.upload(cnf)
        sim.run()
    barrier()
    plain_ms, plain_proc, plain_launches = 0.0, 0, 0
    for cnf in cnfs:
        sim.upload(cnf)
        flush.fill_(1.0)
        torch.cuda.synchronize()    # the engine's stream does not wait on torch's
        st = sim.run()
        plain_ms += st.device_ms
        plain_proc += st.clauses_processed
        plain_launches += st.kernel_launches
    barrier()
    # ---- end to end through the C ABI with host buffers: inputs and results in
    # page-locked host memory, uploaded and downloaded inside the timed region ----
    from parafrost_gb300 import pinned
    pcnfs = [c.pinned() for c in cnfs]
    # the batch goes through simplify_batch(streams=k): k runs of consecutive
    # instances on k contexts and host threads, so one run's copies overlap
    # another's kernels
    rbufs = [pinned.ResultBuffers() for _ in range(a.e2e_streams)]
    sim.simplify_batch(pcnfs, into=rbufs, streams=a.e2e_streams)   # sizes the result buffers (untimed)
    e2e_s, e2e_proc, h2d, d2h = 0.0, 0, 0, 0
    e2e_steps = []
    gc.collect()
    gc.disable()     # no collector pause of this process inside the timed calls
    for _ in range(a.steps):
        t1 = time.perf_counter()
        outs = sim.simplify_batch(pcnfs, into=rbufs, streams=a.e2e_streams)
        e2e_steps.append(time.perf_counter() - t1)
        e2e_s += e2e_steps[-1]
        e2e_proc += sum(int(o.stats["clauses_processed"]) for o in outs)
        h2d = sum(c.lits.nbytes + c.off.nbytes for c in cnfs)
        d2h = sum(result_bytes(o) for o in outs)
    barrier()
    pe2e_s, pe2e_proc = 0.0, 0
    t1 = time.perf_counter()
    for cnf in pcnfs:
        res = sim.simplify(cnf)
        pe2e_proc += int(res.stats["clauses_processed"])
    pe2e_s = time.perf_counter() - t1
    gc.enable()
    barrier()
    serving = None
    if not a.no_serving:
        serving = serve_sweep(serve_pool(rank), a.serve_jobs, rank)
    barrier()
    dev_ms_max = allreduce_max(dev_ms, device="cuda")
    total_proc = allreduce_sum(processed, device="cuda")
    mdev_ms_max = allreduce_max(mdev_ms, device="cuda")
    mtotal_proc = allreduce_sum(mprocessed, device="cuda")
    e2e_max = allreduce_max(e2e_s, device="cuda")
    e2e_total = allreduce_sum(e2e_proc, device="cuda")
    plain_max = allreduce_max(plain_ms, device="cuda")
    plain_total = allreduce_sum(plain_proc, device="cuda")
    pe2e_max = allreduce_max(pe2e_s, device="cuda")
    pe2e_total = allreduce_sum(pe2e_proc, device="cuda")
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    single_value = total_proc / (dev_ms_max / 1000.0)
    value = mtotal_proc / (mdev_ms_max / 1000.0)
    plain_value = plain_total / (plain_max / 1000.0)
    peak, peak_kind = load_peaks()
    # the roofline of the dominant kernel group comes from the one-context run:
    # there a group's launches have the GPU to themselves, so a launch's event
    # time is its own
    dom_name, dom = max(((k, v) for k, v in prof.items() if v["ms"] > 0 and k not in ("upload", "download")),
                        key=lambda kv: kv[1]["ms"])
    achieved = (dom["alg_bytes"] / 1e9) / (dom["ms"] / 1e3) if dom["ms"] > 0 else 0.0
    roofline = {
        "bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_kind, "traffic": TRAFFIC.get(("batched", dom_name)),
        "launches": dom["launches"], "ms_per_launch": dom["ms"] / max(1, dom["launches"]),
        "alg_bytes_per_launch": dom["alg_bytes"] / max(1, dom["launches"]),
        "share": dom["ms"] / sum(v["ms"] for v in prof.values()),
        "all_alg_bytes_gbs": (alg / 1e9) / (dev_ms / 1e3),
        "from": "the one-context run (single_context)",
    }
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": mdev_ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded generators)",
        "config": batch_config(),
        "run": {"instances": n, "clauses_in": cls_in, "literals_in": int(sum(int(c.num_literals) for c in cnfs)),
                "clauses_out": int(last.clauses_out), "max_rounds": int(last.rounds),
                "tuning": dict(tuning, source="pfg_autotune on this batch" if not a.no_autotune else "built-in"),
                "l2": "256 MB buffer written before every timed simplify call (batched and plain)",
                "parallelism": "replicas only" if world > 1 else "single GPU",
                "contexts": len(runs),
                "what": f"the batch as {len(runs)} runs of consecutive instances (about equal clause counts), "
                        f"one context and stream each, simplified at once by pfg_simplify_many"},
        "single_context": {"value": single_value, "unit": UNIT, "ms_per_step": dev_ms_max / a.steps,
                           "gpu_launches": int(launches),
                           "what": "the whole batch in one context (one stream), CUDA events around its rounds"},
        "plain": {"value": plain_value, "unit": UNIT, "ms_per_pass": plain_max,
                  "gpu_launches": int(plain_launches),
                  "e2e": {"value": pe2e_total / pe2e_max, "unit": UNIT, "ms_per_pass": 1000 * pe2e_max},
                  "what": "the same instances, one pfg_upload + pfg_simplify call each"},
        "batched_vs_plain": value / plain_value,
        "serving": serving,
        "served_vs_plain": (serving["value"] / plain_value) if serving else None,
        "e2e": {"value": e2e_total / e2e_max, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000 * e2e_max / a.steps,
                "streams": a.e2e_streams,
                "ms_steps": [round(1000 * t, 2) for t in e2e_steps],
                "ms_median": round(1000 * statistics.median(e2e_steps), 2),
                "ms_p90": round(1000 * sorted(e2e_steps)[min(len(e2e_steps) - 1, int(0.9 * len(e2e_steps)))], 2),
                "spread": "host-link time varies between boxes and calls; median and p90 of the steps beside the "
                          "mean"},
        "roofline": roofline,
        "gpu_launches": int(mlaunches),
        "kernel_ms": {k: round(v["ms"] / a.steps, 4) for k, v in prof.items() if v["launches"]},
        "clocks": clk,
    }
    if not a.no_cpu_baseline:
        specs = batch_sample(batch_specs(0), 4)
        line["cpu_baseline"] = cpu_baseline_line(specs, os.cpu_count() or 1,
                                                 f"every 4th instance of the batch ({len(specs)} instances)")
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# DRAM traffic per launch of the dominant kernel group from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum), keyed by (workload, group).
TRAFFIC = {
    # profiles/ve1w_k_batched.md: all 5 launches on the 64-instance case move 7.65x their algorithmic
    # bytes; a full-batch launch has 218.2 MB algorithmic, so 1.669 GB
    ("batched", "ve_phase1"): 7.645 * 218.2e6,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched", choices=sorted(WORKLOADS) + ["batched"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving stream of the batched line")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched line: built-in launch shapes instead of the autotuner's")
    ap.add_argument("--serve-jobs", type=int, default=SERVE["jobs"])
    ap.add_argument("--streams", type=int, default=4,
                    help="batched value: the batch as k runs on k contexts simplified at once (pfg_simplify_many)")
    ap.add_argument("--e2e-streams", type=int, default=4,
                    help="batched e2e: simplify_batch(streams=k), k contexts overlapping copies and kernels")
    ap.add_argument("--batch-n", type=int, default=None,
                    help="with --single-step or --impl reference: only the first N instances of the batch "
                         "(a small case for profiling and tests)")
    ap.add_argument("--single-step", action="store_true",
                    help="one simplify call of the workload, nothing timed (the command profiled by ncu)")
    ap.add_argument("--groups", action="store_true",
                    help="with --single-step: print each kernel group's launches, event-timed ms and "
                         "algorithmic bytes")
    a = ap.parse_args()
    world, rank, local = dist_setup()
    if a.single_step and a.workload == "batched":
        import parafrost_gb300 as pg
        cnfs = make_batch(0, a.batch_n)
        with pg.Simplifier() as sim:
            if a.groups:
                sim.profile(True)
            outs = sim.simplify_batch(cnfs)
            groups = sim.profile_report() if a.groups else None
        line = {"workload": "batched", "instances": len(outs),
                "clauses_in": int(sum(c.num_clauses for c in cnfs)),
                "literals_in": int(sum(c.num_literals for c in cnfs)),
                "clauses_out": int(sum(o.cnf.num_clauses for o in outs))}
        if groups:
            line["groups"] = {k: v for k, v in groups.items() if v["launches"]}
        print(json.dumps(line))
        return 0
    if a.single_step:
        import parafrost_gb300 as pg
        cnf = make_cnf(WORKLOADS[a.workload])
        with pg.Simplifier() as sim:
            res = sim.simplify(cnf)
        print(json.dumps({"workload": a.workload, "clauses_out": int(res.cnf.num_clauses),
                          "launches": int(res.stats["kernel_launches"])}))
        return 0
    if a.impl == "reference":
        return run_reference(a, world, rank)
    if a.workload == "batched":
        return run_gpu_batch(a, world, rank, local)
    return run_gpu(a, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
