"""Benchmark: accepted transient timesteps per second on one GB300.

Workloads: c2 (default) 1024 Monte Carlo instances of uneven size
(100-3000 transistors, device mismatch) in one launch, a step advancing
every instance by one window of its 2 ns transient; c4 the same form with
4096 instances of 100-5000 transistors; c1 one 10,000-transistor BSIM4
random-logic netlist, the plain drop-in at scale, over the first 500 ps of
its transient; c0 the 32-stage MOS1 inverter chain, 1216 instances, full
20 ns.

Engine arm (default): the GPU transient engine runs `.tran` on the step's
circuits in one launch; a step advances every circuit by one window of its
transient (c0, c1: the whole run).  `value` is device-timed (inputs resident in HBM, CUDA events
around the launches, L2 flushed between steps); `e2e` is the same metric
through the public C ABI starting from host netlist text (compile, upload,
run, read back the accepted points).

Reference arm (--impl reference): the CPU oracle restatement of the
reference transient path (oracle/port) on the host cores, on a bounded
sample of the same workload (see cpu_measure).

Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ngspice-sf-mirror_gb300"))

METRIC = "accepted timesteps/s"
UNIT = "timesteps/s"

# Algorithmic bytes per Newton iteration (8 B per double, 4 B per index):
# distinct fields each device load reads and writes, the matrix and LU
# values the refactorization touches, the solve and convergence vectors.
# BSIM4: 8 x (4 node V + 29 state0 read + 29 state0 write + 15 state1/2 +
# 143 size-dependent parameters + 30 instance scalars + 22 slots + 4 rhs)
# + 4 x 22 slot indices.  Diode: 8 x (3 node V + 22 state0 read/write x 2
# + 4 state1/2 + 27 parameters + 9 slots + 2 rhs) + 4 x 9.
BYTES_MOS1 = 920
BYTES_RES = 72
BYTES_CAP = 136
BYTES_SRC = 120


BYTES_BSIM4 = 2296
BYTES_DIO = 748

DEFAULT_INSTANCES = {"c0": 1216, "c1": 1, "c2": 1024, "c3": 1, "c4": 4096}
DEFAULT_WINDOW = {"c0": "20n", "c1": "500p", "c2": "2n", "c3": "50p", "c4": "2n"}
# transistor-count range of the Monte Carlo instances
MC_RANGE = {"c2": (100, 3000), "c4": (100, 5000)}


def mc_sizes(workload: str, instances: int) -> list[int]:
    """Transistor counts of the Monte Carlo instances: uniform over the
    workload's range, seeded."""
    import random
    lo, hi = MC_RANGE[workload]
    rng = random.Random(20240 if workload == "c2" else 40960)
    return [rng.randint(lo, hi) for _ in range(instances)]


def c2_sizes(instances: int) -> list[int]:
    return mc_sizes("c2", instances)


def workload_texts(name: str, tstop: str | None, instances: int) -> tuple[list[str], dict]:
    """Netlists of one bench step and their description."""
    from ngspice_gb300 import netlists
    tstop = tstop or DEFAULT_WINDOW[name]
    if name == "c0":
        return [netlists.inverter_chain(tstop=tstop)] * instances, {
            "circuit": "32-stage MOS1 CMOS inverter chain (level 1, VTO +-0.7 V, KP 110/50 uA/V^2,"
                       " LAMBDA 0.04, W/L 2u/1u and 4u/1u, VDD 3.3 V, 20 fF loads,"
                       " PULSE(0 3.3 0 100p 100p 2n 4n))",
            "tran": f".tran 10p {tstop}"}
    if name == "c1":
        return [netlists.random_logic(n_transistors=10000, seed=1, tstop=tstop)] * instances, {
            "circuit": "seeded random CMOS logic, 10,000 BSIM4 (level 54) transistors, gate mix"
                       " INV/NAND2/NOR2 40/35/25 %, RC pi nets, 64 PULSE inputs, VDD 1.0 V",
            "tran": f".tran 1p {tstop} (the first {tstop} of the 5n transient)"}
    if name == "c3":
        return [netlists.logic_with_rings(n_transistors=50000, seed=3, rings=16, stages=31,
                                          tstop=tstop)] * instances, {
            "circuit": "seeded random CMOS logic, 50,000 BSIM4 transistors, with 16 embedded"
                       " 31-stage ring oscillators (RC-loaded stages, a 0.2 mA kick each)",
            "tran": f".tran 1p {tstop} (the first {tstop} of the 10n transient)"}
    if name in ("c2", "c4"):
        sizes = mc_sizes(name, instances)
        base = 0 if name == "c2" else 100000
        texts = [netlists.random_logic(n_transistors=n, seed=base + i, tstop=tstop, mismatch=True)
                 for i, n in enumerate(sizes)]
        full = tstop in ("2n", "2000p")
        return texts, {
            "circuit": f"{instances} Monte Carlo instances of seeded random BSIM4 logic,"
                       f" {min(sizes)}-{max(sizes)} transistors ({sum(sizes)} total), per-device"
                       " mismatch vth0 N(nom, 15 mV), toxe N(nom, 2 %), W N(nom, 3 %)",
            "tran": f".tran 1p {tstop}" + ("" if full else f" (the first {tstop} of the 2n transient)"),
            "sizes": sizes}
    raise SystemExit(f"unknown workload {name}")


def progress(msg: str) -> None:
    """One progress line on stderr (the JSON result line alone goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def bytes_per_iteration(w: dict) -> int:
    n, nnz, nlu = w["n"], w["nnz"], w["nlu"]
    return (BYTES_BSIM4 * w["bsim4"] + BYTES_MOS1 * w["mos1"] + BYTES_DIO * w["dio"]
            + BYTES_RES * w["res"] + BYTES_CAP * w["cap"]
            + BYTES_SRC * (w["vsrc"] + w["isrc"])
            + 8 * nnz + 12 * nlu          # refactorization
            + 12 * nlu + 24 * n           # forward/backward substitution
            + 24 * n)                     # convergence test


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.p = None
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                      text=True)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, flag in zip(names, f[4:8]):
                if flag.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def flush_l2():
    """Write a buffer larger than the 129 MB L2 between timed steps."""
    try:
        import torch
        if torch.cuda.is_available():
            buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
            buf.fill_(1)
            torch.cuda.synchronize()
            del buf
    except Exception:
        pass


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


# ---------------------------------------------------------------------------
# CPU oracle (reference arm and cpu_baseline)
# ---------------------------------------------------------------------------
def _cpu_one(text: str) -> tuple[int, float]:
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import port
    t0 = time.perf_counter()
    r = port.simulate(text)
    return int(r["stats"]["accepted"]), time.perf_counter() - t0


def cpu_pool(texts: list[str], procs: int) -> tuple[int, float]:
    """Run the oracle port on every netlist, `procs` processes (spawned);
    returns (accepted steps, makespan seconds)."""
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_one, texts, chunksize=1)
    return sum(a for a, _ in res), time.perf_counter() - t0


def cpu_measure(args) -> dict:
    """One bounded CPU sample of the workload on the host cores.

    c0/c2/c4: independent instances, one port process per core over a
    sample of the instances (throughput = accepted steps / makespan).
    c1/c3: one circuit; the port is single-threaded, so one core; the rate
    is the marginal one between two windows of the same netlist (20p and
    50p; 3p and 8p for the 50,000-transistor c3), accepted steps and
    seconds of the difference, which leaves out the operating point and
    favours the CPU."""
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import port
    port.build()
    procs = os.cpu_count() or 1
    if args.workload == "c1":
        from ngspice_gb300 import netlists
        short = netlists.random_logic(n_transistors=10000, seed=1, tstop="20p")
        long_ = netlists.random_logic(n_transistors=10000, seed=1, tstop="50p")
        a1, t1 = _cpu_one(short)
        a2, t2 = _cpu_one(long_)
        return {"value": (a2 - a1) / max(t2 - t1, 1e-9), "cores": 1, "seconds": t1 + t2,
                "sample": f"C1 netlist on 1 core (single-threaded port): accepted steps between the"
                          f" 20p and 50p windows ({a2 - a1} steps in {t2 - t1:.1f} s; operating"
                          f" point excluded)"}
    if args.workload == "c3":
        from ngspice_gb300 import netlists
        short = netlists.logic_with_rings(n_transistors=50000, seed=3, tstop="3p")
        long_ = netlists.logic_with_rings(n_transistors=50000, seed=3, tstop="8p")
        a1, t1 = _cpu_one(short)
        a2, t2 = _cpu_one(long_)
        return {"value": (a2 - a1) / max(t2 - t1, 1e-9), "cores": 1, "seconds": t1 + t2,
                "sample": f"C3 netlist on 1 core (single-threaded port): accepted steps between the"
                          f" 3p and 8p windows ({a2 - a1} steps in {t2 - t1:.1f} s; operating"
                          f" point excluded)"}
    if args.workload == "c0":
        texts, _ = workload_texts(args.workload, args.tstop, args.instances)
        sample = args.cpu_sample or 4 * procs
        batch = [texts[0]] * sample
        a, dt = cpu_pool(batch, procs)
        return {"value": a / dt, "cores": procs, "seconds": dt,
                "sample": f"{len(batch)} of the step's instances across {procs} processes"
                          f" ({a} accepted steps in {dt:.1f} s)"}
    # Monte Carlo: instances spread over the sorted sizes, each over the
    # first cpu_window of its transient (operating point included), one
    # process per core; throughput = accepted steps / makespan
    win = args.cpu_window
    texts, tdesc = workload_texts(args.workload, win, args.instances)
    sample = args.cpu_sample or 2 * procs
    batch = [texts[i] for i in plain_sample(texts, tdesc.get("sizes"), sample)]
    a, dt = cpu_pool(batch, procs)
    return {"value": a / dt, "cores": procs, "seconds": dt,
            "sample": f"{len(batch)} of the step's instances (spread over the sorted sizes),"
                      f" each over .tran 1p {win} (operating point included), across {procs}"
                      f" processes ({a} accepted steps in {dt:.1f} s)"}


def cpu_arm(args, wdesc) -> dict:
    times, vals, desc = [], [], ""
    for _ in range(args.steps):
        m = cpu_measure(args)
        vals.append(m["value"])
        times.append(m["seconds"])
        desc = m["sample"]
        cores = m["cores"]
    value = statistics.mean(vals)
    return {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {k: v for k, v in wdesc.items() if not k.startswith("_")},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": desc + " (oracle restatement, oracle/port)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# engine arm
# ---------------------------------------------------------------------------
def plain_sample(texts: list[str], sizes: list[int] | None, k: int) -> list[int]:
    """Indices of k instances spread evenly over the sorted sizes (the
    plain drop-in is timed on them, one circuit per call)."""
    n = len(texts)
    k = max(1, min(k, n))
    order = sorted(range(n), key=lambda i: (sizes[i] if sizes else 0, i))
    return [order[(2 * j + 1) * n // (2 * k)] for j in range(k)]


class Windows:
    """Steps of a windowed batched transient: step j advances every circuit
    to the end of window j of the transient (ngsf_run_window), cycling: the
    step after the last window starts fresh runs.  Returns per step the
    device seconds and, per circuit, the accepted steps, Newton iterations
    and rejected steps made in the window."""

    def __init__(self, E, circuits, dt: float, tstop: float):
        self.E, self.cs, self.dt, self.tstop = E, circuits, dt, tstop
        self.nw = max(1, int(round(tstop / dt)))
        self.j = 0
        n = len(circuits)
        self.prev = [(0, 0, 0)] * n
        self.fresh = [True] * n
        self.failed = {}      # instance -> engine status; failed instances leave the batch

    def step(self):
        E = self.E
        w = self.j % self.nw
        t_end = (w + 1) * self.dt if w < self.nw - 1 else 2.0 * self.tstop
        live = [i for i in range(len(self.cs)) if i not in self.failed]
        sec = E.run_window([self.cs[i] for i in live], t_end)
        gained = [(0, 0, 0)] * len(self.cs)
        for i in live:
            r = self.cs[i].results()
            st = int(r[E.R_STATUS])
            now = (int(r[E.R_ACCEPTED]), int(r[E.R_NUMITER]), int(r[E.R_REJECTED]))
            base = (0, 0, 0) if self.fresh[i] else self.prev[i]
            gained[i] = tuple(x - y for x, y in zip(now, base))
            self.prev[i] = now
            self.fresh[i] = st == 0
            if st not in (0, E.PAUSED):
                self.failed[i] = st
                progress(f"instance {i} stopped with engine status {st} at"
                         f" {r[E.R_ACCEPTED]} accepted steps; it leaves the batch")
        self.j += 1
        return sec, gained


def seconds_of(t: str) -> float:
    """A time with a SPICE scale suffix ("25p", "2n", "1e-9")."""
    scale = {"f": 1e-15, "p": 1e-12, "n": 1e-9, "u": 1e-6, "m": 1e-3}
    t = t.strip().lower()
    if t and t[-1] in scale:
        return float(t[:-1]) * scale[t[-1]]
    return float(t)


def replica_totals(seconds: float, accepted: float, world: int, device: str) -> tuple:
    """Whole-job figures of N replicas (one per rank, the same workload
    each): the slowest rank's device time and the accepted steps of all
    ranks (an all-reduce over the process group; a single process returns
    its own)."""
    if world <= 1:
        return seconds, accepted
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    a = torch.tensor([float(accepted)], dtype=torch.float64, device=device)
    dist.all_reduce(a, op=dist.ReduceOp.SUM)
    return float(t.item()), float(a.item())


def engine_arm(args, texts, wdesc, rank, world) -> dict | None:
    from ngspice_gb300 import engine as E
    mc = args.workload in ("c2", "c4")
    # one observed node per instance for the batches (c0: the chain's
    # output, c2/c4: the first gate output); every unknown for the single c1
    probes = {"c0": ["n32"], "c1": None, "c2": ["y0"], "c3": ["ro0_0", "ro15_0", "y0"],
              "c4": ["y0"]}[args.workload]
    outcap = 8192 if args.workload in ("c1", "c3") else (4096 if mc else 1024)
    if mc:
        # Monte Carlo batch: instances stop after their first accepted step
        # until no instance still pauses for new pivots (operating point,
        # MODEINITTRAN), then run their time loops in one launch
        os.environ.setdefault("NGSF_HOLD", "1")

    def open_all(txts):
        # a batch opens through ngsf_open_many (parsing on all host cores)
        if len(txts) > 1:
            return E.open_many(txts, probes=probes, outcap=outcap)
        return [E.Circuit(txts[0], probes=probes, outcap=outcap)]

    tb = time.perf_counter()
    circuits = open_all(texts)
    wls = [c.workload() for c in circuits]
    progress(f"compiled and uploaded {len(circuits)} circuits in {time.perf_counter() - tb:.1f} s")
    tuned = None
    if len(circuits) == 1 and circuits[0].wide_info()[0] and not args.no_tune:
        # one large circuit over the whole grid: the refactorization shape
        # is autotuned over its level schedule (every shape gives the same
        # bits); the tuning runs are short and untimed
        tt = time.perf_counter()
        tuned = E.tune_factor_shape(circuits[0])
        progress(f"refactorization shape {tuned['blocks']} blocks, one-block levels up to"
                 f" {tuned['small_work']} updates ({time.perf_counter() - tt:.1f} s)")
    tstop = seconds_of(args.tstop or DEFAULT_WINDOW[args.workload])
    dt = seconds_of(args.window) if mc else tstop
    win = Windows(E, circuits, dt, tstop) if mc else None

    def one_step():
        if win:
            return win.step()
        sec = E.run(circuits)
        g = []
        for i, c in enumerate(circuits):
            r = c.results()
            if r[E.R_STATUS] != 0:
                raise SystemExit(f"engine status {r[E.R_STATUS]} on instance {i}")
            g.append((int(r[E.R_ACCEPTED]), int(r[E.R_NUMITER]), int(r[E.R_REJECTED])))
        return sec, g

    for k in range(args.warmup):
        tw = time.perf_counter()
        sec, _ = one_step()
        progress(f"warm-up {k}: {sec:.3f} s device, {time.perf_counter() - tw:.1f} s wall,"
                 f" {E.last_launches()} launches")
    first_timed_window = win.j if win else 0
    clocks = Clocks()
    dev_times, accepted, launches, rejected = [], 0, 0, 0
    iters_of = [0] * len(circuits)
    for _ in range(args.steps):
        flush_l2()
        sec, g = one_step()
        dev_times.append(sec)
        launches += E.last_launches()
        for i, (a, it, rj) in enumerate(g):
            accepted += a
            iters_of[i] += it
            rejected += rj
        progress(f"step {len(dev_times) - 1}: {sec:.3f} s device, {E.last_launches()} launches,"
                 f" {sum(x[0] for x in g)} accepted steps")
    clk = clocks.stop()
    iters = sum(iters_of)
    moved = sum(bytes_per_iteration(w) * k for w, k in zip(wls, iters_of))
    total = sum(dev_times)
    total, accepted_all = replica_totals(total, accepted, world, "cuda")
    value = accepted_all / total
    lu_madds = [c.lu_flops() for c in circuits]
    # free the timed batch (device memory and host images) before the
    # end-to-end pass opens the workload again
    failed = dict(win.failed) if win else {}
    n_windows = win.nw if win else 0
    win = None
    del circuits

    # e2e: host netlist text -> compile/upload -> run -> accepted points on
    # host, through the public C ABI (a Monte Carlo batch over the first
    # e2e_window of its transient, operating point included)
    def e2e_run(txts):
        t0 = time.perf_counter()
        h2d = d2h = acc = 0
        cs = open_all(txts)
        if mc:
            E.run_window(cs, seconds_of(args.e2e_window))
        else:
            E.run(cs)
        for c in cs:
            tt, vv = c.points()
            d2h += tt.nbytes + vv.nbytes
            acc += int(c.results()[E.R_ACCEPTED])
            h2d += c.device_bytes()
        del cs
        return acc, time.perf_counter() - t0, h2d, d2h

    e2e_acc, e2e_time, h2d, d2h = e2e_run(texts)
    progress(f"end-to-end pass: {e2e_time:.1f} s wall, {e2e_acc} accepted steps")
    e2e = {"value": world * e2e_acc / e2e_time, "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "includes": "netlist compile, symbolic analysis, upload, run, read-back"
                       + (f"; the first {args.e2e_window} of every instance's transient"
                          if mc else "")}

    out_extra = {}
    if mc and args.plain_sample > 0:
        # the plain drop-in on a sample of the same instances: one circuit
        # per call through the same C ABI (a circuit of >= 1024 transistors
        # alone in a call runs over the whole grid), timed over the same
        # windows as the batched steps; and end to end over e2e_window
        os.environ["NGSF_HOLD"] = "0"
        idx = plain_sample(texts, wdesc.get("_sizes"), args.plain_sample)
        p_acc = p_dev = 0.0
        p_iters = 0
        pe_acc = pe_wall = 0.0
        for i in idx:
            c = open_all([texts[i]])[0]
            pw = Windows(E, [c], dt, tstop)
            for _ in range(first_timed_window):
                pw.step()
            sec_i = acc_i = 0
            for _ in range(args.steps):
                sec, g = pw.step()
                sec_i += sec
                acc_i += g[0][0]
                p_iters += g[0][1]
            c.close()
            a2, w2, _, _ = e2e_run([texts[i]])
            p_acc += acc_i
            p_dev += sec_i
            pe_acc += a2
            pe_wall += w2
            progress(f"plain instance {i} ({wdesc['_sizes'][i]} transistors): {sec_i:.3f} s"
                     f" device for {acc_i} steps; end to end {w2:.1f} s for {a2} steps")
        os.environ["NGSF_HOLD"] = "1"
        plain = p_acc / p_dev
        plain_e2e = pe_acc / pe_wall
        out_extra["forms"] = {
            "batched": {"value": value, "e2e": e2e["value"], "instances": len(texts)},
            "plain_gpu": {"value": plain, "e2e": plain_e2e, "instances": len(idx),
                          "newton_iterations_per_accepted_step": p_iters / max(p_acc, 1),
                          "sample": f"{len(idx)} instances spread over the sorted sizes, each"
                                    " alone in its own call, timed over the same windows as the"
                                    " batched steps (device time); e2e from netlist text over"
                                    f" the first {args.e2e_window}"},
            "batched_vs_plain": value / plain,
            "batched_vs_plain_e2e": e2e["value"] / plain_e2e}
    if mc and args.predictors:
        # the batched form with a Newton predictor on every instance, over
        # the same windows: 3 = the quadratic polynomial guess, 2 = that
        # plus the learned network's correction (trained here on the GPU on
        # plain trajectories of seeded random-logic circuits with device
        # mismatch, 100-1040 transistors over 300 ps, seeds disjoint from
        # the workload's; untimed)
        forms = out_extra.setdefault("forms", {})
        for kind in [int(k) for k in args.predictors.split(",") if k.strip()]:
            params, train_info = None, None
            if kind == 2:
                params, train_info = train_network(args)
                progress(f"network trained in {train_info['seconds']:.1f} s")
            cs = open_all(texts)
            for c in cs:
                c.set_predictor(kind, params)
            pw = Windows(E, cs, dt, tstop)
            for _ in range(first_timed_window):
                pw.step()
            k_sec = k_acc = k_it = 0
            for _ in range(args.steps):
                flush_l2()
                sec, g = pw.step()
                k_sec += sec
                k_acc += sum(x[0] for x in g)
                k_it += sum(x[1] for x in g)
            guesses = sum(int(c.results()[E.R_GUESSES]) for c in cs)
            first = sum(int(c.results()[E.R_GUESS1]) for c in cs)
            pw = None
            del cs
            name = {3: "batched_quadratic_guess", 2: "batched_learned"}.get(kind, f"batched_k{kind}")
            forms[name] = {"value": k_acc / k_sec, "newton_iterations_per_accepted_step":
                           k_it / max(k_acc, 1), "accepted_on_first_iteration": first,
                           "steps_from_a_guess": guesses}
            if train_info:
                forms[name]["training"] = train_info
            if "plain_gpu" in forms:
                forms[name + "_vs_plain"] = (k_acc / k_sec) / forms["plain_gpu"]["value"]
            progress(f"{name}: {k_acc / k_sec:.1f} accepted steps/s,"
                     f" {k_it / max(k_acc, 1):.3f} Newton iterations per step")
    if args.workload == "c3" and args.predictors:
        # the single large circuit with the Newton predictors: the same run
        # from the quadratic guess (3) and with the learned correction (2),
        # against the plain start timed above
        forms = out_extra.setdefault("forms", {})
        forms["plain"] = {"value": value, "newton_iterations_per_accepted_step":
                          iters / max(accepted, 1)}
        for kind in [int(k) for k in args.predictors.split(",") if k.strip()]:
            params, train_info = None, None
            if kind == 2:
                params, train_info = train_network(args)
                progress(f"network trained in {train_info['seconds']:.1f} s")
            c = open_all(texts)[0]
            if tuned:
                c.set_factor_shape(tuned["blocks"], tuned["small_work"])
            c.set_predictor(kind, params)
            k_sec = E.run([c])
            r = c.results()
            name = {3: "quadratic_guess", 2: "learned"}.get(kind, f"k{kind}")
            forms[name] = {"value": int(r[E.R_ACCEPTED]) / k_sec, "status": int(r[E.R_STATUS]),
                           "newton_iterations_per_accepted_step":
                               int(r[E.R_TRANITER]) / max(int(r[E.R_ACCEPTED]), 1),
                           "accepted_on_first_iteration": int(r[E.R_GUESS1]),
                           "steps_from_a_guess": int(r[E.R_GUESSES])}
            if train_info:
                forms[name]["training"] = train_info
            forms[name + "_vs_plain"] = forms[name]["value"] / value
            progress(f"{name}: {forms[name]['value']:.1f} accepted steps/s,"
                     f" {forms[name]['newton_iterations_per_accepted_step']:.3f} Newton"
                     " iterations per step")
            c.close()
    if tuned:
        out_extra["refactor_shape"] = {"blocks": tuned["blocks"],
                                       "one_block_levels_up_to": tuned["small_work"]}
    if failed:
        out_extra["failed_instances"] = {str(i): st for i, st in failed.items()}
    if mc:
        out_extra["windows"] = {
            "window": args.window, "transient": args.tstop or DEFAULT_WINDOW[args.workload],
            "timed": f"windows {first_timed_window}..{first_timed_window + args.steps - 1}"
                     f" (cycling over {n_windows} windows of the transient; the window after the"
                     " last one starts fresh runs)"}

    pk = peaks()
    fp64_peak = E.fp64_peak()
    achieved = moved / total / 1e9
    kernel = "tran_wide_kernel" if (len(texts) <= 4 and wls[0]["bsim4"] + wls[0]["mos1"] >= 1024) \
        else "tran_kernel"
    # DRAM bytes per circuit Newton iteration measured with ncu
    # (dram__bytes_read + dram__bytes_write of one launch over the Newton
    # iterations it ran): the C1 time-loop launch of the first 3 ps, 66.3 MB
    # over about 120 iterations (the working set stays in L2); a timed
    # window of the first 76 C2 instances, 76.65 GB over 8,637 circuit
    # iterations, 2.21x their 4,014,764 algorithmic bytes per iteration
    # (76 circuit arenas do not fit L2 together).  A Monte Carlo batch
    # scales that ratio by its own algorithmic bytes per iteration.
    per_iter = moved / max(iters, 1)
    traffic = {"c1": 66.3e6 / 120,
               "c2": per_iter * (76.652e9 / 8637) / 4014764,
               "c4": per_iter * (76.652e9 / 8637) / 4014764}.get(args.workload)
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"],
            "traffic": traffic, "traffic_unit": "bytes per Newton iteration" if traffic else None,
            "peak_source": pk["src"], "kernel": kernel,
            "algorithmic_bytes_per_newton_iteration": moved // max(iters, 1)}
    # the binding roof: FP64.  Flops per Newton iteration: the BSIM4
    # evaluations (FLOPS_BSIM4 each), the refactorization (2 per
    # multiply-add of the circuit's pivot plan) and the two triangular
    # solves (2 per L+U entry)
    flops = sum(k * (FLOPS_BSIM4 * w["bsim4"] + 2.0 * lf + 2.0 * w["nlu"])
                for w, k, lf in zip(wls, iters_of, lu_madds))
    roof_fp64 = {"bound": "fp64", "achieved": flops / total / 1e12, "peak": fp64_peak / 1e12,
                 "unit": "TFLOP/s", "frac": flops / total / fp64_peak, "traffic": None,
                 "peak_source": "measured in this run: FP64 fused multiply-add chains on every"
                                " SM (ngsf_fp64_peak); MEASURED_PEAKS.json holds no FP64 figure",
                 "kernel": kernel, "flops_per_newton_iteration": flops / max(iters, 1),
                 "flops_per_bsim4_evaluation": FLOPS_BSIM4}
    cfg = {k: v for k, v in wdesc.items() if not k.startswith("_")}
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * total / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": cfg, "clocks": clk, "e2e": e2e,
           "gpu_launches": launches, "roofline": roof_fp64, "roofline_hbm": roof,
           "newton_iterations_per_s": iters * world / total,
           "newton_iterations_per_accepted_step": iters / max(accepted, 1),
           "rejected_steps": rejected}
    out.update(out_extra)
    if rank == 0 and not args.no_cpu_baseline:
        m = cpu_measure(args)
        out["cpu_baseline"] = {"value": m["value"], "unit": UNIT, "cores": m["cores"],
                               "kind": "port", "sample": m["sample"]}
    return out


# FP64 operations of one BSIM4 evaluation (default selectors, transient
# Newton iteration): counted once with ncu over the grid-wide evaluation
# kernel on the 10,000-transistor netlist (python bench.py
# --device-eval-only --eval-reps 1; sm__sass_thread_inst_executed_op_
# {dadd,dmul,dfma}_pred_on = 7,974,223 + 11,682,109 + 23,174,884 FP64
# instructions over 10,002 evaluations, a fused multiply-add counted as 2
# flops): 6,599 flops in 4,282 FP64 instructions per evaluation.
FLOPS_BSIM4 = 6599
DP_INSTRUCTIONS_BSIM4 = 4282


def device_eval(args) -> dict:
    """Stand-alone timing of the BSIM4 device evaluation over the
    10,000-transistor netlist's instances (the transient's device function,
    one instance per grid thread), against the measured FP64 peak."""
    from ngspice_gb300 import engine as E, netlists
    text = netlists.random_logic(n_transistors=10000, seed=1, tstop="5p")
    c = E.Circuit(text, outcap=16)
    E.run([c])                      # a realistic linearisation point: 5 ps in
    r = c.results()
    pt = E.make_point(time=5e-12, delta=1e-13, deltaOld=(1e-13, 1e-13, 1e-13),
                      ag=(2e13, -2e13), gmin=1e-12, mode=0x1 | 0x100, order=1)
    reps = args.eval_reps
    sec = c.eval_bench(pt, 1 << E.DEV_BSIM4, reps=reps)
    nb4 = c.workload()["bsim4"]
    evals = reps * nb4 / sec
    peak = E.fp64_peak()
    out = {"instances": nb4, "reps": reps, "seconds": sec, "evaluations_per_s": evals,
           "fp64_peak_measured_flops": peak, "transient_steps_before": int(r[E.R_ACCEPTED])}
    if FLOPS_BSIM4:
        out["flops_per_evaluation"] = FLOPS_BSIM4
        out["fp64_frac"] = evals * FLOPS_BSIM4 / peak
    c.close()
    return out


def gnn_case(nodes: int, steps: int = 3) -> dict:
    """Training steps of the predictor network on a seeded graph of `nodes`
    nodes (6 random neighbours within a window of 100): the tcgen05
    forward and backward products at a size a batched timestep feeds."""
    from ngspice_gb300 import gnn as G, predictor
    import numpy as np
    rng = np.random.default_rng(0)
    nbs = [set() for _ in range(nodes)]
    for i in range(nodes):
        for j in rng.integers(max(0, i - 50), min(nodes, i + 50), 6):
            if int(j) != i:
                nbs[i].add(int(j))
                nbs[int(j)].add(i)
    ptr, idx = [0], []
    for i in range(nodes):
        idx += sorted(nbs[i])
        ptr.append(len(idx))
    net = G.Net(np.array(ptr, np.int32), np.array(idx, np.int32))
    net.set_params(predictor.init_params(0))
    X = rng.standard_normal((nodes, G.F_IN)).astype(np.float32)
    y = rng.standard_normal(nodes).astype(np.float32)
    w = np.ones(nodes, np.float32)
    t0 = time.perf_counter()
    loss = None
    for _ in range(steps):
        loss, _ = net.train_step(X, y, w, 1e-3)
    out = {"gnn_nodes": nodes, "steps": steps, "loss": float(loss),
           "seconds": time.perf_counter() - t0}
    net.close()
    return out


def train_network(args) -> tuple:
    """The bench's predictor network: trained on the GPU on plain
    trajectories of seeded random-logic circuits with device mismatch
    (100-1040 transistors over 300 ps, seeds disjoint from the
    workloads')."""
    from ngspice_gb300 import netlists, predictor
    tt = time.perf_counter()
    train = [netlists.random_logic(n_transistors=100 + 20 * s, seed=900000 + s, tstop="300p",
                                   mismatch=True) for s in range(args.learn_circuits)]
    data = predictor.collect(train)
    params, losses = predictor.train(data, steps=args.learn_steps, lr=args.learn_lr)
    info = {"circuits": args.learn_circuits, "steps": args.learn_steps, "lr": args.learn_lr,
            "seconds": time.perf_counter() - tt,
            "loss_first": float(losses[0]), "loss_last": float(losses[-1])}
    return params, info


def predictor_study(args) -> dict:
    """Newton iterations per accepted step of 8 held-out instances of the
    C2 distribution (200-2000 transistors, device mismatch, seeds 700000+,
    300 ps) from the reference's start (0), the linear (1) and quadratic (3)
    guesses and the quadratic guess with the trained network (2)."""
    import numpy as np
    from ngspice_gb300 import netlists, predictor
    rng = np.random.default_rng(7)
    test = [netlists.random_logic(n_transistors=int(n), seed=700000 + i, tstop="300p",
                                  mismatch=True)
            for i, n in enumerate(rng.integers(200, 2000, 8))]
    params, info = train_network(args)
    res = predictor.evaluate(test, params, kinds=(0, 1, 3, 2))
    out = {"study": "Newton predictor", "held_out": "8 C2-distribution instances, 300 ps",
           "training": info}
    for k, name in ((0, "plain"), (1, "linear"), (3, "quadratic"), (2, "network")):
        r = res[k]
        out[name] = {"iterations_per_step": r["iterations_per_step"],
                     "accepted_steps": r["accepted"], "status": r["status"],
                     "accepted_on_first_iteration": r["first_iteration"],
                     "steps_from_a_guess": r["guesses"], "plain_retries": r["fallbacks"]}
    return out


def phase_split(args, texts) -> None:
    """Per-phase clock split of one untimed run of the workload (circuits
    opened with NGSF_PHASES=1, so the timed runs carry no clock reads)."""
    from ngspice_gb300 import engine as E
    os.environ["NGSF_PHASES"] = "1"
    if args.workload in ("c2", "c4"):
        os.environ.setdefault("NGSF_HOLD", "1")
    try:
        cs = E.open_many(texts, probes=None if args.workload == "c1" else ["vdd"], outcap=16) \
            if len(texts) > 1 else [E.Circuit(texts[0], outcap=16)]
        sec = E.run(cs)
        tot = {}
        for c in cs:
            for k, v in c.phase_cycles().items():
                tot[k] = tot.get(k, 0) + v
        busy = sum(tot[k] for k in ("load", "gather", "factor", "solve", "conv", "trunc"))
        split = {k: tot[k] / tot["total"] for k in ("load", "gather", "factor", "solve", "conv",
                                                     "trunc")}
        split["rest"] = 1.0 - busy / tot["total"]
        per_it = {k: tot[k] / max(tot["iterations"], 1) for k in
                  ("load", "gather", "factor", "solve", "conv")}
        print(json.dumps({"phases": split, "cycles_per_newton_iteration": per_it,
                          "block_cycles": tot["total"], "newton_iterations": tot["iterations"],
                          "device_seconds": sec, "circuits": len(cs)}), file=sys.stderr,
              flush=True)
        del cs
    finally:
        os.environ.pop("NGSF_PHASES", None)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c0", "c1", "c2", "c3", "c4"])
    ap.add_argument("--window", default="25p",
                    help="Monte Carlo workloads: a step advances every instance by this much of"
                         " its transient")
    ap.add_argument("--e2e-window", default="200p",
                    help="Monte Carlo workloads: transient span of the end-to-end pass")
    ap.add_argument("--predictors", default="3,2",
                    help="Monte Carlo workloads: Newton predictors also timed on the batch"
                         " (3 quadratic guess, 2 with the learned network; empty: none)")
    ap.add_argument("--learn-circuits", type=int, default=48)
    ap.add_argument("--learn-steps", type=int, default=4000)
    ap.add_argument("--learn-lr", type=float, default=3e-3)
    ap.add_argument("--plain-sample", type=int, default=4,
                    help="instances of a Monte Carlo workload timed through the plain drop-in")
    ap.add_argument("--instances", type=int, default=0,
                    help="instances per launch (default: 1216 for c0, 1 for c1, 1024 for c2)")
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--cpu-window", default="100p",
                    help="transient window of each Monte Carlo instance in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the refactorization-shape autotuner of a single large circuit")
    ap.add_argument("--phases", action="store_true",
                    help="one extra untimed run with per-phase SM clock records: prints the"
                         " split of each circuit block's time (loads, gather, refactor, solves,"
                         " convergence, truncation error, the rest) as one JSON line on stderr")
    ap.add_argument("--device-eval", action="store_true",
                    help="also time the BSIM4 evaluation alone over the 10,000-transistor"
                         " netlist and the FP64 peak (one JSON line on stderr, and a"
                         " device_eval key in the result)")
    ap.add_argument("--eval-reps", type=int, default=20)
    ap.add_argument("--gnn-steps", type=int, default=0,
                    help="profiling case: this many training steps of the predictor network"
                         " on a seeded graph of --gnn-nodes nodes, then stop")
    ap.add_argument("--gnn-nodes", type=int, default=8192)
    ap.add_argument("--predictor-study", action="store_true",
                    help="train the bench's network and compare the Newton starts on held-out"
                         " instances (one JSON line)")
    ap.add_argument("--device-eval-only", action="store_true",
                    help="print the device_eval JSON line and stop (profiling case)")
    ap.add_argument("--tstop", default=None,
                    help="shorter .tran stop time (small cases for profiling)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    args.instances = args.instances or DEFAULT_INSTANCES[args.workload]
    if args.predictor_study:
        print(json.dumps(predictor_study(args)))
        return
    if args.gnn_steps:
        print(json.dumps(gnn_case(args.gnn_nodes, args.gnn_steps)))
        return
    if args.device_eval_only:
        print(json.dumps({"device_eval": device_eval(args)}))
        return
    texts, tdesc = workload_texts(args.workload, args.tstop, args.instances)
    steps_desc = (f", a step advances every instance by a {args.window} window of its"
                  " transient" if args.workload in ("c2", "c4") else "")
    wdesc = {"workload": f"{args.workload.upper()}: {tdesc['circuit']}, {tdesc['tran']},"
                         f" {args.instances} independent instance(s) per launch{steps_desc}",
             "instances_per_gpu": args.instances, "l2": "flushed between timed steps",
             "parallelism": f"replicas x{world}", "_sizes": tdesc.get("sizes")}
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(cpu_arm(args, wdesc)))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        dist.barrier()
    if args.phases:
        phase_split(args, texts)
    dev_eval = None
    if args.device_eval:
        dev_eval = device_eval(args)
        print(json.dumps({"device_eval": dev_eval}), file=sys.stderr, flush=True)
    out = engine_arm(args, texts, wdesc, rank, world)
    if dev_eval:
        out["device_eval"] = dev_eval
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
