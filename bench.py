"""Benchmark: accepted transient timesteps per second on one GB300.

Engine arm (default): the GPU transient engine runs `.tran` on a batch of
independent circuit instances in one launch; a step is one complete
transient of the whole batch.  `value` is device-timed (inputs resident in
HBM, CUDA events around the launches, L2 flushed between steps); `e2e` is
the same metric through the public C ABI starting from host netlist text
(compile, upload, run, read back the accepted points).

Reference arm (--impl reference): the CPU oracle restatement of the
reference transient path (oracle/port), on all host cores, one process per
core, over a bounded sample of the same instances.

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
BYTES_MOS1 = 920
BYTES_RES = 72
BYTES_CAP = 136
BYTES_SRC = 120


def workload_text(name: str, tstop: str | None = None) -> tuple[str, dict]:
    from ngspice_gb300 import netlists
    if name == "c0":
        tstop = tstop or "20n"
        return netlists.inverter_chain(tstop=tstop), {
            "circuit": "32-stage MOS1 CMOS inverter chain (level 1, VTO +-0.7 V, KP 110/50 uA/V^2,"
                       " LAMBDA 0.04, W/L 2u/1u and 4u/1u, VDD 3.3 V, 20 fF loads,"
                       " PULSE(0 3.3 0 100p 100p 2n 4n))",
            "tran": f".tran 10p {tstop}"}
    raise SystemExit(f"unknown workload {name}")


def bytes_per_iteration(w: dict) -> int:
    n, nnz, nlu = w["n"], w["nnz"], w["nlu"]
    return (BYTES_MOS1 * w["mos1"] + BYTES_RES * w["res"] + BYTES_CAP * w["cap"]
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
def _cpu_one(text: str) -> int:
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import port
    r = port.simulate(text)
    return int(r["stats"]["accepted"])


def cpu_sample(text: str, instances: int, procs: int) -> tuple[float, int]:
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        acc = sum(pool.map(_cpu_one, [text] * instances, chunksize=1))
    return acc, time.perf_counter() - t0


def cpu_arm(args, text, wdesc) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import port
    port.build()
    procs = os.cpu_count() or 1
    sample = args.cpu_sample or 8 * procs
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_sample(text, procs, procs)
    times, accs = [], []
    for _ in range(args.steps):
        a, dt = cpu_sample(text, sample, procs)
        times.append(dt)
        accs.append(a)
    value = sum(accs) / sum(times)
    desc = f"{sample} instances per step across {procs} processes (oracle restatement, oracle/port)"
    return {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": wdesc,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# engine arm
# ---------------------------------------------------------------------------
def engine_arm(args, text, wdesc, rank, world) -> dict | None:
    from ngspice_gb300 import engine as E
    B = args.instances
    probes = ["n32"] if args.workload == "c0" else None
    circuits = [E.Circuit(text, probes=probes, outcap=8192) for _ in range(B)]
    w = circuits[0].workload()
    for _ in range(args.warmup):
        E.run(circuits)
    clocks = Clocks()
    dev_times, accepted, iters, launches = [], 0, 0, 0
    for _ in range(args.steps):
        flush_l2()
        sec = E.run(circuits)
        dev_times.append(sec)
        launches += E.last_launches()
        for c in circuits:
            r = c.results()
            if r[E.R_STATUS] != 0:
                raise SystemExit(f"engine status {r[E.R_STATUS]}")
            accepted += int(r[E.R_ACCEPTED])
            iters += int(r[E.R_NUMITER])
    clk = clocks.stop()
    total = sum(dev_times)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        a = torch.tensor([accepted], dtype=torch.float64, device="cuda")
        dist.all_reduce(a, op=dist.ReduceOp.SUM)
        total, accepted_all = float(t.item()), float(a.item())
    else:
        accepted_all = accepted
    value = accepted_all / total

    # e2e: host netlist text -> compile/upload -> run -> accepted points on host
    e2e_steps = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    h2d = d2h = 0
    e2e_acc = 0
    for _ in range(e2e_steps):
        cs = [E.Circuit(text, probes=probes, outcap=8192) for _ in range(B)]
        E.run(cs)
        for c in cs:
            tt, vv = c.points()
            d2h += tt.nbytes + vv.nbytes
            e2e_acc += int(c.results()[E.R_ACCEPTED])
            h2d += c.device_bytes()
        del cs
    e2e_time = time.perf_counter() - t0
    e2e = {"value": world * e2e_acc / e2e_time, "unit": UNIT,
           "h2d_bytes_per_step": h2d // e2e_steps, "d2h_bytes_per_step": d2h // e2e_steps}

    pk = peaks()
    bpi = bytes_per_iteration(w)
    achieved = bpi * iters / total / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": None,
            "peak_source": pk["src"], "kernel": "tran_kernel",
            "algorithmic_bytes_per_newton_iteration": bpi}
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * max(dev_times) if args.steps == 1 else 1e3 * total / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": wdesc, "clocks": clk, "e2e": e2e,
           "gpu_launches": launches, "roofline": roof,
           "newton_iterations_per_s": iters * world / total,
           "newton_iterations_per_accepted_step": iters / max(accepted, 1)}
    if rank == 0 and not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        sample = args.cpu_sample or 4 * procs
        a, dt = cpu_sample(text, sample, procs)
        out["cpu_baseline"] = {"value": a / dt, "unit": UNIT, "cores": procs, "kind": "port",
                               "sample": f"{sample} instances of the same circuit across {procs}"
                                         f" processes ({dt:.1f} s of CPU work)"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="c0")
    ap.add_argument("--instances", type=int, default=1216)
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tstop", default=None,
                    help="shorter .tran stop time (small cases for profiling)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    text, tdesc = workload_text(args.workload, args.tstop)
    wdesc = {"workload": f"{args.workload.upper()}: {tdesc['circuit']}, {tdesc['tran']},"
                         f" {args.instances} independent instances per launch",
             "instances_per_gpu": args.instances, "l2": "flushed between timed steps",
             "parallelism": f"replicas x{world}"}
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(cpu_arm(args, text, wdesc)))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        dist.barrier()
    out = engine_arm(args, text, wdesc, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
