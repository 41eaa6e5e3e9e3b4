"""Test infrastructure: times the CPU oracle port against the reference
ngspice (KLU, compiled from the reference sources into oracle/_ref) on the
same netlists, in the container that holds the reference sources.

The benchmark's CPU baseline runs the port on the GPU machine's host cores (the
reference sources, and so the reference binary, are not there); this
calibration gives the factor between the port and reference ngspice-KLU on
one machine, with the reference run single-threaded and with its OpenMP
BSIM4 load on every core (`set num_threads`, read by CKTsetup under USE_OMP,
src/spicelib/analysis/cktsetup.c:89-93; the parallel load is
src/spicelib/devices/bsim4/b4ld.c:74-90).

    python oracle/ref/calibrate.py            # prints one JSON line
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ngspice-sf-mirror_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ngspice_ref")


def time_reference(text: str, threads: int, wd: str) -> dict:
    import make_golden
    cir, out = os.path.join(wd, "cal.cir"), os.path.join(wd, "cal.bin")
    with open(cir, "w") as f:
        f.write(text)
    t0 = time.perf_counter()
    subprocess.run([REF_BIN, cir, out], check=True, capture_output=True,
                   env=dict(os.environ, ORACLE_NUM_THREADS=str(threads)))
    wall = time.perf_counter() - t0
    r = make_golden.read_trace(out)
    return {"wall_s": wall, "tran_s": float(r["cpu_seconds"][0]),
            "accepted": int(r["stats"][3]), "newton": int(r["stats"][0])}


def time_port(text: str) -> dict:
    import port
    t0 = time.perf_counter()
    r = port.simulate(text)
    return {"wall_s": time.perf_counter() - t0, "accepted": int(r["stats"]["accepted"]),
            "newton": int(r["stats"]["numIter"])}


def main() -> int:
    from ngspice_gb300 import netlists
    import port
    port.build()
    cores = os.cpu_count() or 1
    cases = {
        "c1_10k_50p": netlists.random_logic(n_transistors=10000, seed=1, tstop="50p"),
        "mc_3k_100p": netlists.random_logic(n_transistors=3000, seed=103, tstop="100p",
                                            mismatch=True),
    }
    out = {"host_cores": cores, "cases": {}}
    with tempfile.TemporaryDirectory() as wd:
        for name, text in cases.items():
            p = time_port(text)
            r1 = time_reference(text, 1, wd)
            rn = time_reference(text, cores, wd)
            assert p["accepted"] == r1["accepted"] == rn["accepted"]
            out["cases"][name] = {
                "port_1core": p, "reference_klu_1thread": r1,
                f"reference_klu_{cores}threads": rn,
                "reference_1thread_over_port": r1["wall_s"] / p["wall_s"],
                f"reference_{cores}threads_over_port": rn["wall_s"] / p["wall_s"]}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
