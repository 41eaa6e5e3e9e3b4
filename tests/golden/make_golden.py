"""Generate the golden fixtures under tests/golden/ from the reference ngspice.

Test infrastructure.  Runs the reference ngspice transient path, compiled
from the reference sources by ``oracle/ref/Makefile`` into
``oracle/_ref/ngspice_ref``, on the seeded netlists of
``ngspice_gb300.netlists`` and stores, per netlist:

* ``names``            unknown names in equation order (CKTnames order)
* ``times``/``values`` every accepted time point CKTdump emitted
* ``stats``            numIter, tranIter, timePts, accepted, rejected, status
* ``it_*``             the first Newton iterations' stamped matrix (COO in
                       external equation numbers) and right-hand side, taken
                       just before the reference factors them
* ``netlist``          the netlist text itself

Usage (in the container that holds the reference sources)::

    make -C oracle/ref
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ngspice-sf-mirror_gb300"))

from ngspice_gb300 import netlists  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ngspice_ref")

# name -> (netlist text, number of Newton iterations to capture)
CASES = {
    "inverter_chain32": (netlists.inverter_chain(), 400),
    "mos1_mix": (netlists.mos1_mix(), 300),
    "rc_ladder": (netlists.rc_ladder(), 200),
    "diode_rectifier": (netlists.diode_rectifier(), 300),
    "bsim4_logic_s3": (netlists.random_logic(n_transistors=120, seed=3, n_inputs=6,
                                             tstop="1n"), 200),
    "bsim4_chain8": (None, 200),
    # one Monte Carlo instance: per-device mismatch model cards
    "bsim4_mc_s5": (netlists.random_logic(n_transistors=120, seed=5, n_inputs=6,
                                          tstop="600p", mismatch=True), 150),
}


def bsim4_chain(stages: int = 8) -> str:
    lines = ["* bsim4 inverter chain",
             ".model nch nmos level=54 vth0=0.42 toxe=1.75e-9",
             ".model pch pmos level=54 vth0=-0.41 toxe=1.75e-9",
             "vdd vdd 0 1.0",
             "vin n0 0 pulse(0 1 20p 10p 10p 200p 500p)"]
    for k in range(1, stages + 1):
        lines.append(f"mn{k} n{k} n{k-1} 0 0 nch w=200n l=45n")
        lines.append(f"mp{k} n{k} n{k-1} vdd vdd pch w=400n l=45n")
        lines.append(f"c{k} n{k} 0 1f")
    lines += [".tran 1p 1n", ".options klu", ".end", ""]
    return "\n".join(lines)


def read_trace(path: str) -> dict:
    b = open(path, "rb").read()
    assert b[:4] == b"NGOR", path
    o = 4
    _ver, nv, npt = struct.unpack_from("<3i", b, o)
    o += 12
    names = []
    for _ in range(nv):
        (ln,) = struct.unpack_from("<i", b, o)
        o += 4
        names.append(b[o:o + ln].decode())
        o += ln
    t = np.frombuffer(b, "<f8", npt, o).copy()
    o += 8 * npt
    v = np.frombuffer(b, "<f8", npt * nv, o).reshape(npt, nv).copy()
    o += 8 * npt * nv
    st = np.array(struct.unpack_from("<8i", b, o), dtype=np.int32)
    o += 32
    tm = np.array(struct.unpack_from("<6d", b, o))
    return {"names": np.array(names), "times": t, "values": v, "stats": st,
            "cpu_seconds": tm}


def read_iters(path: str) -> dict:
    b = open(path, "rb").read()
    o = 0
    kinds, meta, ptr, rows, cols, vals, rhs, rhsold = [], [], [0], [], [], [], [], []
    while o < len(b):
        kinds.append(b[o:o + 4].decode())
        o += 4
        t, d = struct.unpack_from("<2d", b, o)
        o += 16
        mode, order, n, nnz = struct.unpack_from("<4i", b, o)
        o += 16
        rec = np.frombuffer(b, dtype=np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8")]),
                            count=nnz, offset=o)
        o += 16 * nnz
        rows.append(rec["r"].copy())
        cols.append(rec["c"].copy())
        vals.append(rec["v"].copy())
        ptr.append(ptr[-1] + nnz)
        rhs.append(np.frombuffer(b, "<f8", n + 1, o).copy())
        o += 8 * (n + 1)
        rhsold.append(np.frombuffer(b, "<f8", n + 1, o).copy())
        o += 8 * (n + 1)
        meta.append((t, d, mode, order, n))
    meta = np.array(meta, dtype=np.float64).reshape(-1, 5)
    return {"it_kind": np.array(kinds), "it_meta": meta,
            "it_ptr": np.array(ptr, dtype=np.int64),
            "it_rows": np.concatenate(rows) if rows else np.zeros(0, np.int32),
            "it_cols": np.concatenate(cols) if cols else np.zeros(0, np.int32),
            "it_vals": np.concatenate(vals) if vals else np.zeros(0),
            "it_rhs": np.stack(rhs) if rhs else np.zeros((0, 1)),
            "it_rhsold": np.stack(rhsold) if rhsold else np.zeros((0, 1))}


def run_reference(text: str, iters: int, workdir: str) -> dict:
    cir = os.path.join(workdir, "case.cir")
    out = os.path.join(workdir, "case.bin")
    itf = os.path.join(workdir, "case.iters")
    with open(cir, "w") as f:
        f.write(text)
    cmd = [REF_BIN, cir, out, "--iters", itf, "--max-iters", str(iters)]
    p = subprocess.run(cmd, capture_output=True, text=True,
                       env=dict(os.environ, ORACLE_NUM_THREADS="1"))
    if p.returncode != 0:
        raise RuntimeError(f"reference failed ({p.returncode}): {p.stderr[-2000:]}")
    res = read_trace(out)
    res.update(read_iters(itf))
    return res


def main(argv: list[str]) -> int:
    if not os.path.exists(REF_BIN):
        print(f"missing {REF_BIN}: run `make -C oracle/ref` first", file=sys.stderr)
        return 2
    only = set(argv[1:])
    with tempfile.TemporaryDirectory() as wd:
        for name, (text, iters) in CASES.items():
            if only and name not in only:
                continue
            if text is None:
                text = bsim4_chain()
            res = run_reference(text, iters, wd)
            res["netlist"] = np.array(text)
            path = os.path.join(HERE, f"{name}.npz")
            np.savez_compressed(path, **res)
            print(f"{name}: {len(res['times'])} points, stats={res['stats'].tolist()},"
                  f" {len(res['it_kind'])} iterations -> {os.path.getsize(path)} bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
