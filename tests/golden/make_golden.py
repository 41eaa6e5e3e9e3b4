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

def bsim4_chain_v47_mixed(stages: int = 8) -> str:
    """An inverter chain whose odd stages use version 4.7 model cards (the
    reference's separate BSIM4v7 device) and whose even stages use 4.8
    cards.  The 4.7 nmos card gives toxp and dtox without toxe (BSIM4v7
    defaults cf from the set-up toxe) and a ketac that the BSIM4v7 parser
    ignores; its instances carry m=2 (BSIM4v7 scales each stamp's whole
    sum).  The 4.7 models are referenced first, yet load after the 4.8
    ones."""
    lines = ["* bsim4 inverter chain, version 4.7 and 4.8 cards",
             ".model n47 nmos level=54 version=4.7.0 vth0=0.42 toxp=1.45e-9 dtox=0.3e-9"
             " ketac=-0.04",
             ".model p47 pmos level=54 version=4.7.0 vth0=-0.41 toxe=1.75e-9",
             ".model n48 nmos level=54 version=4.8.3 vth0=0.42 toxe=1.75e-9 ketac=-0.04",
             ".model p48 pmos level=54 vth0=-0.41 toxe=1.75e-9",
             "vdd vdd 0 1.0",
             "vin n0 0 pulse(0 1 20p 10p 10p 200p 500p)"]
    for k in range(1, stages + 1):
        if k % 2:
            lines.append(f"mn{k} n{k} n{k-1} 0 0 n47 w=100n l=45n m=2")
            lines.append(f"mp{k} n{k} n{k-1} vdd vdd p47 w=400n l=45n")
        else:
            lines.append(f"mn{k} n{k} n{k-1} 0 0 n48 w=200n l=45n")
            lines.append(f"mp{k} n{k} n{k-1} vdd vdd p48 w=400n l=45n")
        lines.append(f"c{k} n{k} 0 1f")
    lines += [".tran 1p 1n", ".options klu", ".end", ""]
    return "\n".join(lines)


# name -> (netlist text, number of Newton iterations to capture, record the
# linearisation point of every k-th captured iteration (0: none))
CASES = {
    "inverter_chain32": (netlists.inverter_chain(), 400, 0),
    "mos1_mix": (netlists.mos1_mix(), 300, 0),
    "rc_ladder": (netlists.rc_ladder(), 200, 0),
    "diode_rectifier": (netlists.diode_rectifier(), 300, 0),
    "bsim4_logic_s3": (netlists.random_logic(n_transistors=120, seed=3, n_inputs=6,
                                             tstop="1n"), 200, 4),
    "bsim4_chain8": (None, 200, 1),
    # one Monte Carlo instance: per-device mismatch model cards
    "bsim4_mc_s5": (netlists.random_logic(n_transistors=120, seed=5, n_inputs=6,
                                          tstop="600p", mismatch=True), 150, 5),
    # version 4.7 model cards: the reference's BSIM4v7 device
    "v47_logic_s3": (netlists.random_logic(n_transistors=120, seed=3, n_inputs=6,
                                           tstop="1n").replace("level=54",
                                                               "level=54 version=4.7.0"),
                     200, 4),
    "v47_chain_mixed": (bsim4_chain_v47_mixed(), 200, 1),
}

# Circuits at the sizes the benchmarks run, with no iteration capture:
# accepted points, statistics, and the waveforms of NPROBE unknowns spread
# evenly over the equation numbering.
#   c1_10k_30p   the 10,000-transistor random-logic netlist of the plain
#                drop-in benchmark, first 30 ps of its transient
#   mc_1k/2k/3k  Monte Carlo instances (device mismatch) of about 1,000,
#                2,000 and 3,000 transistors, first 50 ps
#   mc_c4_1314   instance 1314 of the 4096-instance Monte Carlo workload
#                (4,714 transistors, seed 101314), first 150 ps: its L
#                entries grow past 1e6 in the transient, so it is the
#                batch's most rounding-sensitive refactorization
#   mc_c4_3893   instance 3893 (3,547 transistors, seed 103893), first
#                200 ps: on the engine's pivots its second transient step's
#                Newton iterations fail until the retry takes new pivots
NPROBE = 256

# A tight-tolerance reference (reltol 1e-5, vntol 1e-8 V, abstol 1e-14 A)
# of the 120-transistor deck over 400 ps, every unknown: the "true"
# waveform against which runs at the default tolerances are checked at
# their own time points (runs whose accepted steps differ from the
# reference's, e.g. with a Newton predictor).
TIGHT_OPTIONS = ".options klu reltol=1e-5 vntol=1e-8 abstol=1e-14"


# Gear integration (.options method=gear, maxord 2): the 120-transistor
# BSIM4 deck over 400 ps and the diode/MOS1/RC decks, every unknown.
# Ring oscillators embedded in random logic (the C3 generator at a small
# size): 300 logic transistors and two 7-stage rings over 300 ps, every
# unknown, started off their metastable point by current kicks.
RING_CASES = {
    "rings_300": lambda: netlists.logic_with_rings(n_transistors=300, seed=3, rings=2, stages=7,
                                                    tstop="300p"),
}

GEAR_CASES = {
    "gear_bsim4_logic_s3": lambda: netlists.random_logic(
        n_transistors=120, seed=3, n_inputs=6, tstop="400p").replace(
            ".options klu", ".options klu method=gear"),
    "gear_mos1_mix": lambda: netlists.mos1_mix().replace(".options klu",
                                                         ".options klu method=gear"),
    "gear_diode_rectifier": lambda: netlists.diode_rectifier().replace(
        ".options klu", ".options klu method=gear"),
    # maxord 6 (the largest the reference accepts): DCtran still never
    # raises the order past 2
    "gear6_bsim4_logic_s3": lambda: netlists.random_logic(
        n_transistors=120, seed=3, n_inputs=6, tstop="400p").replace(
            ".options klu", ".options klu method=gear maxord=6"),
}


# Diode temperature equations away from the nominal temperature: tlev 1
# (scaled breakdown voltage) with tlevc 1 (linear junction potential and
# capacitance) at 75 C; sidewall junctions with tlevc 0 at 75 C (the
# reference stops with "timestep too small" on this deck's sidewall junction
# under tlevc 1); tlev 2 (band-gap saturation current) at -20 C, tnom 30 C.
_DR = ".model dr d is=2e-14 n=1.1 rs=2 cjo=2p vj=0.8 m=0.4 tt=5p"
DIODE_TEMP_CASES = {
    "dio_tlev1_75c": lambda: netlists.diode_rectifier().replace(
        _DR, _DR + " bv=1.8 tcv=1e-3 tlev=1 tlevc=1 cta=1e-3 tpb=1.5e-3 ttt1=1e-3"
        " trs1=2e-3").replace(".options klu", ".options klu temp=75"),
    "dio_sw_75c": lambda: netlists.diode_rectifier().replace(
        _DR, _DR + " cjsw=0.3p pj=2 vjsw=0.7 mjsw=0.3").replace(
        ".options klu", ".options klu temp=75"),
    "dio_tlev2_m20c": lambda: netlists.diode_rectifier().replace(
        _DR, _DR + " tlev=2 eg=1.12 gap1=7.5e-4 gap2=1200 xti=3.2 bv=3 tcv=2e-3").replace(
        ".options klu", ".options klu temp=-20 tnom=30"),
}


def bsim4_logic_s3_tight() -> str:
    text = netlists.random_logic(n_transistors=120, seed=3, n_inputs=6, tstop="400p")
    return text.replace(".options klu", TIGHT_OPTIONS)


LARGE_CASES = {
    "c1_10k_30p": lambda: netlists.random_logic(n_transistors=10000, seed=1, tstop="30p"),
    "mc_1k_50p": lambda: netlists.random_logic(n_transistors=1000, seed=101, tstop="50p",
                                               mismatch=True),
    "mc_2k_50p": lambda: netlists.random_logic(n_transistors=2000, seed=102, tstop="50p",
                                               mismatch=True),
    "mc_3k_50p": lambda: netlists.random_logic(n_transistors=3000, seed=103, tstop="50p",
                                               mismatch=True),
    "mc_c4_1314": lambda: netlists.random_logic(n_transistors=4714, seed=101314, tstop="150p",
                                                mismatch=True),
    "mc_c4_3893": lambda: netlists.random_logic(n_transistors=3547, seed=103893, tstop="200p",
                                                mismatch=True),
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


def read_states(path: str) -> dict:
    """Linearisation points of the selected iterations (driver --states)."""
    b = open(path, "rb").read()
    o = 0
    idx, scal, st, von = [], [], [], []
    while o < len(b):
        i, nst, nvon, _ = struct.unpack_from("<4i", b, o)
        o += 16
        scal.append(struct.unpack_from("<6d", b, o))
        o += 48
        st.append(np.frombuffer(b, "<f8", 3 * nst, o).reshape(3, nst).copy())
        o += 24 * nst
        von.append(np.frombuffer(b, "<f8", nvon, o).copy())
        o += 8 * nvon
        idx.append(i)
    if not idx:
        return {}
    return {"st_iter": np.array(idx, np.int32),
            "st_scal": np.array(scal),          # ag0, ag1, deltaOld0, deltaOld1, gmin, srcFact
            "st_states": np.stack(st),          # [k][3][nstates] before the load
            "st_von": np.stack(von)}            # [k][BSIM4 instances]


def run_reference(text: str, iters: int, workdir: str, states_every: int = 0,
                  keep_iters: bool = True) -> dict:
    cir = os.path.join(workdir, "case.cir")
    out = os.path.join(workdir, "case.bin")
    itf = os.path.join(workdir, "case.iters")
    stf = os.path.join(workdir, "case.states")
    with open(cir, "w") as f:
        f.write(text)
    cmd = [REF_BIN, cir, out, "--iters", itf, "--max-iters", str(iters)]
    if states_every > 0:
        cmd += ["--states", stf, "--states-every", str(states_every)]
    p = subprocess.run(cmd, capture_output=True, text=True,
                       env=dict(os.environ, ORACLE_NUM_THREADS="1"))
    if p.returncode != 0:
        raise RuntimeError(f"reference failed ({p.returncode}): {p.stderr[-2000:]}")
    res = read_trace(out)
    if keep_iters:
        res.update(read_iters(itf))
    if states_every > 0:
        res.update(read_states(stf))
    return res


def main(argv: list[str]) -> int:
    if not os.path.exists(REF_BIN):
        print(f"missing {REF_BIN}: run `make -C oracle/ref` first", file=sys.stderr)
        return 2
    only = set(argv[1:])
    with tempfile.TemporaryDirectory() as wd:
        for name, (text, iters, every) in CASES.items():
            if only and name not in only:
                continue
            if text is None:
                text = bsim4_chain()
            res = run_reference(text, iters, wd, states_every=every)
            res["netlist"] = np.array(text)
            path = os.path.join(HERE, f"{name}.npz")
            np.savez_compressed(path, **res)
            print(f"{name}: {len(res['times'])} points, stats={res['stats'].tolist()},"
                  f" {len(res['it_kind'])} iterations -> {os.path.getsize(path)} bytes")
        if not only or "bsim4_logic_s3_tight" in only:
            text = bsim4_logic_s3_tight()
            res = run_reference(text, 0, wd, keep_iters=False)
            out = {k: res[k] for k in ("names", "times", "values", "stats", "cpu_seconds")}
            out["netlist"] = np.array(text)
            path = os.path.join(HERE, "bsim4_logic_s3_tight.npz")
            np.savez_compressed(path, **out)
            print(f"bsim4_logic_s3_tight: {len(res['times'])} points, stats={res['stats'].tolist()}"
                  f" -> {os.path.getsize(path)} bytes")
        for name, make in (list(GEAR_CASES.items()) + list(RING_CASES.items()) +
                           list(DIODE_TEMP_CASES.items())):
            if only and name not in only:
                continue
            text = make()
            res = run_reference(text, 0, wd, keep_iters=False)
            out = {k: res[k] for k in ("names", "times", "values", "stats", "cpu_seconds")}
            out["netlist"] = np.array(text)
            path = os.path.join(HERE, f"{name}.npz")
            np.savez_compressed(path, **out)
            print(f"{name}: {len(res['times'])} points, stats={res['stats'].tolist()}"
                  f" -> {os.path.getsize(path)} bytes")
        for name, make in LARGE_CASES.items():
            if only and name not in only:
                continue
            text = make()
            res = run_reference(text, 0, wd, keep_iters=False)
            nv = len(res["names"])
            cols = np.unique(np.linspace(0, nv - 1, min(NPROBE, nv)).round().astype(int))
            out = {"names": res["names"][cols], "cols": cols.astype(np.int32),
                   "nvars": np.int32(nv), "times": res["times"],
                   "values": res["values"][:, cols], "stats": res["stats"],
                   "cpu_seconds": res["cpu_seconds"], "netlist": np.array(text)}
            path = os.path.join(HERE, f"{name}.npz")
            np.savez_compressed(path, **out)
            print(f"{name}: {nv} unknowns, {len(res['times'])} points,"
                  f" stats={res['stats'].tolist()} -> {os.path.getsize(path)} bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
