"""Seeded netlist generators for the transient workloads.

Every generator returns plain SPICE text in the flat subset both the GPU
engine and the reference ngspice parse identically: no ``.subckt``, no
``.param``, no braces, lower-case cards, ``.options klu`` so the reference
runs its KLU path.

Workloads (sizes as named in the project configuration):

* ``inverter_chain``  32-stage MOS1 CMOS inverter chain, ``.tran 10p 20n``
  (about 34 unknowns).
* ``mos1_mix``        small MOS1 circuit that exercises drain/source
  resistances, junction and Meyer capacitances, PWL sources, a current
  source and a diode.
* ``rc_ladder``       RC ladder driven by a PULSE source (breakpoints).
* ``random_logic``    seeded random CMOS logic (INV/NAND2/NOR2), each net an
  RC pi segment, BSIM4 (level 54) or MOS1 devices.
"""
from __future__ import annotations

import math
import random

__all__ = ["inverter_chain", "mos1_mix", "rc_ladder", "diode_rectifier",
           "random_logic", "RandomLogicSpec"]


def _fmt(x: float) -> str:
    """Format a float the way the generators write every number: repr-exact
    scientific notation, which both parsers read to the same double."""
    return f"{x:.17g}"


def inverter_chain(stages: int = 32, tstep: str = "10p", tstop: str = "20n",
                   load: str = "20f", vdd: float = 3.3) -> str:
    """32-stage MOS1 CMOS inverter chain (level 1, VTO=+-0.7 V,
    KP=110/50 uA/V^2, LAMBDA=0.04, W/L=2u/1u N and 4u/1u P, VDD=3.3 V,
    20 fF load per stage, input PULSE(0 3.3 0 100p 100p 2n 4n))."""
    lines = [f"* {stages}-stage mos1 cmos inverter chain",
             ".model nch nmos level=1 vto=0.7 kp=110u lambda=0.04",
             ".model pch pmos level=1 vto=-0.7 kp=50u lambda=0.04",
             f"vdd vdd 0 {vdd}",
             f"vin n0 0 pulse(0 {vdd} 0 100p 100p 2n 4n)"]
    for k in range(1, stages + 1):
        a, y = f"n{k-1}", f"n{k}"
        lines.append(f"mn{k} {y} {a} 0 0 nch w=2u l=1u")
        lines.append(f"mp{k} {y} {a} vdd vdd pch w=4u l=1u")
        lines.append(f"cl{k} {y} 0 {load}")
    lines += [f".tran {tstep} {tstop}", ".options klu", ".end", ""]
    return "\n".join(lines)


def mos1_mix(tstop: str = "10n") -> str:
    """Small MOS1 circuit covering the load paths the inverter chain does
    not: RD/RS internal nodes, bulk junction capacitances (CJ, CJSW, MJ != .5),
    gate overlap and Meyer capacitances (TOX given), GAMMA/PHI body effect,
    a PWL source, a DC current source and a junction diode."""
    return "\n".join([
        "* mos1 mixed-feature circuit",
        ".model nm nmos level=1 vto=0.6 kp=80u gamma=0.5 phi=0.7 lambda=0.02"
        " rd=20 rs=15 cbd=2f cbs=2f cj=3e-4 mj=0.4 cjsw=2e-10 mjsw=0.3"
        " cgso=3e-10 cgdo=3e-10 cgbo=1e-10 tox=2e-8 is=1e-15 pb=0.75",
        ".model pm pmos level=1 vto=-0.65 kp=35u gamma=0.45 phi=0.65 lambda=0.03"
        " cj=4e-4 mj=0.5 cjsw=2.5e-10 mjsw=0.5 cgso=2.5e-10 cgdo=2.5e-10"
        " tox=2e-8",
        ".model dd d is=1e-14 n=1.05 rs=5 cjo=1p vj=0.7 m=0.45 tt=10p",
        "vdd vdd 0 2.5",
        "vin in 0 pwl(0 0 1n 2.5 3n 2.5 3.5n 0 6n 0 6.2n 1.2)",
        "mp1 o1 in vdd vdd pm w=6u l=1u ad=6p as=6p pd=14u ps=14u",
        "mn1 o1 in 0 0 nm w=3u l=1u ad=3p as=3p pd=8u ps=8u",
        "mp2 o2 o1 vdd vdd pm w=6u l=1u",
        "mn2 o2 o1 x 0 nm w=3u l=1u",
        "mn3 x in 0 0 nm w=3u l=1u",
        "r1 o2 o3 2k",
        "c1 o3 0 50f",
        "d1 o3 dn dd",
        "rd dn 0 10k",
        "i1 vdd o1 5u",
        "cl1 o1 0 10f",
        f".tran 5p {tstop}",
        ".options klu",
        ".end", ""])


def rc_ladder(sections: int = 8, tstop: str = "8n") -> str:
    """RC ladder driven by a trapezoidal PULSE source: exercises the
    breakpoint table, order switching and the LTE control on linear
    devices only."""
    lines = ["* rc ladder",
             "vin n0 0 pulse(0 1 0.2n 50p 80p 1n 2.5n)"]
    for k in range(1, sections + 1):
        lines.append(f"r{k} n{k-1} n{k} {100 * k}")
        lines.append(f"c{k} n{k} 0 {10 + 3 * k}f")
    lines += [f".tran 10p {tstop}", ".options klu", ".end", ""]
    return "\n".join(lines)


def diode_rectifier(tstop: str = "20n") -> str:
    """Half-wave rectifier with a smoothing capacitor: diode load, limiting
    and junction-capacitance integration."""
    return "\n".join([
        "* diode rectifier",
        ".model dr d is=2e-14 n=1.1 rs=2 cjo=2p vj=0.8 m=0.4 tt=5p",
        "vin a 0 sin(0 2 200meg)",
        "d1 a b dr",
        "c1 b 0 2p",
        "r1 b 0 5k",
        f".tran 20p {tstop}",
        ".options klu",
        ".end", ""])


# ---------------------------------------------------------------------------
# seeded random CMOS logic
# ---------------------------------------------------------------------------
class RandomLogicSpec:
    """Parameters of the random-logic generator.

    Gate mix INV/NAND2/NOR2 = 40/35/25 %, logic depth <= ``depth``, fanout
    1-4, every net an RC pi segment (R log-uniform 10-500 ohm, C log-uniform
    0.2-10 fF split half/half), ``n_inputs`` PULSE inputs with seeded periods
    log-uniform 200 ps-2 ns.  Fanin is drawn from a sliding window of recently
    created nets, which keeps the circuit graph local (as placed logic is) and
    the LU fill bounded.
    """

    def __init__(self, n_transistors: int = 10000, seed: int = 1,
                 n_inputs: int = 64, depth: int = 30, model: str = "bsim4",
                 vdd: float = 1.0, tstep: str = "1p", tstop: str = "5n",
                 mismatch: bool = False, window: int = 96):
        self.n_transistors = n_transistors
        self.seed = seed
        self.n_inputs = n_inputs
        self.depth = depth
        self.model = model
        self.vdd = vdd
        self.tstep = tstep
        self.tstop = tstop
        self.mismatch = mismatch
        self.window = window


_GATES = (("inv", 0.40, 2), ("nand2", 0.35, 4), ("nor2", 0.25, 4))


def _model_cards(model: str, vdd: float) -> list[str]:
    if model == "bsim4":
        return [".model nch nmos level=54 vth0=0.42 toxe=1.75e-9",
                ".model pch pmos level=54 vth0=-0.41 toxe=1.75e-9"]
    if model == "mos1":
        return [".model nch nmos level=1 vto=0.42 kp=200u lambda=0.05 tox=2e-9",
                ".model pch pmos level=1 vto=-0.41 kp=90u lambda=0.05 tox=2e-9"]
    raise ValueError(f"unknown device model {model!r}")


def random_logic(spec: RandomLogicSpec | None = None, **kw) -> str:
    """Seeded random combinational CMOS logic netlist (see RandomLogicSpec)."""
    s = spec or RandomLogicSpec(**kw)
    rng = random.Random(s.seed)
    lines = [f"* random logic seed={s.seed} transistors~{s.n_transistors} model={s.model}"]
    lines += _model_cards(s.model, s.vdd)
    lines.append(f"vdd vdd 0 {s.vdd}")
    # primary inputs
    nets: list[tuple[str, int]] = []       # (driven far-end net name, level)
    for i in range(s.n_inputs):
        per = math.exp(rng.uniform(math.log(200e-12), math.log(2e-9)))
        tr = 0.05 * per
        pw = 0.5 * per - tr
        td = rng.uniform(0.0, per)
        lines.append(f"vi{i} i{i} 0 pulse(0 {s.vdd} {_fmt(td)} {_fmt(tr)} {_fmt(tr)}"
                     f" {_fmt(pw)} {_fmt(per)})")
        nets.append((f"i{i}", 0))
    fanout_left: dict[str, int] = {n: rng.randint(1, 4) for n, _ in nets}
    ntr = 0
    gate_id = 0
    mm_id = 0
    w_lo, w_hi = 90e-9, 720e-9

    def pick_inputs(k: int) -> list[tuple[str, int]]:
        pool = [x for x in nets[-s.window:] if x[1] < s.depth and fanout_left[x[0]] > 0]
        if len(pool) < k:
            pool = [x for x in nets[-4 * s.window:] if x[1] < s.depth]
        if len(pool) < k:
            # every recent net is at the depth limit (circuits much larger
            # than depth x window): restart a cone from the primary inputs
            pool = nets[:s.n_inputs]
        chosen = []
        for _ in range(k):
            cand = rng.choice(pool)
            tries = 0
            while cand in chosen and tries < 8:
                cand = rng.choice(pool)
                tries += 1
            chosen.append(cand)
            fanout_left[cand[0]] = fanout_left.get(cand[0], 1) - 1
        return chosen

    def mos(name, d, g, src, b, mtype, w):
        nonlocal mm_id
        if s.mismatch:
            w = w * (1.0 + 0.03 * rng.gauss(0.0, 1.0))
            mm_id += 1
            mod = f"{mtype}{mm_id}"
            base = 0.42 if mtype == "nch" else -0.41
            vth = base + 0.015 * rng.gauss(0.0, 1.0)
            tox = 1.75e-9 * (1.0 + 0.02 * rng.gauss(0.0, 1.0))
            kind = "nmos" if mtype == "nch" else "pmos"
            if s.model == "bsim4":
                lines.append(f".model {mod} {kind} level=54 vth0={_fmt(vth)} toxe={_fmt(tox)}")
            else:
                kp = "200u" if mtype == "nch" else "90u"
                lines.append(f".model {mod} {kind} level=1 vto={_fmt(vth)} kp={kp}"
                             f" lambda=0.05 tox={_fmt(tox)}")
            mtype = mod
        lines.append(f"{name} {d} {g} {src} {b} {mtype} w={_fmt(w)} l=45n")

    while ntr < s.n_transistors:
        r = rng.random()
        acc = 0.0
        for gname, frac, ntrans in _GATES:
            acc += frac
            if r < acc:
                break
        k = 1 if gname == "inv" else 2
        ins = pick_inputs(k)
        level = 1 + max(l for _, l in ins)
        g = gate_id
        gate_id += 1
        y = f"y{g}"
        wn = rng.uniform(w_lo, w_hi)
        wp = rng.uniform(w_lo, w_hi)
        if gname == "inv":
            a = ins[0][0]
            mos(f"mn{g}", y, a, "0", "0", "nch", wn)
            mos(f"mp{g}", y, a, "vdd", "vdd", "pch", wp)
        elif gname == "nand2":
            a, b = ins[0][0], ins[1][0]
            mos(f"mna{g}", y, a, f"x{g}", "0", "nch", wn)
            mos(f"mnb{g}", f"x{g}", b, "0", "0", "nch", wn)
            mos(f"mpa{g}", y, a, "vdd", "vdd", "pch", wp)
            mos(f"mpb{g}", y, b, "vdd", "vdd", "pch", wp)
        else:
            a, b = ins[0][0], ins[1][0]
            mos(f"mna{g}", y, a, "0", "0", "nch", wn)
            mos(f"mnb{g}", y, b, "0", "0", "nch", wn)
            mos(f"mpa{g}", f"x{g}", a, "vdd", "vdd", "pch", wp)
            mos(f"mpb{g}", y, b, f"x{g}", "vdd", "pch", wp)
        ntr += ntrans
        # RC pi segment from the gate output y to the net's far end z
        rval = math.exp(rng.uniform(math.log(10.0), math.log(500.0)))
        cval = math.exp(rng.uniform(math.log(0.2e-15), math.log(10e-15)))
        z = f"z{g}"
        lines.append(f"rw{g} {y} {z} {_fmt(rval)}")
        lines.append(f"cwa{g} {y} 0 {_fmt(0.5 * cval)}")
        lines.append(f"cwb{g} {z} 0 {_fmt(0.5 * cval)}")
        nets.append((z, level))
        fanout_left[z] = rng.randint(1, 4)
    lines += [f".tran {s.tstep} {s.tstop}", ".options klu", ".end", ""]
    return "\n".join(lines)


def logic_with_rings(n_transistors: int = 50000, seed: int = 3, rings: int = 16,
                     stages: int = 31, tstep: str = "1p", tstop: str = "10n") -> str:
    """The random-logic netlist of `n_transistors` BSIM4 transistors with
    `rings` embedded ring oscillators of `stages` inverters each (odd), the
    single large circuit of the learned-predictor workload.  Every stage
    drives an RC pi segment like the logic's nets; each ring's first stage
    gets a 0.2 mA, 20 ps current kick (staggered per ring) that moves it off
    its metastable operating point, and each ring's first node also drives
    a loaded inverter, as a tap of the ring would."""
    base = random_logic(n_transistors=n_transistors, seed=seed, tstep=tstep, tstop=tstop)
    rng = random.Random(seed + 7919)
    body = base.split("\n")
    tail = [ln for ln in body if ln.startswith(".tran") or ln.startswith(".options")
            or ln == ".end" or ln == ""]
    head = [ln for ln in body if ln not in tail]
    lines = list(head)
    for r in range(rings):
        for k in range(stages):
            a = f"ro{r}_{k}"
            y = f"ro{r}_{(k + 1) % stages}"
            wn = rng.uniform(180e-9, 360e-9)
            wp = 2.0 * wn
            lines.append(f"mrn{r}_{k} {y}x {a} 0 0 nch w={_fmt(wn)} l=45n")
            lines.append(f"mrp{r}_{k} {y}x {a} vdd vdd pch w={_fmt(wp)} l=45n")
            rval = math.exp(rng.uniform(math.log(10.0), math.log(200.0)))
            cval = math.exp(rng.uniform(math.log(0.5e-15), math.log(4e-15)))
            lines.append(f"rro{r}_{k} {y}x {y} {_fmt(rval)}")
            lines.append(f"cra{r}_{k} {y}x 0 {_fmt(0.5 * cval)}")
            lines.append(f"crb{r}_{k} {y} 0 {_fmt(0.5 * cval)}")
        td = 5e-12 + 3e-12 * r
        lines.append(f"iro{r} 0 ro{r}_0 pulse(0 200u {_fmt(td)} 2p 2p 20p 1)")
        # the ring's output loads an inverter whose output joins the logic
        lines.append(f"mron{r} rq{r} ro{r}_0 0 0 nch w=180n l=45n")
        lines.append(f"mrop{r} rq{r} ro{r}_0 vdd vdd pch w=360n l=45n")
        lines.append(f"crq{r} rq{r} 0 2f")
    return "\n".join(lines + tail)
