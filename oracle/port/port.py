"""Test infrastructure: Python front end of the CPU oracle (port.c).

Reads a flat netlist the way the reference parser passes do (INPpas1 models,
INPpas2 instances, src/spicelib/parser/), numbers the equations in the
reference order (external nodes in order of first appearance, then the
internal nodes and branch equations CKTsetup creates device type by device
type, newest model and newest instance first: analysis/cktmcrt.c:38-39,
devices/cktcrte.c:62-64), computes the temperature-dependent MOS1
parameters as MOS1temp does (devices/mos1/mos1temp.c:36-332), and hands the
compiled circuit to the C restatement of the transient loop.

Only tests, smoke() and bench.py's CPU baseline use this module.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(os.path.dirname(HERE), "_port")
LIB = os.path.join(OUT, "libngport.so")

K_BSIM4, K_CAP, K_DIO, K_ISRC, K_MOS1, K_RES, K_VSRC = range(7)

BOLTZ = 1.38064852e-23
CHARGE = 1.6021766208e-19
KOVERQ = BOLTZ / CHARGE
REFTEMP = 27.0 + 273.15
ROOT2 = 1.4142135623730950488016887242097
CTOK = 273.15


CSRC = os.path.join(ROOT, "ngspice-sf-mirror_gb300", "csrc")


def build(force: bool = False) -> str:
    """Compile port.c (gcc) and the BSIM4 glue b4port.cpp with the shared
    model arithmetic (g++) into oracle/_port/libngport.so, without
    floating-point contraction."""
    src = os.path.join(HERE, "port.c")
    cxx = [os.path.join(HERE, "b4port.cpp"), os.path.join(HERE, "sparse_port.cpp"),
           os.path.join(CSRC, "bsim4_setup.cpp"), os.path.join(CSRC, "dio_setup.cpp"),
           os.path.join(CSRC, "sparse.cpp")]
    deps = [src] + cxx + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                          if f.endswith((".h", ".cuh", ".def"))]
    os.makedirs(OUT, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(map(os.path.getmtime, deps)):
        objs = []
        flags = ["-O2", "-ffp-contract=off", "-fPIC"]
        o = os.path.join(OUT, "port.o")
        subprocess.run(["gcc"] + flags + ["-c", src, "-o", o], check=True)
        objs.append(o)
        for f in cxx:
            o = os.path.join(OUT, os.path.basename(f) + ".o")
            subprocess.run(["g++", "-std=c++17"] + flags + [f"-I{CSRC}", "-c", f, "-o", o],
                           check=True)
            objs.append(o)
        tmp = LIB + ".tmp"
        subprocess.run(["g++", "-shared", "-o", tmp] + objs + ["-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        vp = C.c_void_p
        L.port_new.restype = vp
        L.port_new.argtypes = [C.c_int, C.c_int]
        L.port_free.argtypes = [vp]
        L.port_set_ntype.argtypes = [vp, C.POINTER(C.c_int)]
        L.port_set_options.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.port_add_res.argtypes = [vp, C.c_int, C.c_int, C.c_double]
        L.port_add_cap.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                   C.c_double]
        L.port_add_src.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.c_double), C.c_double, C.c_int, C.c_double]
        L.port_add_mos1.argtypes = [vp, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double)]
        L.port_add_b4.argtypes = [vp, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double)]
        L.port_add_dio.argtypes = [vp, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double)]
        L.port_dio_nparam.restype = C.c_int
        L.port_dio_nstate.restype = C.c_int
        L.port_dio_params.restype = C.c_int
        L.port_dio_params.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p),
                                      C.POINTER(C.c_double), C.c_char_p, C.c_int,
                                      C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.c_double,
                                      C.c_double, C.c_double, C.POINTER(C.c_double),
                                      C.POINTER(C.c_int), C.c_char_p, C.c_int]
        L.port_b4_nparam.restype = C.c_int
        L.port_b4_nstate.restype = C.c_int
        cp = C.POINTER(C.c_char_p)
        dp = C.POINTER(C.c_double)
        L.port_b4_params.restype = C.c_int
        L.port_b4_params.argtypes = [C.c_char_p, C.c_int, C.c_int, cp, dp, C.c_char_p, C.c_int,
                                     cp, dp, C.c_double, C.c_double, dp,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_char_p, C.c_int]
        L.port_set_output.argtypes = [vp, C.POINTER(C.c_double), C.c_int]
        L.port_set_dump.argtypes = [vp] + [C.POINTER(C.c_double)] * 4 + [C.c_int]
        L.port_run.restype = C.c_int
        L.port_run.argtypes = [vp, C.POINTER(C.c_long), C.c_long]
        _lib = L
    return _lib


# ---------------------------------------------------------------------------
# netlist reading
# ---------------------------------------------------------------------------
def evaluate(tok: str):
    """INPevaluate (src/spicelib/parser/inpeval.c:16-204): digits into one
    double mantissa, optional exponent, one scale letter."""
    i = 0
    sign = 1
    if tok[:1] == "+":
        i = 1
    elif tok[:1] == "-":
        i = 1
        sign = -1
    if i >= len(tok) or not (tok[i].isdigit() or tok[i] == "."):
        return None
    mantis = 0.0
    expo1 = expo2 = 0
    expsgn = 1
    while i < len(tok) and tok[i].isdigit():
        mantis = 10 * mantis + (ord(tok[i]) - 48)
        i += 1
    if i >= len(tok):
        return mantis * sign
    if tok[i] == ".":
        i += 1
        if i >= len(tok):
            return mantis * sign
        while i < len(tok) and tok[i].isdigit():
            mantis = 10 * mantis + (ord(tok[i]) - 48)
            expo1 -= 1
            i += 1
    if i < len(tok) and tok[i] in "ed":
        i += 1
        if i < len(tok) and tok[i] == "+":
            i += 1
        elif i < len(tok) and tok[i] == "-":
            i += 1
            expsgn = -1
        while i < len(tok) and tok[i].isdigit():
            expo2 = 10 * expo2 + (ord(tok[i]) - 48)
            i += 1
    ch = tok[i] if i < len(tok) else ""
    if ch == "t":
        expo1 += 12
    elif ch == "g":
        expo1 += 9
    elif ch == "k":
        expo1 += 3
    elif ch == "u":
        expo1 -= 6
    elif ch == "n":
        expo1 -= 9
    elif ch == "p":
        expo1 -= 12
    elif ch == "f":
        expo1 -= 15
    elif ch == "a":
        expo1 -= 18
    elif ch == "m":
        if tok[i:i + 3] == "meg":
            expo1 += 6
        elif tok[i:i + 3] == "mil":
            expo1 -= 6
            mantis *= 25.4
        else:
            expo1 -= 3
    return sign * mantis * math.pow(10.0, float(expo1 + expsgn * expo2))


def tokens(line: str) -> list[str]:
    out, cur = [], ""
    for ch in line:
        if ch.isspace() or ch in ",()":
            if cur:
                out.append(cur)
                cur = ""
        elif ch == "=":
            if cur:
                out.append(cur)
                cur = ""
            out.append("=")
        else:
            cur += ch
    if cur:
        out.append(cur)
    return out


def params(t: list[str], i: int) -> dict:
    p = {}
    while i < len(t):
        if i + 1 < len(t) and t[i + 1] == "=":
            v = evaluate(t[i + 2])
            p[t[i]] = v
            i += 3
            while i < len(t) and evaluate(t[i]) is not None:
                i += 1
        else:
            p[t[i]] = 1.0
            i += 1
    return p


class Circuit:
    """Compiled circuit for the oracle."""

    def __init__(self, text: str):
        lines = []
        first = True
        for raw in text.splitlines():
            s = raw.lower().strip()
            if first:
                first = False
                continue
            if not s or s.startswith("*"):
                continue
            if ";" in s:
                s = s[:s.index(";")]
            if s.startswith("+"):
                lines[-1] += " " + s[1:]
                continue
            if s.split()[0] == ".end":
                break
            lines.append(s)
        self.models = {}
        for s in lines:
            if s.startswith(".model"):
                t = tokens(s)
                self.models[t[1]] = (t[2], params(t, 3))
        self.names = ["0"]
        self.index = {"0": 0}
        self.ntype = [1]
        self.tran = None
        self.opts = {}
        model_order = {}
        inst = []
        for s in lines:
            t = tokens(s)
            if t[0].startswith("."):
                if t[0] == ".tran":
                    vals = [evaluate(x) for x in t[1:] if evaluate(x) is not None]
                    self.tran = vals
                elif t[0] in (".options", ".option", ".opt"):
                    i = 1
                    while i < len(t):
                        if i + 2 < len(t) and t[i + 1] == "=":
                            self.opts[t[i]] = t[i + 2]
                            i += 3
                        else:
                            self.opts[t[i]] = "1"
                            i += 1
                continue
            k = t[0][0]
            if k in "rc":
                nodes = [self.node(t[1]), self.node(t[2])]
                value = evaluate(t[3]) if len(t) > 3 else None
                kind = K_RES if k == "r" else K_CAP
                p = params(t, 4)
                inst.append((kind, t[0], nodes, value, p, None))
                key = ("default", kind)
            elif k in "vi":
                nodes = [self.node(t[1]), self.node(t[2])]
                kind = K_VSRC if k == "v" else K_ISRC
                wf = self.source(t)
                inst.append((kind, t[0], nodes, None, {}, wf))
                key = ("default", kind)
            elif k == "d":
                nodes = [self.node(t[1]), self.node(t[2])]
                mname = t[3]
                p = {}
                i = 4
                while i < len(t):           # optional area value, then key=value
                    if i + 1 < len(t) and t[i + 1] == "=":
                        p[t[i]] = evaluate(t[i + 2])
                        i += 3
                    elif evaluate(t[i]) is not None and "area" not in p:
                        p["area"] = evaluate(t[i])
                        i += 1
                    else:
                        p[t[i]] = 1.0
                        i += 1
                inst.append((K_DIO, t[0], nodes, mname, p, None))
                key = mname
            elif k == "m":
                nodes = [self.node(x) for x in t[1:5]]
                mname = t[5]
                mtype, mp = self.models[mname]
                level = int(mp.get("level", 1))
                if level == 1:
                    inst.append((K_MOS1, t[0], nodes, mname, params(t, 6), None))
                elif level in (14, 54):
                    inst.append((K_BSIM4, t[0], nodes, mname, params(t, 6), None))
                else:
                    raise ValueError("oracle port: MOS levels 1 and 54 only")
                key = mname
            else:
                raise ValueError(f"oracle port: unsupported element {t[0]}")
            if key not in model_order:
                model_order[key] = len(model_order)
        # per kind: newest model first, newest instance first
        self.order = {kk: [] for kk in range(7)}
        groups = {}
        for idx, e in enumerate(inst):
            key = ("default", e[0]) if e[0] not in (K_MOS1, K_BSIM4, K_DIO) else e[3]
            groups.setdefault(key, []).append(idx)
        def v47(key):
            # version 4.7 cards select the BSIM4v7 device, which follows
            # BSIM4 in the device table (devices/dev.c:154-157)
            if not isinstance(key, str) or key not in self.models:
                return False
            ver = self.models[key][1].get("version")
            return ver is not None and 4.7 - 1e-9 <= ver < 4.8 - 1e-9

        for kk in range(7):
            keys = [key for key in groups if (inst[groups[key][0]][0] == kk)]
            keys.sort(key=lambda q: (v47(q), -model_order[q]))
            for key in keys:
                self.order[kk] += list(reversed(groups[key]))
        self.inst = inst
        self.setup()

    def node(self, nm: str) -> int:
        if nm == "gnd":
            nm = "0"
        if nm not in self.index:
            self.index[nm] = len(self.names)
            self.names.append(nm)
            self.ntype.append(1)
        return self.index[nm]

    def source(self, t):
        wf = {"kind": 0, "coef": [], "dc": 0.0, "dcgiven": 0}
        i = 3
        while i < len(t):
            v = evaluate(t[i])
            if v is not None:
                wf["dc"], wf["dcgiven"] = v, 1
                i += 1
            elif t[i] == "dc":
                wf["dc"], wf["dcgiven"] = evaluate(t[i + 1]), 1
                i += 2
            elif t[i] in ("pulse", "sin", "pwl"):
                wf["kind"] = {"pulse": 1, "sin": 2, "pwl": 4}[t[i]]
                i += 1
                while i < len(t) and evaluate(t[i]) is not None:
                    wf["coef"].append(evaluate(t[i]))
                    i += 1
            else:
                raise ValueError(f"oracle port: unsupported source token {t[i]}")
        return wf

    def mk(self, name: str, voltage: bool) -> int:
        self.names.append(name)
        self.ntype.append(1 if voltage else 0)
        return len(self.names) - 1

    # CKTsetup order: bsim4, cap, dio, isrc, mos1, res, vsrc
    def setup(self):
        st = 0
        self.dev = {kk: [] for kk in range(7)}
        for kk in range(7):
            for idx in self.order[kk]:
                kind, name, nodes, extra, p, wf = self.inst[idx]
                if kind == K_CAP:
                    self.dev[kk].append((nodes, st, extra, p))
                    st += 2
                elif kind == K_BSIM4:
                    mtype, mp = self.models[extra]
                    par, need_dp, need_sp = bsim4_params(extra, mtype, mp, name, p, self.opts)
                    d, g, s, b = nodes
                    dp = self.mk(name + "#drain", True) if need_dp else d
                    sp = self.mk(name + "#source", True) if need_sp else s
                    self.dev[kk].append(([d, g, s, b, dp, sp], st, par))
                    st += lib().port_b4_nstate()
                elif kind == K_DIO:
                    mtype, mp = self.models[extra]
                    par, need_pp = dio_params(extra, mp, name, p, self.opts)
                    pos, neg = nodes
                    pp = self.mk(name + "#internal", True) if need_pp else pos
                    self.dev[kk].append(([pos, neg, pp], st, par))
                    st += lib().port_dio_nstate()
                elif kind == K_MOS1:
                    mtype, mp = self.models[extra]
                    par, need_dp, need_sp = mos1_params(mtype, mp, p, self.opts)
                    d, g, s, b = nodes
                    dp = self.mk(name + "#drain", True) if need_dp else d
                    sp = self.mk(name + "#source", True) if need_sp else s
                    self.dev[kk].append(([d, g, s, b, dp, sp], st, par))
                    st += 17
                elif kind == K_VSRC:
                    br = self.mk(name + "#branch", False)
                    self.dev[kk].append((nodes + [br], wf))
                elif kind == K_ISRC:
                    self.dev[kk].append((nodes + [0], wf))
                elif kind == K_RES:
                    self.dev[kk].append((nodes, extra, p))
        self.nstates = st
        self.n = len(self.names) - 1

    def run(self, dump: int = 0, max_steps: int = 10**8) -> dict:
        L = lib()
        h = L.port_new(self.n, self.nstates)
        try:
            nt = (C.c_int * (self.n + 1))(*self.ntype)
            L.port_set_ntype(h, nt)
            tstep, tstop = self.tran[0], self.tran[1]
            tstart = self.tran[2] if len(self.tran) > 2 else 0.0
            tmax = self.tran[3] if len(self.tran) > 3 else 0.0
            if tmax == 0:
                tmax = tstep if tstep < (tstop - tstart) / 50.0 else (tstop - tstart) / 50.0
            delmin = 1e-11 * tmax
            o = self.opts

            def opt(k, d):
                return evaluate(o[k]) if k in o else d
            dv = [opt("reltol", 1e-3), opt("abstol", 1e-12), opt("vntol", 1e-6),
                  opt("chgtol", 1e-14), opt("trtol", 7.0), opt("gmin", 1e-12),
                  opt("pivtol", 1e-13), opt("pivrel", 1e-3), 0.5, tstep, tstop, tstart,
                  tmax, delmin, 10.0 * delmin]
            # integration method (cktsopt.c OPT_METHOD): "method=gear" or
            # the bare flags "gear" / "trap", the last one given winning
            method = 0
            for k, v in o.items():
                if k == "method":
                    method = 1 if v == "gear" else 0
                elif k in ("gear", "trap"):
                    method = 1 if k == "gear" else 0
            # the order never exceeds 2 (DCtran raises it from 1 to 2 only), so
            # maxord >= 2 runs as 2 on the port's four state vectors
            iv = [int(opt("itl1", 100)), int(opt("itl4", 10)), min(int(opt("maxord", 2)), 2),
                  method]
            L.port_set_options(h, (C.c_double * len(dv))(*dv), (C.c_int * 4)(*iv))
            for nodes, st, cval, p in self.dev[K_CAP]:
                L.port_add_cap(h, nodes[0], nodes[1], st, cval, p.get("m", 1.0), p.get("ic", 0.0))
            for kk, isv in ((K_ISRC, 0), (K_VSRC, 1)):
                for nodes, wf in self.dev[kk]:
                    cf = (C.c_double * 64)(*wf["coef"])
                    # ISRC binds its first netlist node as the negative node
                    # (isrcdefs.h:30-31); VSRC binds it as the positive node
                    p_, n_ = (nodes[1], nodes[0]) if kk == K_ISRC else (nodes[0], nodes[1])
                    L.port_add_src(h, isv, p_, n_, nodes[2], wf["kind"],
                                   len(wf["coef"]), cf, wf["dc"], wf["dcgiven"], 1.0)
            for nodes, st, par in self.dev[K_MOS1]:
                L.port_add_mos1(h, (C.c_int * 6)(*nodes), st, (C.c_double * len(par))(*par))
            for nodes, st, par in self.dev[K_DIO]:
                L.port_add_dio(h, (C.c_int * 3)(*nodes), st, (C.c_double * len(par))(*par))
            for nodes, st, par in self.dev[K_BSIM4]:
                L.port_add_b4(h, (C.c_int * 6)(*nodes), st, (C.c_double * len(par))(*par))
            for nodes, r, p in self.dev[K_RES]:
                L.port_add_res(h, nodes[0], nodes[1], p.get("m", 1.0) / (r * 1.0 * 1.0))
            outcap = 1 << 16
            out = np.zeros((outcap, self.n + 1))
            L.port_set_output(h, out.ctypes.data_as(C.POINTER(C.c_double)), outcap)
            if dump:
                dax = np.zeros((dump, self.n + 1, self.n + 1))
                drhs = np.zeros((dump, self.n + 1))
                dro = np.zeros((dump, self.n + 1))
                dmeta = np.zeros((dump, 4))
                P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
                L.port_set_dump(h, P(dax), P(drhs), P(dro), P(dmeta), dump)
            stats = (C.c_long * 15)()
            L.port_run(h, stats, max_steps)
            st = list(stats)
            npts = min(st[7], outcap)
            res = {"names": self.names[1:], "times": out[:npts, 0].copy(),
                   "values": out[:npts, 1:].copy(),
                   "stats": {"numIter": st[0], "tranIter": st[1], "timePts": st[2],
                             "accepted": st[3], "rejected": st[4], "status": st[5],
                             "opIter": st[6], "npoints": st[7], "reorders": st[8]},
                   "plan": {"nlu": st[10], "levels": st[11], "rl_levels": st[12],
                            "btf_blocks": st[13], "multiply_adds": st[14]}}
            if dump:
                k = st[9]
                res.update(dump_ax=dax[:k], dump_rhs=drhs[:k], dump_rhsold=dro[:k],
                           dump_meta=dmeta[:k])
            return res
        finally:
            L.port_free(h)


def mos1_params(mtype: str, mp: dict, ip: dict, opts: dict):
    """MOS1setup defaults + MOS1temp + the hoisted head of MOS1load."""
    typ = 1 if mtype == "nmos" else -1
    g = mp.get
    latDiff = g("ld", 0.0)
    js = g("js", 0.0)
    is_ = g("is", 1e-14)
    kpGiven = "kp" in mp
    kp = g("kp", 2e-5)
    cgso, cgdo, cgbo = g("cgso", 0.0), g("cgdo", 0.0), g("cgbo", 0.0)
    vt0Given = "vto" in mp or "vt0" in mp
    vt0 = g("vto", g("vt0", 0.0))
    cjGiven, cjswGiven = "cj" in mp, "cjsw" in mp
    cj, cjsw = g("cj", 0.0), g("cjsw", 0.0)
    pb, mj, mjsw, fc = g("pb", 0.8), g("mj", 0.5), g("mjsw", 0.5), g("fc", 0.5)
    phiGiven = "phi" in mp
    phi = g("phi", 0.6)
    lam = g("lambda", 0.0)
    gammaGiven = "gamma" in mp
    gamma = g("gamma", 0.0)
    rd, rs, rsh = g("rd", 0.0), g("rs", 0.0), g("rsh", 0.0)
    cbd, cbs = g("cbd", 0.0), g("cbs", 0.0)
    toxGiven = "tox" in mp
    tox = g("tox", 0.0)
    u0Given = "u0" in mp or "uo" in mp
    u0 = g("u0", g("uo", 0.0))
    nsub = g("nsub", 0.0)
    tpg = g("tpg", 0.0)
    nss = g("nss", 0.0)
    tnom = (g("tnom", 0.0) + CTOK) if "tnom" in mp else 300.15
    temp = 300.15
    fact1 = tnom / REFTEMP
    vtnom = tnom * KOVERQ
    kt1 = BOLTZ * tnom
    egfet1 = 1.16 - (7.02e-4 * tnom * tnom) / (tnom + 1108)
    arg1 = -egfet1 / (kt1 + kt1) + 1.1150877 / (BOLTZ * (REFTEMP + REFTEMP))
    pbfact1 = -2 * vtnom * (1.5 * math.log(fact1) + CHARGE * arg1)
    oxideCapFactor = 0.0
    if toxGiven and tox != 0:
        oxideCapFactor = 3.9 * 8.854214871e-12 / tox
        if not kpGiven:
            if not u0Given:
                u0 = 600
            kp = u0 * oxideCapFactor * 1e-4
        if "nsub" in mp:
            if nsub * 1e6 > 1.45e16:
                if not phiGiven:
                    phi = max(.1, 2 * vtnom * math.log(nsub * 1e6 / 1.45e16))
                fermis = typ * .5 * phi
                wkfng = 3.2
                if "tpg" not in mp:
                    tpg = 1
                if tpg != 0:
                    fermig = typ * tpg * .5 * egfet1
                    wkfng = 3.25 + .5 * egfet1 - fermig
                wkfngs = wkfng - (3.25 + .5 * egfet1 + fermis)
                if not gammaGiven:
                    gamma = math.sqrt(2 * 11.70 * 8.854214871e-12 * CHARGE * nsub * 1e6) / oxideCapFactor
                if not vt0Given:
                    vfb = wkfngs - nss * 1e4 * CHARGE / oxideCapFactor
                    vt0 = vfb + typ * (gamma * math.sqrt(phi) + phi)
            else:
                raise ValueError("Nsub < Ni")
    mm = ip.get("m", 1.0)
    l, w = ip.get("l", 1e-4), ip.get("w", 1e-4)
    ad, as_ = ip.get("ad", 0.0), ip.get("as", 0.0)
    pd, ps = ip.get("pd", 0.0), ip.get("ps", 0.0)
    nrd, nrs = ip.get("nrd", 1.0), ip.get("nrs", 1.0)
    vt = temp * KOVERQ
    ratio = temp / tnom
    fact2 = temp / REFTEMP
    kt = temp * BOLTZ
    egfet = 1.16 - (7.02e-4 * temp * temp) / (temp + 1108)
    arg = -egfet / (kt + kt) + 1.1150877 / (BOLTZ * (REFTEMP + REFTEMP))
    pbfact = -2 * vt * (1.5 * math.log(fact2) + CHARGE * arg)
    ratio4 = ratio * math.sqrt(ratio)
    tTrans = kp / ratio4
    phio = (phi - pbfact1) / fact1
    tPhi = fact2 * phio + pbfact
    tVbi = vt0 - typ * (gamma * math.sqrt(phi)) + .5 * (egfet1 - egfet) + typ * .5 * (tPhi - phi)
    tVto = tVbi + typ * gamma * math.sqrt(tPhi)
    tSatCur = is_ * math.exp(-egfet / vt + egfet1 / vtnom)
    tSatCurDens = js * math.exp(-egfet / vt + egfet1 / vtnom)
    pbo = (pb - pbfact1) / fact1
    gmaold = (pb - pbo) / pbo
    capfact = 1 / (1 + mj * (4e-4 * (tnom - REFTEMP) - gmaold))
    tCbd, tCbs, tCj = cbd * capfact, cbs * capfact, cj * capfact
    capfact = 1 / (1 + mjsw * (4e-4 * (tnom - REFTEMP) - gmaold))
    tCjsw = cjsw * capfact
    tBulkPot = fact2 * pbo + pbfact
    gmanew = (tBulkPot - pbo) / pbo
    capfact = (1 + mj * (4e-4 * (temp - REFTEMP) - gmanew))
    tCbd *= capfact
    tCbs *= capfact
    tCj *= capfact
    capfact = (1 + mjsw * (4e-4 * (temp - REFTEMP) - gmanew))
    tCjsw *= capfact
    tDepCap = fc * tBulkPot
    if tSatCurDens == 0 or ad == 0 or as_ == 0:
        svc = dvc = vt * math.log(vt / (ROOT2 * mm * tSatCur))
    else:
        dvc = vt * math.log(vt / (ROOT2 * mm * tSatCurDens * ad))
        svc = vt * math.log(vt / (ROOT2 * mm * tSatCurDens * as_))
    czbd = tCbd * mm if "cbd" in mp else (tCj * mm * ad if cjGiven else 0.0)
    czbdsw = tCjsw * pd * mm if cjswGiven else 0.0
    a1 = 1 - fc
    sarg = math.exp((-mj) * math.log(a1))
    sargsw = math.exp((-mjsw) * math.log(a1))
    f2d = czbd * (1 - fc * (1 + mj)) * sarg / a1 + czbdsw * (1 - fc * (1 + mjsw)) * sargsw / a1
    f3d = czbd * mj * sarg / a1 / tBulkPot + czbdsw * mjsw * sargsw / a1 / tBulkPot
    f4d = (czbd * tBulkPot * (1 - a1 * sarg) / (1 - mj) + czbdsw * tBulkPot * (1 - a1 * sargsw) / (1 - mjsw)
           - f3d / 2 * (tDepCap * tDepCap) - tDepCap * f2d)
    czbs = tCbs * mm if "cbs" in mp else (tCj * as_ * mm if cjGiven else 0.0)
    czbssw = tCjsw * ps * mm if cjswGiven else 0.0
    f2s = czbs * (1 - fc * (1 + mj)) * sarg / a1 + czbssw * (1 - fc * (1 + mjsw)) * sargsw / a1
    f3s = czbs * mj * sarg / a1 / tBulkPot + czbssw * mjsw * sargsw / a1 / tBulkPot
    f4s = (czbs * tBulkPot * (1 - a1 * sarg) / (1 - mj) + czbssw * tBulkPot * (1 - a1 * sargsw) / (1 - mjsw)
           - f3s / 2 * (tDepCap * tDepCap) - tDepCap * f2s)
    if "rd" in mp:
        gd = mm / rd if rd != 0 else 0.0
    elif "rsh" in mp:
        gd = mm / (rsh * nrd) if rsh != 0 else 0.0
    else:
        gd = 0.0
    if "rs" in mp:
        gs = mm / rs if rs != 0 else 0.0
    elif "rsh" in mp:
        gs = mm / (rsh * nrs) if (rsh != 0 and nrs != 0) else 0.0
    else:
        gs = 0.0
    Leff = l - 2 * latDiff
    if tSatCurDens == 0 or ad == 0 or as_ == 0:
        dsat = ssat = mm * tSatCur
    else:
        dsat = tSatCurDens * mm * ad
        ssat = tSatCurDens * mm * as_
    par = [typ, KOVERQ * temp, dsat, ssat, cgso * mm * w, cgdo * mm * w, cgbo * mm * Leff,
           tTrans * mm * w / Leff, oxideCapFactor * Leff * mm * w, tPhi, tVbi, tVto, gamma, lam,
           svc, dvc, czbs, czbssw, czbd, czbdsw, tDepCap, tBulkPot, f2s, f3s, f4s, f2d, f3d, f4d,
           mj, mjsw, gd, gs, 1.0 if "off" in ip else 0.0, ip.get("icvds", 0.0),
           ip.get("icvgs", 0.0), ip.get("icvbs", 0.0)]
    need_dp = rd != 0 or (rsh != 0 and nrd != 0)
    need_sp = rs != 0 or (rsh != 0 and nrs != 0)
    return [float(x) for x in par], need_dp, need_sp


def _temps(opts: dict) -> tuple[float, float]:
    temp = evaluate(opts["temp"]) + CTOK if "temp" in opts else 300.15
    tnom = evaluate(opts["tnom"]) + CTOK if "tnom" in opts else 300.15
    return temp, tnom


def bsim4_params(mname: str, mtype: str, mp: dict, iname: str, ip: dict, opts: dict):
    """BSIM4setup + BSIM4temp for one instance through the shared model
    arithmetic (b4port.cpp); returns the parameter vector and whether
    internal drain/source nodes are needed."""
    L = lib()
    mk = [k for k in mp if k != "level"]
    ik = list(ip)
    temp, tnom = _temps(opts)
    npar = L.port_b4_nparam()
    out = (C.c_double * npar)()
    ndp, nsp = C.c_int(), C.c_int()
    err = C.create_string_buffer(512)
    rc = L.port_b4_params(mname.encode(), 1 if mtype == "nmos" else -1, len(mk),
                          (C.c_char_p * max(1, len(mk)))(*[k.encode() for k in mk]),
                          (C.c_double * max(1, len(mk)))(*[float(mp[k]) for k in mk]),
                          iname.encode(), len(ik),
                          (C.c_char_p * max(1, len(ik)))(*[k.encode() for k in ik]),
                          (C.c_double * max(1, len(ik)))(*[float(ip[k]) for k in ik]),
                          temp, tnom, out, C.byref(ndp), C.byref(nsp), err, 512)
    if rc != 0:
        raise ValueError("oracle port: " + err.value.decode())
    return list(out), bool(ndp.value), bool(nsp.value)


def dio_params(mname: str, mp: dict, iname: str, ip: dict, opts: dict):
    """DIOsetup + DIOtemp for one diode through the shared arithmetic
    (b4port.cpp); returns the parameter vector and whether the series
    resistance needs an internal node."""
    L = lib()
    mk = list(mp)
    ik = list(ip)
    temp, tnom = _temps(opts)
    reltol = evaluate(opts["reltol"]) if "reltol" in opts else 1e-3
    out = (C.c_double * L.port_dio_nparam())()
    npp = C.c_int()
    err = C.create_string_buffer(512)
    rc = L.port_dio_params(mname.encode(), len(mk),
                           (C.c_char_p * max(1, len(mk)))(*[k.encode() for k in mk]),
                           (C.c_double * max(1, len(mk)))(*[float(mp[k]) for k in mk]),
                           iname.encode(), len(ik),
                           (C.c_char_p * max(1, len(ik)))(*[k.encode() for k in ik]),
                           (C.c_double * max(1, len(ik)))(*[float(ip[k]) for k in ik]),
                           temp, tnom, reltol, out, C.byref(npp), err, 512)
    if rc != 0:
        raise ValueError("oracle port: " + err.value.decode())
    return list(out), bool(npp.value)


def simulate(text: str, **kw) -> dict:
    return Circuit(text).run(**kw)
