"""ctypes binding of libngspice_gb300.so (include/ngspice_gb300.h and
include/sharedspice.h).

The library is the product: this module only loads it and converts
arguments.  There is no CPU fallback: if the library or a CUDA device is
missing, the calls fail with the library's error message.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libngspice_gb300.so")

# integer result slots (ngsf_types.h NGSF_R_*)
R_STATUS, R_NPOINTS, R_ACCEPTED, R_REJECTED, R_NUMITER, R_TRANITER, R_TIMEPTS, \
    R_NCAP, R_OPITER, R_BADPIVOT, R_REORDERS, R_GUESSES, R_GUESS1, R_FALLBACKS = range(14)
R_COUNT = 14
F_COUNT = 3

# C-ABI symbols declared in include/*.h
EXPORTS = [
    "ngsf_open", "ngsf_open_many", "ngsf_compile", "ngsf_close", "ngsf_last_error", "ngsf_info",
    "ngsf_eq_name", "ngsf_pattern", "ngsf_probes", "ngsf_run", "ngsf_run_window", "ngsf_results",
    "ngsf_points", "ngsf_capture", "ngsf_lu_flops", "ngsf_device_bytes",
    "ngsf_last_launches", "ngsf_workload", "ngsf_stamp_initial_static",
    "ngsf_gnn_param_count", "ngsf_gnn_create", "ngsf_gnn_destroy", "ngsf_gnn_set_params",
    "ngsf_gnn_get_params", "ngsf_gnn_forward", "ngsf_gnn_train_step", "ngsf_gnn_gemm_test",
    "ngsf_node_graph", "ngsf_set_predictor", "ngsf_wide_info", "ngsf_set_factor_shape",
    "ngsf_dev_table", "ngsf_ckt_load", "ngsf_ckt_read_states", "ngsf_ckt_trunc",
    "ngsf_ni_convtest", "ngsf_smp_set_matrix", "ngsf_smp_get_matrix", "ngsf_smp_reorder",
    "ngsf_smp_lufac", "ngsf_smp_solve", "ngsf_phase_cycles", "ngsf_eval_bench",
    "ngsf_fp64_peak", "ngsf_smp_preorder", "ngsf_set_sync", "ngsf_sync_point",
    "ngsf_sync_reply",
    "ngSpice_Init", "ngSpice_Init_Sync", "ngSpice_Command", "ngGet_Vec_Info",
    "ngSpice_Circ", "ngSpice_CurPlot", "ngSpice_AllPlots", "ngSpice_AllVecs",
    "ngSpice_running", "ngSpice_SetBkpt", "ngSpice_nospinit", "ngSpice_nospiceinit",
    "ngSpice_LockRealloc", "ngSpice_UnlockRealloc", "ngSpice_Reset",
]

_lib = None

# device types in the reference's device-table order (NGSF_DEV_*)
DEV_BSIM4, DEV_CAP, DEV_DIO, DEV_ISRC, DEV_MOS1, DEV_RES, DEV_VSRC = range(7)
DEV_ALL = (1 << 7) - 1
E_SINGULAR = 102


class EngineError(RuntimeError):
    pass


class Point(C.Structure):
    """ngsf_point: the CKTcircuit control scalars of one operation."""
    _fields_ = [("time", C.c_double), ("delta", C.c_double), ("deltaOld", C.c_double * 3),
                ("ag", C.c_double * 3), ("gmin", C.c_double), ("srcFact", C.c_double),
                ("diagGmin", C.c_double), ("mode", C.c_int), ("order", C.c_int)]


class DevInfo(C.Structure):
    _fields_ = [("name", C.c_char_p), ("states", C.c_int), ("stamps", C.c_int),
                ("has_load", C.c_int), ("has_trunc", C.c_int), ("has_accept", C.c_int)]


def make_point(time=0.0, delta=0.0, deltaOld=(0.0, 0.0, 0.0), ag=(0.0, 0.0, 0.0), gmin=1e-12,
               srcFact=1.0, diagGmin=0.0, mode=0, order=1) -> Point:
    p = Point()
    p.time, p.delta, p.gmin, p.srcFact, p.diagGmin = time, delta, gmin, srcFact, diagGmin
    p.mode, p.order = int(mode), int(order)
    for k in range(3):
        p.deltaOld[k] = deltaOld[k] if k < len(deltaOld) else 0.0
    for k in range(3):
        p.ag[k] = ag[k] if k < len(ag) else 0.0
    return p


def dev_table() -> list[dict]:
    """The device table (ngsf_dev_table), one dict per device type."""
    n = C.c_int()
    t = C.POINTER(DevInfo)()
    lib().ngsf_dev_table(C.byref(n), C.byref(t))
    return [{"name": t[k].name.decode(), "states": t[k].states, "stamps": t[k].stamps,
             "load": bool(t[k].has_load), "trunc": bool(t[k].has_trunc),
             "accept": bool(t[k].has_accept)} for k in range(n.value)]


def lib(path: str | None = None) -> C.CDLL:
    """Load (once) and type the shared library."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise EngineError(f"{p} is missing: build it with ngspice_gb300.build.build()")
    L = C.CDLL(p)
    vp, ip, dp, cp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_char_p
    L.ngsf_open.restype = vp
    L.ngsf_open.argtypes = [cp, cp, C.c_int, C.c_int]
    L.ngsf_open_many.argtypes = [C.POINTER(cp), C.c_int, cp, C.c_int, C.c_int, C.POINTER(vp)]
    L.ngsf_compile.restype = vp
    L.ngsf_wide_info.argtypes = [vp, ip, ip]
    L.ngsf_set_factor_shape.argtypes = [vp, C.c_int, C.c_int]
    L.ngsf_compile.argtypes = [cp]
    L.ngsf_close.argtypes = [vp]
    L.ngsf_last_error.restype = cp
    L.ngsf_info.argtypes = [vp, ip, ip, ip, ip]
    L.ngsf_eq_name.argtypes = [vp, C.c_int, cp, C.c_int]
    L.ngsf_pattern.argtypes = [vp, ip, ip]
    L.ngsf_probes.argtypes = [vp, ip, C.c_int]
    L.ngsf_run.argtypes = [C.POINTER(vp), C.c_int, C.c_longlong, dp]
    L.ngsf_run_window.argtypes = [C.POINTER(vp), C.c_int, C.c_double, C.c_longlong, dp]
    L.ngsf_results.argtypes = [vp, ip, dp]
    L.ngsf_points.argtypes = [vp, dp, C.c_int]
    L.ngsf_capture.argtypes = [vp, dp, dp, dp, dp, C.c_int]
    L.ngsf_lu_flops.restype = C.c_double
    L.ngsf_lu_flops.argtypes = [vp]
    L.ngsf_device_bytes.restype = C.c_longlong
    L.ngsf_device_bytes.argtypes = [vp]
    L.ngsf_last_launches.restype = C.c_int
    L.ngsf_workload.argtypes = [vp, C.POINTER(C.c_longlong)]
    pp = C.POINTER(Point)
    L.ngsf_dev_table.argtypes = [ip, C.POINTER(C.POINTER(DevInfo))]
    L.ngsf_ckt_load.argtypes = [vp, pp, C.c_int, dp, dp, C.c_int, dp, dp, dp, ip]
    L.ngsf_ckt_read_states.argtypes = [vp, dp, C.c_int]
    L.ngsf_ckt_trunc.argtypes = [vp, pp, dp, C.c_int, dp]
    L.ngsf_ni_convtest.argtypes = [vp, dp, dp, ip]
    L.ngsf_smp_set_matrix.argtypes = [vp, dp]
    L.ngsf_smp_get_matrix.argtypes = [vp, dp]
    L.ngsf_smp_reorder.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    L.ngsf_smp_lufac.argtypes = [vp, C.c_double]
    L.ngsf_smp_solve.argtypes = [vp, dp]
    L.ngsf_phase_cycles.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.ngsf_eval_bench.argtypes = [vp, pp, C.c_int, C.c_int, C.c_int, dp]
    L.ngsf_fp64_peak.argtypes = [dp]
    L.ngsf_smp_preorder.argtypes = [vp, ip, ip]
    L.ngsf_set_sync.argtypes = [vp, C.c_int]
    L.ngsf_sync_point.argtypes = [vp, ip, ip, dp, dp, dp]
    L.ngsf_sync_reply.argtypes = [vp, C.c_double, C.c_int]
    fp = C.POINTER(C.c_float)
    if hasattr(L, "ngsf_node_graph"):
        L.ngsf_node_graph.argtypes = [vp, ip, ip, ip, ip, ip, fp]
        L.ngsf_set_predictor.argtypes = [vp, C.c_int, fp]
    _lib = L
    return L


def last_error() -> str:
    return (lib().ngsf_last_error() or b"").decode()


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Circuit:
    """One compiled circuit (device resident unless host_only)."""

    def __init__(self, netlist: str, probes: list[str] | None = None, outcap: int = 200000,
                 capmax: int = 0, host_only: bool = False):
        L = lib()
        if host_only:
            h = L.ngsf_compile(netlist.encode())
        else:
            pr = " ".join(probes).encode() if probes else None
            h = L.ngsf_open(netlist.encode(), pr, int(outcap), int(capmax))
        if not h:
            raise EngineError(last_error())
        self._adopt(h, host_only)

    @classmethod
    def _from_handle(cls, h) -> "Circuit":
        c = cls.__new__(cls)
        c._adopt(h, False)
        return c

    def _adopt(self, h, host_only: bool):
        L = lib()
        self._h = C.c_void_p(h)
        n, nnz, ns, nlu = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.ngsf_info(self._h, C.byref(n), C.byref(nnz), C.byref(ns), C.byref(nlu))
        self.n, self.nnz, self.nstates, self.nlu = n.value, nnz.value, ns.value, nlu.value
        self.host_only = host_only

    def wide_info(self) -> tuple[bool, int]:
        """(runs over the whole grid when alone, blocks of that launch)"""
        w, b = C.c_int(), C.c_int()
        if lib().ngsf_wide_info(self._h, C.byref(w), C.byref(b)):
            raise EngineError(last_error())
        return bool(w.value), b.value

    def set_factor_shape(self, blocks: int = 0, small_work: int = 0):
        """Refactorization shape of the wide launch (0 = default); every
        shape gives the same result."""
        if lib().ngsf_set_factor_shape(self._h, int(blocks), int(small_work)):
            raise EngineError(last_error())

    def close(self):
        if self._h:
            lib().ngsf_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def names(self) -> list[str]:
        buf = C.create_string_buffer(512)
        out = []
        for i in range(1, self.n + 1):
            lib().ngsf_eq_name(self._h, i, buf, 512)
            out.append(buf.value.decode())
        return out

    def pattern(self) -> tuple[np.ndarray, np.ndarray]:
        cp = np.zeros(self.n + 1, np.int32)
        ri = np.zeros(self.nnz, np.int32)
        lib().ngsf_pattern(self._h, _ptr(cp, C.c_int), _ptr(ri, C.c_int))
        return cp, ri

    def probes(self) -> np.ndarray:
        buf = np.zeros(self.n + 1, np.int32)
        k = lib().ngsf_probes(self._h, _ptr(buf, C.c_int), self.n + 1)
        return buf[:k].copy()

    def results(self) -> np.ndarray:
        ires = np.zeros(R_COUNT, np.int32)
        fres = np.zeros(F_COUNT)
        if lib().ngsf_results(self._h, _ptr(ires, C.c_int), _ptr(fres, C.c_double)):
            raise EngineError(last_error())
        return ires

    def points(self) -> tuple[np.ndarray, np.ndarray]:
        """(times[np], values[np, nprobe]) of the accepted points."""
        ires = self.results()
        npts = int(ires[R_NPOINTS])
        w = 1 + len(self.probes())
        buf = np.zeros((max(npts, 1), w))
        k = lib().ngsf_points(self._h, _ptr(buf, C.c_double), npts)
        return buf[:k, 0].copy(), buf[:k, 1:].copy()

    def capture(self, maxcap: int) -> dict:
        ax = np.zeros((maxcap, self.nnz))
        rhs = np.zeros((maxcap, self.n + 1))
        rhsold = np.zeros((maxcap, self.n + 1))
        meta = np.zeros((maxcap, 4))
        k = lib().ngsf_capture(self._h, _ptr(ax, C.c_double), _ptr(rhs, C.c_double),
                               _ptr(rhsold, C.c_double), _ptr(meta, C.c_double), maxcap)
        if k < 0:
            raise EngineError(last_error())
        return {"ax": ax[:k], "rhs": rhs[:k], "rhsold": rhsold[:k], "meta": meta[:k]}

    def lu_flops(self) -> float:
        return float(lib().ngsf_lu_flops(self._h))

    def device_bytes(self) -> int:
        return int(lib().ngsf_device_bytes(self._h))

    def node_graph(self) -> dict:
        """The predictor's view: voltage unknowns (0-based equation index),
        neighbour CSR and log(1 + terminal counts)."""
        L = lib()
        nv, ne = C.c_int(), C.c_int()
        L.ngsf_node_graph(self._h, C.byref(nv), C.byref(ne), None, None, None, None)
        vnode = np.zeros(nv.value, np.int32)
        gptr = np.zeros(nv.value + 1, np.int32)
        gidx = np.zeros(max(ne.value, 1), np.int32)
        stat = np.zeros((nv.value, 6), np.float32)
        if L.ngsf_node_graph(self._h, None, None, _ptr(vnode, C.c_int), _ptr(gptr, C.c_int),
                             _ptr(gidx, C.c_int), stat.ctypes.data_as(C.POINTER(C.c_float))):
            raise EngineError(last_error())
        return {"vnode": vnode - 1, "gptr": gptr, "gidx": gidx[:ne.value], "stat": stat}

    def set_predictor(self, kind: int, params: np.ndarray | None = None):
        """0: off (the reference's Newton start), 1: linear extrapolation,
        3: quadratic extrapolation, 2: quadratic plus the trained network's
        correction (flat parameters)."""
        p = None
        if params is not None:
            params = np.ascontiguousarray(params, np.float32)
            self._pred_params = params
            p = params.ctypes.data_as(C.POINTER(C.c_float))
        if lib().ngsf_set_predictor(self._h, int(kind), p):
            raise EngineError(last_error())

    def smp_preorder(self) -> tuple[int, int]:
        """SMPpreOrder's block triangular analysis: (diagonal blocks,
        largest block)."""
        nb, big = C.c_int(), C.c_int()
        if lib().ngsf_smp_preorder(self._h, C.byref(nb), C.byref(big)):
            raise EngineError(last_error())
        return nb.value, big.value

    # ---- synchronised runs (sharedspice GetSyncData) ----
    def set_sync(self, on: bool = True):
        """Stop also at the two sharedsync points of every step."""
        if lib().ngsf_set_sync(self._h, 1 if on else 0):
            raise EngineError(last_error())

    def sync_point(self) -> dict | None:
        """The sharedsync stop the run is at, or None."""
        loc, redo = C.c_int(), C.c_int()
        t, d, od = C.c_double(), C.c_double(), C.c_double()
        if not lib().ngsf_sync_point(self._h, C.byref(loc), C.byref(redo), C.byref(t),
                                     C.byref(d), C.byref(od)):
            return None
        return {"loc": loc.value, "redostep": redo.value, "time": t.value, "delta": d.value,
                "olddelta": od.value}

    def sync_reply(self, delta: float, redo: int = 0):
        """The caller's delta for the next step and its return value."""
        if lib().ngsf_sync_reply(self._h, float(delta), int(redo)):
            raise EngineError(last_error())

    # ---- operator surface (CKTload / DEVload, CKTtrunc, NIconvTest, SMP*) ----
    def ckt_load(self, point: Point, types: int = DEV_ALL, rhs_old=None, states=None,
                 von=None) -> tuple[np.ndarray, np.ndarray, int]:
        """(ax[nnz], rhs[n+1], noncon) of one CKTload at the given point."""
        ax = np.zeros(self.nnz)
        rhs = np.zeros(self.n + 1)
        nc = C.c_int()
        ro = None if rhs_old is None else np.ascontiguousarray(rhs_old, np.float64)
        st = None if states is None else np.ascontiguousarray(states, np.float64)
        vo = None if von is None else np.ascontiguousarray(von, np.float64)
        nvec = 0 if st is None else st.shape[0]
        if lib().ngsf_ckt_load(self._h, C.byref(point), int(types),
                               None if ro is None else _ptr(ro, C.c_double),
                               None if st is None else _ptr(st, C.c_double), nvec,
                               None if vo is None else _ptr(vo, C.c_double),
                               _ptr(ax, C.c_double), _ptr(rhs, C.c_double), C.byref(nc)):
            raise EngineError(last_error())
        return ax, rhs, nc.value

    def read_states(self, nvec: int = 4) -> np.ndarray:
        out = np.zeros((nvec, self.nstates))
        if lib().ngsf_ckt_read_states(self._h, _ptr(out, C.c_double), nvec):
            raise EngineError(last_error())
        return out

    def ckt_trunc(self, point: Point, states) -> float:
        st = np.ascontiguousarray(states, np.float64)
        t = C.c_double()
        if lib().ngsf_ckt_trunc(self._h, C.byref(point), _ptr(st, C.c_double), st.shape[0],
                                C.byref(t)):
            raise EngineError(last_error())
        return t.value

    def ni_convtest(self, rhs, rhs_old) -> int:
        a = np.ascontiguousarray(rhs, np.float64)
        b = np.ascontiguousarray(rhs_old, np.float64)
        nc = C.c_int()
        if lib().ngsf_ni_convtest(self._h, _ptr(a, C.c_double), _ptr(b, C.c_double),
                                  C.byref(nc)):
            raise EngineError(last_error())
        return nc.value

    def smp_set_matrix(self, ax):
        a = np.ascontiguousarray(ax, np.float64)
        if lib().ngsf_smp_set_matrix(self._h, _ptr(a, C.c_double)):
            raise EngineError(last_error())

    def smp_get_matrix(self) -> np.ndarray:
        a = np.zeros(self.nnz)
        if lib().ngsf_smp_get_matrix(self._h, _ptr(a, C.c_double)):
            raise EngineError(last_error())
        return a

    def smp_reorder(self, pivtol: float = 1e-13, pivrel: float = 1e-3,
                    diag_gmin: float = 0.0) -> int:
        """0, or E_SINGULAR; raises on an error."""
        r = lib().ngsf_smp_reorder(self._h, pivtol, pivrel, diag_gmin)
        if r not in (0, E_SINGULAR):
            raise EngineError(last_error())
        return r

    def smp_lufac(self, diag_gmin: float = 0.0) -> int:
        r = lib().ngsf_smp_lufac(self._h, diag_gmin)
        if r not in (0, E_SINGULAR):
            raise EngineError(last_error())
        return r

    def smp_solve(self, rhs) -> np.ndarray:
        x = np.array(rhs, dtype=np.float64, copy=True)
        if lib().ngsf_smp_solve(self._h, _ptr(x, C.c_double)):
            raise EngineError(last_error())
        return x

    def phase_cycles(self) -> dict:
        """SM clock cycles per phase of the last run (opened with NGSF_PHASES=1)."""
        a = (C.c_longlong * 8)()
        if lib().ngsf_phase_cycles(self._h, a):
            raise EngineError(last_error())
        keys = ["load", "gather", "factor", "solve", "conv", "trunc", "total", "iterations"]
        return dict(zip(keys, [int(x) for x in a]))

    def eval_bench(self, point: Point, types: int, reps: int = 10, blocks: int = 0) -> float:
        """Device seconds of `reps` grid-wide evaluations of the selected
        device types (ngsf_eval_bench)."""
        sec = C.c_double()
        if lib().ngsf_eval_bench(self._h, C.byref(point), int(types), int(reps), int(blocks),
                                 C.byref(sec)):
            raise EngineError(last_error())
        return sec.value

    def workload(self) -> dict:
        a = (C.c_longlong * 10)()
        lib().ngsf_workload(self._h, a)
        keys = ["mos1", "res", "cap", "vsrc", "isrc", "nnz", "nlu", "n", "bsim4", "dio"]
        return dict(zip(keys, [int(x) for x in a]))


def fp64_peak() -> float:
    """Measured FP64 FMA throughput of the device, flop/s (ngsf_fp64_peak)."""
    f = C.c_double()
    if lib().ngsf_fp64_peak(C.byref(f)):
        raise EngineError(last_error())
    return f.value


def last_launches() -> int:
    return int(lib().ngsf_last_launches())


def open_many(netlists: list[str], probes: list[str] | None = None, outcap: int = 200000,
              capmax: int = 0) -> list[Circuit]:
    """Circuit(...) for a batch of netlists with the same probes (ngsf_open_many:
    parsing and setup on all host cores)."""
    n = len(netlists)
    if n == 0:
        return []
    texts = (C.c_char_p * n)(*[t.encode() for t in netlists])
    out = (C.c_void_p * n)()
    pr = " ".join(probes).encode() if probes else None
    if lib().ngsf_open_many(texts, n, pr, int(outcap), int(capmax), out):
        raise EngineError(last_error())
    return [Circuit._from_handle(out[i]) for i in range(n)]


def tune_factor_shape(circuit: Circuit, blocks=(16, 24, 32, 48, 64, 96, 152),
                      small_works=(256, 1024, 4096, 16384, 1 << 30), warm: float = 6e-12,
                      window: float = 3e-12, repeats: int = 2) -> dict:
    """Autotuner of the wide refactorization over the circuit's level
    schedule.  One run is advanced untimed to `warm` (the operating point
    and the first steps); then each shape is timed over the next windows of
    `window` seconds of that run, as device time per Newton iteration (the
    refactorization and solve structure is fixed, so the cost per iteration
    compares shapes across windows), best of `repeats`: first every group
    size at the default small-level threshold, then each threshold at the
    best group size (the largest threshold runs every level in one block).
    The fastest shape is left set on the circuit; every shape computes the
    same bits, so tuning changes no waveform.  A circuit that does not run
    wide keeps the default.  Returns the choice and the timings."""
    wide, nb = circuit.wide_info()
    if not wide:
        return {"blocks": 0, "small_work": 0, "timings": {}}
    state = {"t": warm}
    run_window([circuit], warm)

    def time_shape(b: int, sw: int) -> float:
        circuit.set_factor_shape(b, sw)
        best = float("inf")
        for _ in range(repeats):
            before = int(circuit.results()[R_NUMITER])
            state["t"] += window
            sec = run_window([circuit], state["t"])
            r = circuit.results()
            iters = int(r[R_NUMITER]) - before
            if r[R_STATUS] == PAUSED and iters > 0:
                best = min(best, sec / iters)
        return best

    timings = {}
    for b in [b for b in blocks if b <= nb] or [nb]:
        timings[(b, 0)] = time_shape(b, 0)
    best_b = min(timings, key=timings.get)[0]
    for sw in small_works:
        timings[(best_b, sw)] = time_shape(best_b, sw)
    best = min(timings, key=timings.get)
    circuit.set_factor_shape(*best)
    return {"blocks": best[0], "small_work": best[1], "timings": timings}


# status of a circuit stopped at the end of a window (ngsf_run_window)
PAUSED = -3


def run(circuits: list[Circuit], max_steps: int = 0) -> float:
    """Run .tran on all circuits in one GPU launch; returns device seconds."""
    arr = (C.c_void_p * len(circuits))(*[c.handle for c in circuits])
    sec = C.c_double(0)
    if lib().ngsf_run(arr, len(circuits), int(max_steps), C.byref(sec)):
        raise EngineError(last_error())
    return sec.value


def run_window(circuits: list[Circuit], t_until: float, max_steps: int = 0) -> float:
    """Advance every circuit's transient to t_until (ngsf_run_window):
    circuits stopped by an earlier window continue, the others start
    fresh.  Returns device seconds."""
    arr = (C.c_void_p * len(circuits))(*[c.handle for c in circuits])
    sec = C.c_double(0)
    if lib().ngsf_run_window(arr, len(circuits), float(t_until), int(max_steps), C.byref(sec)):
        raise EngineError(last_error())
    return sec.value
