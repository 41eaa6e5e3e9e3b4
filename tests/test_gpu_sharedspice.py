"""GPU: the sharedspice-compatible C API driven the way an embedding
application drives the reference shared library."""
import ctypes as C
import time

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


class VectorInfo(C.Structure):
    _fields_ = [("v_name", C.c_char_p), ("v_type", C.c_int), ("v_flags", C.c_short),
                ("v_realdata", C.POINTER(C.c_double)), ("v_compdata", C.c_void_p),
                ("v_length", C.c_int)]


SendChar = C.CFUNCTYPE(C.c_int, C.c_char_p, C.c_int, C.c_void_p)
SendStat = C.CFUNCTYPE(C.c_int, C.c_char_p, C.c_int, C.c_void_p)
ControlledExit = C.CFUNCTYPE(C.c_int, C.c_int, C.c_bool, C.c_bool, C.c_int, C.c_void_p)
SendData = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p)
SendInitData = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_void_p)
BGThreadRunning = C.CFUNCTYPE(C.c_int, C.c_bool, C.c_int, C.c_void_p)


# The library keeps the callback pointers registered by ngSpice_Init (as the
# reference does), so the ctypes thunks must live as long as the module.
_KEEP = []


@pytest.fixture(scope="module")
def ng(built_lib):
    L = C.CDLL(built_lib)
    L.ngGet_Vec_Info.restype = C.POINTER(VectorInfo)
    L.ngGet_Vec_Info.argtypes = [C.c_char_p]
    L.ngSpice_Command.argtypes = [C.c_char_p]
    L.ngSpice_Circ.argtypes = [C.POINTER(C.c_char_p)]
    L.ngSpice_CurPlot.restype = C.c_char_p
    L.ngSpice_AllVecs.restype = C.POINTER(C.c_char_p)
    L.ngSpice_AllVecs.argtypes = [C.c_char_p]
    L.ngSpice_running.restype = C.c_bool
    return L


def test_circ_tran_and_vectors(ng):
    out, points = [], []
    keep = _KEEP
    cb_char = SendChar(lambda s, i, u: out.append(s) or 0)
    cb_stat = SendStat(lambda s, i, u: 0)
    cb_exit = ControlledExit(lambda *a: 0)
    cb_data = SendData(lambda p, n, i, u: points.append(n) or 0)
    cb_init = SendInitData(lambda p, i, u: 0)
    cb_bg = BGThreadRunning(lambda r, i, u: 0)
    keep += [cb_char, cb_stat, cb_exit, cb_data, cb_init, cb_bg]
    assert ng.ngSpice_Init(cb_char, cb_stat, cb_exit, cb_data, cb_init, cb_bg, None) == 0
    g = golden("rc_ladder")
    lines = [ln.encode() for ln in str(g["netlist"]).splitlines()]
    arr = (C.c_char_p * (len(lines) + 1))(*lines, None)
    assert ng.ngSpice_Circ(arr) == 0
    assert ng.ngSpice_Command(b"run") == 0
    assert ng.ngSpice_CurPlot().decode().startswith("tran")
    t = ng.ngGet_Vec_Info(b"time").contents
    v = ng.ngGet_Vec_Info(b"v(n8)").contents
    assert t.v_length == len(g["times"]) == v.v_length
    tt = np.ctypeslib.as_array(t.v_realdata, shape=(t.v_length,))
    vv = np.ctypeslib.as_array(v.v_realdata, shape=(v.v_length,))
    names = list(g["names"])
    np.testing.assert_array_equal(tt, g["times"])
    assert np.max(np.abs(vv - g["values"][:, names.index("n8")])) < 1e-12
    assert len(points) == len(g["times"])
    vecs = ng.ngSpice_AllVecs(ng.ngSpice_CurPlot())
    got = []
    i = 0
    while vecs[i]:
        got.append(vecs[i].decode())
        i += 1
    assert "time" in got and "n8" in got


def test_tran_command_overrides_deck(ng):
    g = golden("rc_ladder")
    lines = [ln.encode() for ln in str(g["netlist"]).splitlines()]
    arr = (C.c_char_p * (len(lines) + 1))(*lines, None)
    assert ng.ngSpice_Circ(arr) == 0
    assert ng.ngSpice_Command(b"tran 10p 4n") == 0
    t = ng.ngGet_Vec_Info(b"time").contents
    tt = np.ctypeslib.as_array(t.v_realdata, shape=(t.v_length,))
    assert abs(tt[-1] - 4e-9) < 1e-18


def test_bg_run_and_errors(ng):
    g = golden("rc_ladder")
    lines = [ln.encode() for ln in str(g["netlist"]).splitlines()]
    arr = (C.c_char_p * (len(lines) + 1))(*lines, None)
    assert ng.ngSpice_Circ(arr) == 0
    assert ng.ngSpice_Command(b"bg_run") == 0
    assert ng.ngSpice_Command(b"bg_halt") == 0     # waits for the run
    assert not ng.ngSpice_running()
    assert ng.ngSpice_Command(b"frobnicate") == 1


def test_points_stream_and_halt_resume(ng):
    """SendData streams accepted points as the run's windows end, with
    SendStat progress in between; bg_halt stops a background run at a
    window end and bg_resume continues it to the same result as an
    uninterrupted run."""
    stats, points, done = [], [], []
    keep = _KEEP
    cb_char = SendChar(lambda s, i, u: 0)
    cb_stat = SendStat(lambda s, i, u: stats.append(s.decode()) or 0)
    cb_exit = ControlledExit(lambda *a: 0)
    cb_data = SendData(lambda p, n, i, u: points.append(len(stats)) or 0)
    cb_init = SendInitData(lambda p, i, u: 0)
    cb_bg = BGThreadRunning(lambda r, i, u: done.append(bool(r)) or 0)
    keep += [cb_char, cb_stat, cb_exit, cb_data, cb_init, cb_bg]
    assert ng.ngSpice_Init(cb_char, cb_stat, cb_exit, cb_data, cb_init, cb_bg, None) == 0
    g = golden("rc_ladder")
    lines = [ln.encode() for ln in str(g["netlist"]).splitlines()]
    arr = (C.c_char_p * (len(lines) + 1))(*lines, None)
    assert ng.ngSpice_Circ(arr) == 0
    assert ng.ngSpice_Command(b"bg_run") == 0
    assert ng.ngSpice_Command(b"bg_halt") == 0
    assert not ng.ngSpice_running()
    halted_at = ng.ngGet_Vec_Info(b"time").contents.v_length
    # a halted run resumes until it ends (halting again on the way)
    for _ in range(200):
        if ng.ngGet_Vec_Info(b"time").contents.v_length >= len(g["times"]):
            break
        assert ng.ngSpice_Command(b"bg_resume") == 0
        time.sleep(0.01)
        assert ng.ngSpice_Command(b"bg_halt") == 0
        assert not ng.ngSpice_running()
    t = ng.ngGet_Vec_Info(b"time").contents
    tt = np.ctypeslib.as_array(t.v_realdata, shape=(t.v_length,))
    np.testing.assert_array_equal(tt, g["times"])
    assert len(points) == len(g["times"])
    assert halted_at <= len(g["times"])
    # points arrived window by window: progress reports between them
    progress = [s for s in stats if s.startswith("tran ") and s != "tran 0.0%"]
    assert len(progress) >= 8
    assert len(set(points)) >= 8


GetSyncData = C.CFUNCTYPE(C.c_int, C.c_double, C.POINTER(C.c_double), C.c_double, C.c_int,
                          C.c_int, C.c_int, C.c_void_p)


def _run_with_sync(ng, callback):
    """One `run` of the rc_ladder deck with `callback` as GetSyncData;
    returns the accepted times and the callback's records."""
    calls = []

    def cb(t, pdelta, olddelta, redo, ident, loc, user):
        calls.append((loc, redo, t, pdelta[0], olddelta))
        return callback(loc, redo, t, pdelta, olddelta, len(calls))

    f = GetSyncData(cb)
    _KEEP.append(f)
    ng.ngSpice_Init_Sync.argtypes = [C.c_void_p, C.c_void_p, GetSyncData, C.c_void_p, C.c_void_p]
    assert ng.ngSpice_Init_Sync(None, None, f, None, None) == 0
    try:
        g = golden("rc_ladder")
        lines = [ln.encode() for ln in str(g["netlist"]).splitlines()]
        arr = (C.c_char_p * (len(lines) + 1))(*lines, None)
        assert ng.ngSpice_Circ(arr) == 0
        assert ng.ngSpice_Command(b"run") == 0
        t = ng.ngGet_Vec_Info(b"time").contents
        tt = np.ctypeslib.as_array(t.v_realdata, shape=(t.v_length,)).copy()
    finally:
        assert ng.ngSpice_Init_Sync(None, None, GetSyncData(), None, None) == 0
    return g, tt, calls


def test_sync_callback_sees_every_step(ng):
    """GetSyncData is called where the reference's sharedsync is: before
    every step (loc 0, olddelta 0) and after every step's verdict (loc 1).
    A callback that changes nothing leaves every accepted point of the
    undisturbed run in place up to the final approach, where sharedsync
    keeps delta 1.1 delmin short of the final time: with the breakpoint
    rule that halves a step landing within 1.9 steps of a breakpoint, the
    run then closes in on tstop by halving steps, as the reference does
    with a callback registered."""
    g, tt, calls = _run_with_sync(ng, lambda *a: 0)
    gt = g["times"]
    tstop = gt[-1]
    np.testing.assert_array_equal(tt[:len(gt) - 2], gt[:-2])
    assert abs(tt[-1] - tstop) <= 1e-9 * tstop
    assert np.all(np.diff(tt) > 0)
    assert np.all(tt[len(gt) - 2:] >= gt[-3])
    loc0 = [c for c in calls if c[0] == 0]
    loc1 = [c for c in calls if c[0] == 1]
    assert len(loc0) == len(tt) - 1
    assert all(c[4] == 0.0 and c[1] == 0 for c in loc0)
    accepted = [c[2] for c in loc1 if c[1] == 0]
    np.testing.assert_array_equal(np.array(accepted), tt[1:])
    # each loc-1 call follows the loc-0 call of its step; the step tried is
    # the delta handed out before it
    for a, b in zip(calls, calls[1:]):
        if b[0] == 1 and a[0] == 0:
            assert b[4] == a[3]


def test_sync_callback_limits_the_step(ng):
    """A callback that caps delta at 20 ps before every step: no accepted
    step is longer, and the run still reaches its final time."""
    cap = 20e-12

    def limit(loc, redo, t, pdelta, olddelta, k):
        if loc == 0:
            pdelta[0] = min(pdelta[0], cap)
        return 0

    g, tt, calls = _run_with_sync(ng, limit)
    assert abs(tt[-1] - g["times"][-1]) <= 1e-9 * g["times"][-1]
    assert np.max(np.diff(tt)) <= cap * (1 + 1e-9)
    assert len(tt) > len(g["times"])


def test_sync_callback_redoes_a_step(ng):
    """A callback that returns 1 once after an accepted step, handing back
    that step's own delta: the step is discarded (time moves back by
    olddelta) and tried again, so the same time point is accepted again;
    the points before it are those of the undisturbed run and the run
    reaches its final time."""
    state = {"redone": None}

    def redo_once(loc, redo, t, pdelta, olddelta, k):
        if loc == 1 and redo == 0 and state["redone"] is None and t > 1e-9:
            state["redone"] = t
            pdelta[0] = olddelta
            return 1
        return 0

    g, tt, calls = _run_with_sync(ng, redo_once)
    t0 = state["redone"]
    assert t0 is not None
    assert np.sum(np.isclose(tt, t0, rtol=1e-12, atol=0)) == 1
    assert np.all(np.diff(tt) > 0)
    before = g["times"][g["times"] < t0]
    np.testing.assert_array_equal(tt[:len(before)], before)
    assert abs(tt[-1] - g["times"][-1]) <= 1e-9 * g["times"][-1]
    # the loc-1 record of the repeated step reports the same time again
    again = [c for c in calls if c[0] == 1 and np.isclose(c[2], t0, rtol=1e-12, atol=0)]
    assert len(again) >= 2
