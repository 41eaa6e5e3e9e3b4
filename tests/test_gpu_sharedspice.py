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
