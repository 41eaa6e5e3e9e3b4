"""GPU: ngsf_stamp_initial_static, the entry point that allocates nothing,
against the existing path (ngsf_open + ngsf_run + ngsf_capture): the first
Newton iteration's stamped matrix and right-hand side must agree, on two
calls in a row.  The file name sorts last so that the test also runs after
every other GPU test in the same process; it passes alone as well."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from tolerances import rhs_violation

pytestmark = pytest.mark.gpu

CASES = ["rc_ladder", "inverter_chain32", "bsim4_chain8"]


@pytest.fixture(scope="module")
def E(built_lib):
    from ngspice_gb300 import engine
    L = engine.lib()
    L.ngsf_stamp_initial_static.restype = C.c_int
    L.ngsf_stamp_initial_static.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
    return engine


def static_stamps(E, c):
    ax = np.full(len(c.pattern()[1]), np.nan)
    rhs = np.full(c.n + 1, np.nan)
    rc = E.lib().ngsf_stamp_initial_static(
        c._h, ax.ctypes.data_as(C.POINTER(C.c_double)), rhs.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0, E.last_error()
    return ax, rhs


@pytest.mark.parametrize("name", CASES)
def test_static_stamps_equal_first_captured_iteration(E, name):
    text = str(golden(name)["netlist"])
    ref = E.Circuit(text, capmax=4)
    E.run([ref], max_steps=1_000_000)
    cap = ref.capture(4)
    assert int(cap["meta"][0][2]) & 0x200            # MODEINITJCT
    ax_ref, rhs_ref = cap["ax"][0], cap["rhs"][0]

    c = E.Circuit(text)                              # a second, untouched circuit
    for _ in range(2):                               # two calls in a row
        ax, rhs = static_stamps(E, c)
        scale = np.maximum(np.abs(ax_ref), 1e-300)
        assert np.max(np.abs(ax - ax_ref) / scale) <= 1e-12
        assert rhs_violation(rhs_ref[1:], rhs[1:]) <= 1.0


def test_static_stamps_refuse_circuits_beyond_the_static_size(E):
    from ngspice_gb300 import netlists
    c = E.Circuit(netlists.random_logic(n_transistors=10000, seed=1, tstop="2p"))
    ax = np.zeros(len(c.pattern()[1]))
    rhs = np.zeros(c.n + 1)
    rc = E.lib().ngsf_stamp_initial_static(
        c._h, ax.ctypes.data_as(C.POINTER(C.c_double)), rhs.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc != 0
    assert "bytes of scratch" in E.last_error()
