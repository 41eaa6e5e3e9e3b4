"""CPU: the oracle port against the reference's golden fixtures.

The fixtures come from the reference ngspice compiled from its own sources
(tests/golden/make_golden.py).  The port must reproduce the accepted time
points exactly, the Newton iteration counts of the transient, and the
waveforms within the option tolerances.
"""
import numpy as np
import pytest

import port
from conftest import golden
from tolerances import waveform_violation

CASES = ["rc_ladder", "inverter_chain32"]


@pytest.mark.parametrize("name", CASES)
def test_port_matches_reference(name):
    g = golden(name)
    r = port.simulate(str(g["netlist"]))
    st = r["stats"]
    ref = g["stats"]
    assert r["names"] == list(g["names"])
    assert st["status"] == 0
    assert st["accepted"] == ref[3]
    assert st["rejected"] == ref[4]
    assert st["tranIter"] == ref[1]
    np.testing.assert_array_equal(r["times"], g["times"])
    # identical time points; values agree to rounding (1% of the tolerance)
    assert waveform_violation(r["names"], g["times"], g["values"], r["times"], r["values"]) < 0.01


def test_planted_mistake_is_caught():
    """A wrong MOS1 transconductance in the oracle must be detected by the
    same comparison the tests use."""
    g = golden("inverter_chain32")
    text = str(g["netlist"]).replace("kp=110u", "kp=111u")
    r = port.simulate(text)
    same_points = len(r["times"]) == len(g["times"]) and np.array_equal(r["times"], g["times"])
    if same_points:
        assert waveform_violation(r["names"], g["times"], g["values"], r["times"], r["values"]) > 1
    else:
        assert True


def test_number_evaluation_matches_reference_rules():
    ev = port.evaluate
    assert ev("2u") == 2 * 10.0 ** -6
    assert ev("0.7") == 7 * 10.0 ** -1
    assert ev("1meg") == 1.0 * 10.0 ** 6
    assert ev("3mil") == 3 * 25.4 * 10.0 ** -6
    assert ev("-1.5e-3k") == -15 * 10.0 ** (-1 - 3 + 3)
    assert ev("abc") is None
