"""CPU: the oracle port against reference fixtures at benchmark scale.

The fixtures (tests/golden/make_golden.py, LARGE_CASES) come from the
reference ngspice compiled from its own sources: the 10,000-transistor
random-logic netlist over its first 30 ps, Monte Carlo instances of
about 1,000, 2,000 and 3,000 transistors (device mismatch) over 50 ps, and
instance 1314 of the 4096-instance workload (4,714 transistors) over
150 ps.
They hold the reference's statistics, accepted time points and the
waveforms of 256 unknowns spread over the equation numbering.  The port
must reproduce the Newton and step counts and stay within the option
tolerances at every reference time point; this anchors the port (and
through it the CPU baseline) to the reference at the sizes the
benchmarks run."""
import numpy as np
import pytest

import port
from conftest import golden
from tolerances import waveform_violation

CASES = ["mc_1k_50p", "mc_2k_50p", "mc_3k_50p", "c1_10k_30p", "mc_c4_1314"]


@pytest.mark.parametrize("name", CASES)
def test_port_matches_reference_at_scale(name):
    g = golden(name)
    r = port.simulate(str(g["netlist"]))
    st, ref = r["stats"], g["stats"]
    assert len(r["names"]) == int(g["nvars"])
    assert [r["names"][i] for i in g["cols"]] == list(g["names"])
    assert (st["numIter"], st["tranIter"], st["accepted"], st["rejected"]) == \
        (ref[0], ref[1], ref[3], ref[4])
    assert np.max(np.abs(r["times"] - g["times"])) <= 1e-9 * g["times"][-1]
    v = waveform_violation(list(g["names"]), g["times"], g["values"], r["times"],
                           r["values"][:, g["cols"]])
    print(f"{name}: worst waveform error {v:.2e} of the tolerance")
    assert v < 1.0
