"""GPU: the CUDA transient engine against the reference golden fixtures and
the CPU oracle port, through the C ABI."""
import numpy as np
import pytest

import port
from conftest import golden
from tolerances import matrix_violation, rhs_violation, waveform_violation

pytestmark = pytest.mark.gpu

CASES = ["rc_ladder", "inverter_chain32"]
BSIM4_CASES = ["bsim4_chain8", "bsim4_logic_s3", "v47_chain_mixed", "v47_logic_s3"]
# the rectifier away from the nominal temperature: tlev 1 / tlevc 1 with
# breakdown at 75 C, sidewall junctions at 75 C, tlev 2 at -20 C
DIODE_CASES = ["diode_rectifier", "mos1_mix", "dio_tlev1_75c", "dio_sw_75c", "dio_tlev2_m20c"]


@pytest.fixture(scope="module")
def E(built_lib):
    from ngspice_gb300 import engine
    return engine


def run_one(E, text, capmax=0, **kw):
    c = E.Circuit(text, capmax=capmax, **kw)
    E.run([c], max_steps=1_000_000)
    return c


@pytest.mark.parametrize("name", CASES)
def test_tran_matches_reference(E, name):
    g = golden(name)
    c = run_one(E, str(g["netlist"]))
    r = c.results()
    ref = g["stats"]
    assert r[E.R_STATUS] == 0
    assert r[E.R_ACCEPTED] == ref[3]
    assert r[E.R_REJECTED] == ref[4]
    assert r[E.R_TRANITER] == ref[1]
    t, v = c.points()
    np.testing.assert_array_equal(t, g["times"])
    assert waveform_violation(c.names(), g["times"], g["values"], t, v) < 0.01


@pytest.mark.parametrize("name", CASES)
def test_newton_iterations_stamp_like_reference(E, name):
    """Per-iteration stamped matrix and right-hand side against the reference
    dump, from the first transient iteration on (the operating-point Newton
    path may take a different number of gmin steps when its iterates are
    chaotic, but it converges to the same point)."""
    g = golden(name)
    k = len(g["it_kind"])
    c = run_one(E, str(g["netlist"]), capmax=k + 400)
    cap = c.capture(k + 400)
    cp, ri = c.pattern()
    ref_modes = g["it_meta"][:, 2].astype(int)
    my_modes = cap["meta"][:, 2].astype(int)
    r0 = int(np.argmax(ref_modes & 0x1000))
    m0 = int(np.argmax(my_modes & 0x1000))
    if name == "rc_ladder":
        assert r0 == m0            # linear circuit: identical OP path
    n = c.n
    checked = 0
    for i in range(k - r0):
        kr, km = r0 + i, m0 + i
        if km >= len(cap["ax"]):
            break
        assert g["it_meta"][kr][0] == cap["meta"][km][0]      # same time point
        assert ref_modes[kr] == my_modes[km]                  # same mode
        p0, p1 = g["it_ptr"][kr], g["it_ptr"][kr + 1]
        assert matrix_violation(g["it_rows"][p0:p1], g["it_cols"][p0:p1],
                                g["it_vals"][p0:p1], cp, ri, cap["ax"][km]) <= 1.0
        assert rhs_violation(g["it_rhs"][kr][1:n + 1], cap["rhs"][km][1:n + 1]) <= 1.0
        checked += 1
    assert checked > 20


@pytest.mark.parametrize("name", DIODE_CASES)
def test_diode_decks_match_reference(E, name):
    """Junction diodes and the mixed MOS1 deck (current source, series
    resistances): the reference's Newton and step counts, time points equal
    to rounding, waveforms within the option tolerances."""
    g = golden(name)
    c = run_one(E, str(g["netlist"]))
    r = c.results()
    ref = g["stats"]
    assert r[E.R_STATUS] == 0
    assert (r[E.R_ACCEPTED], r[E.R_REJECTED], r[E.R_TRANITER]) == (ref[3], ref[4], ref[1])
    t, v = c.points()
    assert len(t) == len(g["times"])
    assert np.max(np.abs(t - g["times"])) <= 1e-9 * g["times"][-1]
    assert waveform_violation(c.names(), g["times"], g["values"], t, v) < 1.0


GEAR_CASES = ["gear_mos1_mix", "gear_diode_rectifier", "gear_bsim4_logic_s3",
              "gear6_bsim4_logic_s3"]


@pytest.mark.parametrize("name", GEAR_CASES + ["rings_300"])
def test_gear_and_ring_decks_match_reference(E, name):
    """Gear integration (.options method=gear, maxord 2), and kicked ring
    oscillators in random logic (the C3 generator at a small size): the
    reference's Newton and step counts, time points equal to rounding,
    waveforms within reltol=1e-3, vntol=1 uV, abstol=1 pA."""
    g = golden(name)
    c = run_one(E, str(g["netlist"]))
    r = c.results()
    ref = g["stats"]
    assert r[E.R_STATUS] == 0
    assert (r[E.R_NUMITER], r[E.R_TRANITER], r[E.R_ACCEPTED], r[E.R_REJECTED]) == \
        (ref[0], ref[1], ref[3], ref[4])
    t, v = c.points()
    assert len(t) == len(g["times"])
    assert np.max(np.abs(t - g["times"])) <= 1e-9 * g["times"][-1]
    assert waveform_violation(c.names(), g["times"], g["values"], t, v) < 1.0


def test_gear_batch_equals_single_runs(E):
    """Gear decks in one batched launch give the bits of their single runs."""
    texts = [str(golden(n)["netlist"]) for n in GEAR_CASES]
    singles = [run_one(E, t) for t in texts]
    cs = [E.Circuit(t) for t in texts]
    E.run(cs, max_steps=1_000_000)
    for a, b in zip(singles, cs):
        assert list(a.results()[:7]) == list(b.results()[:7])
        ta, va = a.points()
        tb, vb = b.points()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(va, vb)


@pytest.mark.parametrize("name", BSIM4_CASES)
def test_bsim4_tran_matches_reference(E, name):
    """BSIM4 decks: the same Newton and step counts as the reference; time
    points equal to rounding (the device libm and the host libm differ in
    the last bit of exp/log, which moves the accepted steps by ~1e-12 of
    the run) and waveforms within the tolerance reltol=1e-3, vntol=1 uV,
    abstol=1 pA at every reference time point."""
    g = golden(name)
    c = run_one(E, str(g["netlist"]))
    r = c.results()
    ref = g["stats"]
    assert r[E.R_STATUS] == 0
    assert (r[E.R_ACCEPTED], r[E.R_REJECTED], r[E.R_TRANITER]) == (ref[3], ref[4], ref[1])
    t, v = c.points()
    assert len(t) == len(g["times"])
    assert np.max(np.abs(t - g["times"])) <= 1e-9 * g["times"][-1]
    assert waveform_violation(c.names(), g["times"], g["values"], t, v) < 1.0


@pytest.mark.parametrize("name", BSIM4_CASES)
def test_bsim4_newton_iterations_stamp_like_reference(E, name):
    """Stamped Jacobian / right-hand side of the captured BSIM4 Newton
    iterations from the first transient iteration on, against the
    reference's (row-scaled): within 1e-12 for the first 10 iterations.
    Later iterations inherit the trajectory's drift (the device exp/log and
    the host libm differ in the last bit, so the iterates separate by a
    few ulps per step on the larger deck); they are held to 1e-10 here, and
    the waveforms to the option tolerances in the test above."""
    g = golden(name)
    k = len(g["it_kind"])
    c = run_one(E, str(g["netlist"]), capmax=k + 400)
    cap = c.capture(k + 400)
    cp, ri = c.pattern()
    ref_modes = g["it_meta"][:, 2].astype(int)
    my_modes = cap["meta"][:, 2].astype(int)
    r0 = int(np.argmax(ref_modes & 0x1000))
    m0 = int(np.argmax(my_modes & 0x1000))
    assert ref_modes[r0] & 0x1000 and my_modes[m0] & 0x1000
    n = c.n
    checked = 0
    for i in range(k - r0):
        kr, km = r0 + i, m0 + i
        if km >= len(cap["ax"]):
            break
        assert ref_modes[kr] == my_modes[km]
        p0, p1 = g["it_ptr"][kr], g["it_ptr"][kr + 1]
        bound = 1.0 if i < 10 else 100.0
        assert matrix_violation(g["it_rows"][p0:p1], g["it_cols"][p0:p1],
                                g["it_vals"][p0:p1], cp, ri, cap["ax"][km]) <= bound, kr
        assert rhs_violation(g["it_rhs"][kr][1:n + 1], cap["rhs"][km][1:n + 1]) <= bound, kr
        checked += 1
    assert checked > 20


def test_wide_launch_equals_single_block(E, monkeypatch):
    """The cooperative wide launch (transistor evaluation spread over every
    SM, the rest of the Newton iteration in block 0) computes exactly what
    the one-block launch computes: same counts, bit-identical points."""
    g = golden("bsim4_logic_s3")
    text = str(g["netlist"])
    out = {}
    for wide in ("0", "1"):
        monkeypatch.setenv("NGSF_WIDE", wide)
        c = run_one(E, text)
        r = c.results()
        assert r[E.R_STATUS] == 0
        out[wide] = (list(r[[E.R_ACCEPTED, E.R_REJECTED, E.R_NUMITER, E.R_TRANITER]]),
                     c.points())
    assert out["0"][0] == out["1"][0]
    np.testing.assert_array_equal(out["0"][1][0], out["1"][1][0])
    np.testing.assert_array_equal(out["0"][1][1], out["1"][1][1])


def test_wide_right_looking_equals_single_block(E, monkeypatch):
    """The right-looking refactorization spread over the cooperative grid
    (grid barriers, small phases in block 0) and the grid-wide gather give
    bit-identical points to the same schedule in one block."""
    monkeypatch.setenv("NGSF_LU", "rl")
    g = golden("bsim4_logic_s3")
    text = str(g["netlist"])
    out = {}
    for wide in ("0", "1"):
        monkeypatch.setenv("NGSF_WIDE", wide)
        c = run_one(E, text)
        r = c.results()
        assert r[E.R_STATUS] == 0
        out[wide] = (list(r[[E.R_ACCEPTED, E.R_REJECTED, E.R_NUMITER, E.R_TRANITER]]),
                     c.points())
    assert out["0"][0] == out["1"][0]
    np.testing.assert_array_equal(out["0"][1][0], out["1"][1][0])
    np.testing.assert_array_equal(out["0"][1][1], out["1"][1][1])


def test_right_looking_lu_matches_reference(E, monkeypatch):
    """The right-looking level-scheduled refactorization (the large-matrix
    path) forced on the BSIM4 logic deck: same Newton and step counts as the
    reference and waveforms within the option tolerances."""
    monkeypatch.setenv("NGSF_LU", "rl")
    g = golden("bsim4_logic_s3")
    c = run_one(E, str(g["netlist"]))
    r = c.results()
    ref = g["stats"]
    assert r[E.R_STATUS] == 0
    assert (r[E.R_ACCEPTED], r[E.R_REJECTED], r[E.R_TRANITER]) == (ref[3], ref[4], ref[1])
    t, v = c.points()
    assert waveform_violation(c.names(), g["times"], g["values"], t, v) < 1.0


def test_engine_matches_oracle_port(E):
    """A circuit with no golden fixture: GPU against the CPU oracle port."""
    from ngspice_gb300 import netlists
    text = netlists.inverter_chain(stages=12, tstop="8n", load="35f")
    c = run_one(E, text)
    o = port.simulate(text)
    r = c.results()
    assert r[E.R_ACCEPTED] == o["stats"]["accepted"]
    t, v = c.points()
    np.testing.assert_array_equal(t, o["times"])
    assert waveform_violation(c.names(), o["times"], o["values"], t, v) < 0.01


def test_batch_equals_single_runs(E):
    """Circuits of different size in one launch give bit-identical results
    to the same circuits run alone (each block owns its circuit)."""
    from ngspice_gb300 import netlists
    texts = [netlists.inverter_chain(stages=s, tstop="4n") for s in (4, 9, 16)]
    texts.append(str(golden("rc_ladder")["netlist"]))
    alone = [run_one(E, t) for t in texts]
    batch = [E.Circuit(t) for t in texts]
    E.run(batch, max_steps=1_000_000)
    for a, b in zip(alone, batch):
        ta, va = a.points()
        tb, vb = b.points()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(va, vb)


def test_uneven_monte_carlo_batch_equals_single_runs(E):
    """Monte Carlo instances of uneven size (device mismatch) in one launch,
    largest first: every circuit's result is bit-identical to its run
    alone."""
    from ngspice_gb300 import netlists
    texts = [netlists.random_logic(n_transistors=n, seed=40 + i, tstop="30p", mismatch=True)
             for i, n in enumerate((60, 220, 40, 150, 90))]
    alone = [run_one(E, t) for t in texts]
    batch = [E.Circuit(t) for t in texts]
    E.run(batch, max_steps=1_000_000)
    for a, b in zip(alone, batch):
        ra, rb = a.results(), b.results()
        assert rb[E.R_STATUS] == 0
        assert list(ra[:7]) == list(rb[:7])
        ta, va = a.points()
        tb, vb = b.points()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(va, vb)


def test_step_budget_stops_with_status(E):
    g = golden("inverter_chain32")
    c = E.Circuit(str(g["netlist"]))
    E.run([c], max_steps=50)
    r = c.results()
    assert r[E.R_STATUS] == 121          # step budget exhausted, no hang
    assert 0 < r[E.R_ACCEPTED] <= 51


def test_probe_subset(E):
    g = golden("inverter_chain32")
    c = E.Circuit(str(g["netlist"]), probes=["n32", "n1"])
    E.run([c], max_steps=1_000_000)
    t, v = c.points()
    names = list(g["names"])
    ref = g["values"][:, [names.index("n32"), names.index("n1")]]
    np.testing.assert_array_equal(t, g["times"])
    assert np.max(np.abs(v - ref)) < 1e-9
