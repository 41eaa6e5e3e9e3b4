"""GPU: batch paths of the engine.

* Holding circuits after their first accepted transient step while other
  circuits of the batch still pause for new pivots (NGSF_HOLD=1): a held
  circuit resumes exactly where it stopped, so every result is
  bit-identical to the run without holding.
* ngsf_open_many (parsing and setup on all host cores): the same circuits,
  and the same results, as one ngsf_open per netlist.
* One Monte Carlo instance (per-device mismatch model cards) against the
  reference: the same counts, time points to rounding, waveforms within
  tolerance."""
import numpy as np
import pytest

from conftest import golden
from tolerances import waveform_violation

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E(built_lib):
    from ngspice_gb300 import engine
    return engine


def _batch(E, texts):
    cs = [E.Circuit(t) for t in texts]
    E.run(cs, max_steps=1_000_000)
    return cs, E.last_launches()


def test_held_batch_equals_plain_batch(E, monkeypatch):
    from ngspice_gb300 import netlists
    texts = [netlists.random_logic(n_transistors=n, seed=70 + i, tstop="30p", mismatch=True)
             for i, n in enumerate((180, 40, 260, 90, 130, 60))]
    monkeypatch.setenv("NGSF_HOLD", "0")
    plain, _ = _batch(E, texts)
    monkeypatch.setenv("NGSF_HOLD", "1")
    held, _ = _batch(E, texts)
    for a, b in zip(plain, held):
        ra, rb = a.results(), b.results()
        assert rb[E.R_STATUS] == 0
        assert list(ra[:7]) == list(rb[:7])
        assert ra[E.R_REORDERS] == rb[E.R_REORDERS]
        ta, va = a.points()
        tb, vb = b.points()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(va, vb)


def test_open_many_equals_single_opens(E):
    from ngspice_gb300 import netlists
    texts = [netlists.random_logic(n_transistors=n, seed=90 + i, tstop="20p", mismatch=True)
             for i, n in enumerate((120, 50, 200, 80))]
    single = [E.Circuit(t, probes=["y0"], outcap=4096) for t in texts]
    many = E.open_many(texts, probes=["y0"], outcap=4096)
    assert [(c.n, c.nnz, c.nstates) for c in single] == [(c.n, c.nnz, c.nstates) for c in many]
    E.run(single, max_steps=1_000_000)
    E.run(many, max_steps=1_000_000)
    for a, b in zip(single, many):
        assert b.results()[E.R_STATUS] == 0
        assert list(a.results()[:7]) == list(b.results()[:7])
        ta, va = a.points()
        tb, vb = b.points()
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(va, vb)



def test_monte_carlo_instance_matches_reference(E):
    g = golden("bsim4_mc_s5")
    c = E.Circuit(str(g["netlist"]))
    E.run([c], max_steps=1_000_000)
    r = c.results()
    ref = g["stats"]
    assert r[E.R_STATUS] == 0
    assert (r[E.R_ACCEPTED], r[E.R_REJECTED], r[E.R_TRANITER]) == (ref[3], ref[4], ref[1])
    t, v = c.points()
    assert len(t) == len(g["times"])
    assert np.max(np.abs(t - g["times"])) <= 1e-9 * g["times"][-1]
    assert waveform_violation(c.names(), g["times"], g["values"], t, v) < 1.0
