"""GPU: batched launches that hold circuits after their first accepted
transient step while other circuits of the batch still pause for new pivots
(NGSF_HOLD=1).  A held circuit resumes exactly where it stopped, so every
result is bit-identical to the run without holding."""
import numpy as np
import pytest

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
