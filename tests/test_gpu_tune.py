"""GPU: the autotuner of the wide refactorization (engine.tune_factor_shape)
picks one of its candidate shapes, and every shape computes the same
result: the run after tuning is bit-identical to the run with the default
shape."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E(built_lib):
    from ngspice_gb300 import engine
    return engine


def test_tuned_shape_gives_identical_results(E):
    from ngspice_gb300 import netlists
    text = netlists.random_logic(n_transistors=1100, seed=2, tstop="14p")
    ref = E.Circuit(text, probes=["y0", "y1"], outcap=4096)
    assert ref.wide_info()[0]
    E.run([ref], max_steps=1_000_000)

    c = E.Circuit(text, probes=["y0", "y1"], outcap=4096)
    choice = E.tune_factor_shape(c, blocks=(16, 48), small_works=(256,), warm=3e-12,
                                 window=2e-12, repeats=1)
    assert choice["blocks"] in (16, 48)
    assert choice["small_work"] in (0, 256)
    assert len(choice["timings"]) == 3
    E.run([c], max_steps=1_000_000)
    ra, rb = ref.results(), c.results()
    assert rb[E.R_STATUS] == 0
    assert list(ra[:7]) == list(rb[:7])
    ta, va = ref.points()
    tb, vb = c.points()
    np.testing.assert_array_equal(ta, tb)
    np.testing.assert_array_equal(va, vb)

    # an explicit shape far from the default: still the same result
    c.set_factor_shape(8, 65536)
    E.run([c], max_steps=1_000_000)
    tc, vc = c.points()
    np.testing.assert_array_equal(ta, tc)
    np.testing.assert_array_equal(va, vc)
