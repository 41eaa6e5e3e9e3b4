"""GPU: windowed runs and block sizes.

* ngsf_run_window stops every circuit at the first accepted point at or
  after the window's end and continues from the saved device state in the
  next window; a run cut into windows is bit-identical to the uncut run
  (accepted points, waveforms, Newton and step counts), for a batch and
  for one circuit alone (run over the whole grid).
* The batched launch gives the same bits with 64-, 128- and 256-thread
  circuit blocks: every loop is strided by the block size and every sum
  keeps its order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E(built_lib):
    from ngspice_gb300 import engine
    return engine


def texts():
    from ngspice_gb300 import netlists
    return [netlists.random_logic(n_transistors=n, seed=300 + i, tstop="60p", mismatch=True)
            for i, n in enumerate((220, 60, 340, 120, 150))]


def same(E, a, b):
    ra, rb = a.results(), b.results()
    assert rb[E.R_STATUS] == 0
    assert list(ra[:7]) == list(rb[:7])
    ta, va = a.points()
    tb, vb = b.points()
    np.testing.assert_array_equal(ta, tb)
    np.testing.assert_array_equal(va, vb)


@pytest.mark.parametrize("hold", ["0", "1"])
def test_windows_equal_one_run(E, monkeypatch, hold):
    monkeypatch.setenv("NGSF_HOLD", hold)
    ts = texts()
    whole = [E.Circuit(t) for t in ts]
    E.run(whole, max_steps=1_000_000)
    cut = [E.Circuit(t) for t in ts]
    ends = [5e-12, 17e-12, 30e-12, 44e-12, 1.0]
    for k, t_end in enumerate(ends):
        E.run_window(cut, t_end, max_steps=1_000_000)
        for c in cut:
            r = c.results()
            if k < len(ends) - 1:
                assert r[E.R_STATUS] in (0, E.PAUSED)
                t, _ = c.points()
                if r[E.R_STATUS] == E.PAUSED:
                    assert t[-1] >= t_end and (len(t) < 2 or t[-2] < t_end)
    for a, b in zip(whole, cut):
        same(E, a, b)


def test_window_single_wide_circuit(E):
    from ngspice_gb300 import netlists
    text = netlists.random_logic(n_transistors=1500, seed=11, tstop="12p")
    whole = E.Circuit(text)
    E.run([whole], max_steps=1_000_000)
    cut = E.Circuit(text)
    for t_end in (3e-12, 7e-12, 1.0):
        E.run_window([cut], t_end, max_steps=1_000_000)
    same(E, whole, cut)


def test_batch_block_sizes_give_the_same_bits(E, monkeypatch):
    ts = texts()
    runs = []
    for threads in ("256", "128", "64"):
        monkeypatch.setenv("NGSF_BATCH_THREADS", threads)
        cs = [E.Circuit(t) for t in ts]
        E.run(cs, max_steps=1_000_000)
        runs.append(cs)
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            same(E, a, b)


@pytest.mark.parametrize("wide", ["0", "1"])
def test_passive_sync_stops_equal_one_run(E, monkeypatch, wide):
    """A synchronised run (stops at both sharedsync points of every step)
    answered with the engine's own delta and no redo is bit-identical to the
    plain run, in one block and over the whole grid; every stop reports a
    step time inside the transient and a positive delta."""
    from ngspice_gb300 import netlists
    monkeypatch.setenv("NGSF_WIDE", wide)
    text = netlists.random_logic(n_transistors=1100 if wide == "1" else 200, seed=321,
                                 tstop="12p", mismatch=True)
    plain = E.Circuit(text)
    E.run([plain], max_steps=1_000_000)
    c = E.Circuit(text)
    c.set_sync(True)
    stops = {0: 0, 1: 0}
    for _ in range(20000):
        E.run_window([c], 1.0, max_steps=1_000_000)
        sp = c.sync_point()
        if sp is None:
            break
        assert 0.0 <= sp["time"] <= 12e-12 and sp["delta"] > 0
        stops[sp["loc"]] += 1
        c.sync_reply(sp["delta"], 0)
    assert c.results()[E.R_STATUS] == 0
    same(E, plain, c)
    acc = int(plain.results()[E.R_ACCEPTED])
    assert stops[0] == acc - 1
    assert stops[1] >= acc - 1
