"""GPU: the Newton predictor in the transient kernel — the linear guess
keeps the reference tolerances, the network run inside the kernel on its
tensor cores gives exactly the stand-alone network's guess, and a trained
network's effect on Newton iterations (measured against the linear guess
and the plain start on held-out circuits)."""
import numpy as np
import pytest

from conftest import golden
from tolerances import waveform_violation

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E(built_lib):
    from ngspice_gb300 import engine
    return engine


def test_linear_guess_keeps_reference_tolerances(E):
    g = golden("bsim4_logic_s3")
    text = str(g["netlist"])
    plain = E.Circuit(text)
    E.run([plain], max_steps=200000)
    c = E.Circuit(text)
    c.set_predictor(1)
    E.run([c], max_steps=200000)
    r, rp = c.results(), plain.results()
    assert r[E.R_STATUS] == 0
    assert r[E.R_GUESSES] > 0.9 * r[E.R_ACCEPTED]
    assert r[E.R_TRANITER] <= rp[E.R_TRANITER]
    t, v = c.points()
    assert waveform_violation(c.names(), g["times"], g["values"], t, v) < 1.0


def test_in_kernel_network_equals_standalone_forward(E):
    from ngspice_gb300 import gnn, netlists, predictor
    params = predictor.init_params(3)
    text = netlists.random_logic(n_transistors=200, seed=300, tstop="30p")
    host = E.Circuit(text, host_only=True)
    g = host.node_graph()
    names = host.names()
    probes = [names[k] for k in g["vnode"]]
    c = E.Circuit(text, probes=probes, outcap=4096, capmax=3000)
    c.set_predictor(2, params)
    E.run([c], max_steps=200000)
    assert c.results()[E.R_STATUS] == 0
    t, V = c.points()
    cap = c.capture(3000)
    net = gnn.Net(g["gptr"], g["gidx"])
    net.set_params(params)
    checked = 0
    for k in range(len(cap["meta"])):
        tm, dl, mode, _ = cap["meta"][k]
        if not (int(mode) & 0x100000):
            continue
        n = int(np.argmin(np.abs(t - (tm - dl))))
        if abs(t[n] - (tm - dl)) > 1e-20 or n < 2:
            continue
        X, vlin = gnn.features(V[n], V[n - 1], V[n - 2], dl, t[n] - t[n - 1],
                               t[n - 1] - t[n - 2], g["stat"])
        gate = gnn.gate(V[n], V[n - 1], V[n - 2])
        expect = vlin + gnn.VSCALE * gate * net.forward(X).astype(np.float64)
        got = cap["rhsold"][k][g["vnode"] + 1]
        assert np.max(np.abs(got - expect)) <= 1e-6
        checked += 1
    assert checked >= 10


def test_trained_network_against_linear_guess(E):
    """Trains on the GPU on plain trajectories of six circuits and runs two
    held-out circuits three ways.  Every run meets the reference tolerances
    (status 0, same accepted-step count order); the measured iterations per
    step of the three starts are printed and the network must stay within
    10 % of the linear guess."""
    from ngspice_gb300 import netlists, predictor
    train = [netlists.random_logic(n_transistors=200 + 20 * s, seed=500 + s, tstop="120p")
             for s in range(6)]
    data = predictor.collect(train)
    params, losses = predictor.train(data, steps=600)
    assert np.mean(losses[-50:]) < losses[0]
    test = [netlists.random_logic(n_transistors=250, seed=600 + s, tstop="120p") for s in range(2)]
    res = predictor.evaluate(test, params, kinds=(0, 1, 2))
    for k in (0, 1, 2):
        assert res[k]["status"] == [0, 0]
    print("iterations per step: plain %.3f linear %.3f network %.3f" %
          (res[0]["iterations_per_step"], res[1]["iterations_per_step"],
           res[2]["iterations_per_step"]))
    assert res[2]["iterations_per_step"] <= 1.10 * res[1]["iterations_per_step"]
