"""GPU: one CKTload at the reference's own linearisation points.

The reference oracle records, for selected Newton iterations, the point
its CKTload started from -- rhsOld, CKTstates[0..2] before the load, the
integration coefficients, gmin, srcFact and every BSIM4 instance's
BSIM4von (tests/golden/make_golden.py, driver --states).  Loading the
engine's circuit at exactly that point (ngsf_ckt_load) isolates the device
evaluation and the stamp gather from trajectory drift: the stamped matrix
and right-hand side must agree with the reference's dump of the same
iteration within the row-scaled 1e-12 bound at every recorded iteration,
operating point and transient alike."""
import numpy as np
import pytest

from conftest import golden
from tolerances import matrix_violation, rhs_violation_rowscaled

pytestmark = pytest.mark.gpu

CASES = ["bsim4_chain8", "bsim4_logic_s3", "bsim4_mc_s5", "v47_chain_mixed", "v47_logic_s3"]


@pytest.fixture(scope="module")
def E(built_lib):
    from ngspice_gb300 import engine
    return engine


@pytest.mark.parametrize("name", CASES)
def test_load_at_reference_points(E, name):
    g = golden(name)
    c = E.Circuit(str(g["netlist"]))
    cp, ri = c.pattern()
    n = c.n
    assert g["st_states"].shape[2] == c.nstates
    worst_m = worst_r = 0.0
    for j, k in enumerate(g["st_iter"]):
        t, delta, mode, order, _ = g["it_meta"][k]
        ag0, ag1, do0, do1, gmin, src = g["st_scal"][j]
        pt = E.make_point(time=t, delta=delta, deltaOld=(do0, do1, 0.0), ag=(ag0, ag1),
                          gmin=gmin, srcFact=src, mode=int(mode), order=int(order))
        ax, rhs, _ = c.ckt_load(pt, rhs_old=g["it_rhsold"][k], states=g["st_states"][j],
                                von=g["st_von"][j])
        p0, p1 = g["it_ptr"][k], g["it_ptr"][k + 1]
        vm = matrix_violation(g["it_rows"][p0:p1], g["it_cols"][p0:p1], g["it_vals"][p0:p1],
                              cp, ri, ax)
        vr = rhs_violation_rowscaled(g["it_rows"][p0:p1], g["it_vals"][p0:p1],
                                     g["it_rhs"][k][1:n + 1], rhs[1:n + 1],
                                     g["it_rhsold"][k][1:n + 1])
        worst_m, worst_r = max(worst_m, vm), max(worst_r, vr)
        assert vm <= 1.0, (k, vm)
        assert vr <= 1.0, (k, vr)
    print(f"{name}: {len(g['st_iter'])} iterations, worst matrix {worst_m:.3f},"
          f" rhs {worst_r:.3f} of the 1e-12 bound")
    assert len(g["st_iter"]) >= 30


def test_device_table_and_type_masks(E):
    """DEVload per device type: the loads of disjoint type sets add up to
    the whole CKTload, entry by entry (the gather sums each cell in the
    reference's order, so the split can differ only by rounding)."""
    table = E.dev_table()
    assert [t["name"] for t in table] == ["BSIM4", "Capacitor", "Diode", "Isource", "Mos1",
                                         "Resistor", "Vsource"]
    g = golden("bsim4_chain8")
    c = E.Circuit(str(g["netlist"]))
    j = len(g["st_iter"]) // 2
    k = g["st_iter"][j]
    t, delta, mode, order, _ = g["it_meta"][k]
    ag0, ag1, do0, do1, gmin, src = g["st_scal"][j]
    pt = E.make_point(time=t, delta=delta, deltaOld=(do0, do1, 0.0), ag=(ag0, ag1), gmin=gmin,
                      srcFact=src, mode=int(mode), order=int(order))
    args = dict(rhs_old=g["it_rhsold"][k], states=g["st_states"][j], von=g["st_von"][j])
    ax_all, rhs_all, _ = c.ckt_load(pt, E.DEV_ALL, **args)
    ax_b, rhs_b, _ = c.ckt_load(pt, 1 << E.DEV_BSIM4, **args)
    ax_r, rhs_r, _ = c.ckt_load(pt, E.DEV_ALL & ~(1 << E.DEV_BSIM4), **args)
    scale = np.max(np.abs(ax_all))
    assert np.max(np.abs(ax_b + ax_r - ax_all)) <= 1e-12 * scale
    assert np.max(np.abs(rhs_b + rhs_r - rhs_all)) <= 1e-12 * np.max(np.abs(rhs_all))
    assert np.any(ax_b != 0) and np.any(ax_r != 0)


def test_smp_reorder_lufac_solve(E):
    """SMPreorder / SMPluFac / SMPsolve on the device matrix against a dense
    solve of the same system: the stamped matrix of a reference iteration,
    then the same pattern with every value scaled (refactor on the kept
    pivots)."""
    g = golden("bsim4_logic_s3")
    c = E.Circuit(str(g["netlist"]))
    cp, ri = c.pattern()
    n = c.n
    k = int(g["st_iter"][len(g["st_iter"]) // 2])
    p0, p1 = g["it_ptr"][k], g["it_ptr"][k + 1]
    ref = {(int(r), int(cc)): v for r, cc, v in zip(g["it_rows"][p0:p1], g["it_cols"][p0:p1],
                                                    g["it_vals"][p0:p1])}
    ax = np.array([ref[(int(ri[p]), j)] for j in range(n) for p in range(cp[j], cp[j + 1])])
    b = g["it_rhs"][k][:n + 1].copy()

    def dense(vals):
        A = np.zeros((n, n))
        for j in range(n):
            for p in range(cp[j], cp[j + 1]):
                A[ri[p], j] += vals[p]
        return A

    c.smp_set_matrix(ax)
    assert c.smp_reorder(pivtol=1e-13, pivrel=1e-3) == 0
    x = c.smp_solve(b)
    xd = np.linalg.solve(dense(ax), b[1:])
    assert np.max(np.abs(x[1:] - xd)) <= 1e-9 * np.max(np.abs(xd))
    rng = np.random.default_rng(7)
    ax2 = ax * rng.uniform(0.9, 1.1, size=ax.shape)
    c.smp_set_matrix(ax2)
    assert c.smp_lufac() == 0
    x2 = c.smp_solve(b)
    xd2 = np.linalg.solve(dense(ax2), b[1:])
    assert np.max(np.abs(x2[1:] - xd2)) <= 1e-9 * np.max(np.abs(xd2))
    np.testing.assert_array_equal(c.smp_get_matrix(), ax2)
    # a zero column cannot be refactored on the kept pivots
    ax3 = ax2.copy()
    ax3[cp[0]:cp[1]] = 0.0
    c.smp_set_matrix(ax3)
    assert c.smp_lufac() == E.E_SINGULAR


def test_convtest_and_trunc(E):
    """NIconvTest on two vectors and CKTtrunc on recorded states."""
    g = golden("bsim4_chain8")
    c = E.Circuit(str(g["netlist"]))
    n = c.n
    x = g["it_rhsold"][-1]
    assert c.ni_convtest(x, x) == 0
    y = x.copy()
    y[1] += 1e-2 * max(1.0, abs(x[1]))
    assert c.ni_convtest(y, x) == 1
    # a transient iteration: the truncation-error step is positive and at
    # most twice the current step
    j = [i for i, k in enumerate(g["st_iter"]) if int(g["it_meta"][k][2]) & 0x1][-1]
    k = g["st_iter"][j]
    t, delta, mode, order, _ = g["it_meta"][k]
    ag0, ag1, do0, do1, gmin, src = g["st_scal"][j]
    pt = E.make_point(time=t, delta=delta, deltaOld=(do0, do1, do1), ag=(ag0, ag1), gmin=gmin,
                      srcFact=src, mode=int(mode), order=1)
    st = np.concatenate([g["st_states"][j], g["st_states"][j][-1:]], axis=0)
    dt = c.ckt_trunc(pt, st)
    assert 0 < dt <= 2 * delta
    assert n > 0
