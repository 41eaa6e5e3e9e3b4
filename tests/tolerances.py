"""Comparison tolerances used by the parity tests.

* Matrix / right-hand side of a Newton iteration: |a-b| <= 1e-12 *
  max(|a|, |b|, rowscale), rowscale = largest |entry| of that matrix row
  (right-hand-side entries use the largest |rhs|): cancellation in terms
  such as cdreq = cdrain - gds*vds - gm*vgs - gmbs*vbs makes a pure
  relative bound meaningless for small entries.
* Waveforms at every reference time point: |a-b| <= reltol*max(|a|,|b|) +
  vntol (node voltages) or abstol (branch currents), with the reference
  options reltol=1e-3, vntol=1e-6, abstol=1e-12.
"""
import numpy as np

RELTOL, VNTOL, ABSTOL = 1e-3, 1e-6, 1e-12


def waveform_violation(names, ref_t, ref_v, t, v):
    """Largest |a-b| / tol over all reference time points (<= 1 passes),
    with the engine waveform interpolated linearly at reference times."""
    worst = 0.0
    for j, nm in enumerate(names):
        vi = np.interp(ref_t, t, v[:, j])
        a, b = vi, ref_v[:, j]
        atol = ABSTOL if nm.endswith("#branch") else VNTOL
        tol = RELTOL * np.maximum(np.abs(a), np.abs(b)) + atol
        worst = max(worst, float(np.max(np.abs(a - b) / tol)))
    return worst


def matrix_violation(ref_rows, ref_cols, ref_vals, cp, ri, ax):
    """Largest |a-b| / (1e-12 * max(|a|,|b|,rowscale)) over the entries."""
    ref = {(int(r), int(c)): v for r, c, v in zip(ref_rows, ref_cols, ref_vals)}
    n = len(cp) - 1
    rowscale = {}
    for (r, c), v in ref.items():
        rowscale[r] = max(rowscale.get(r, 0.0), abs(v))
    worst = 0.0
    for j in range(n):
        for p in range(cp[j], cp[j + 1]):
            a = ax[p]
            b = ref[(int(ri[p]), j)]
            scale = max(abs(a), abs(b), rowscale.get(int(ri[p]), 0.0), 1e-300)
            worst = max(worst, abs(a - b) / (1e-12 * scale))
    return worst


def rhs_violation(ref_rhs, rhs):
    scale = max(float(np.max(np.abs(ref_rhs))), 1e-300)
    return float(np.max(np.abs(ref_rhs - rhs))) / (1e-12 * scale)


def matrix_violation_dense(ref_rows, ref_cols, ref_vals, a):
    """matrix_violation for a dense (n+1)x(n+1) matrix whose row/column 0 is
    ground; the reference entries carry 0-based equation indices."""
    ref = np.zeros_like(a)
    ref[np.asarray(ref_rows) + 1, np.asarray(ref_cols) + 1] = ref_vals
    m, r = a[1:, 1:], ref[1:, 1:]
    rowscale = np.max(np.abs(r), axis=1, keepdims=True)
    scale = np.maximum(np.maximum(np.abs(m), np.abs(r)), np.maximum(rowscale, 1e-300))
    return float(np.max(np.abs(m - r) / (1e-12 * scale)))


def rhs_violation_rowscaled(ref_rows, ref_vals, ref_rhs, rhs, rhs_old):
    """Largest |a-b| / (1e-12 * scale_i) over the right-hand-side entries
    1..n, scale_i = max(|a_i|, |b_i|, rowscale_i * max|rhsOld|): a device's
    right-hand-side term is a current such as cdreq = cd - gds*vds - gm*vgs,
    a sum of conductance x voltage products, so the row's largest
    conductance times the largest voltage bounds the terms that cancel.
    ref_rows are the 0-based equation indices of the reference's matrix
    entries; ref_rhs / rhs / rhs_old hold equations 1..n."""
    n = len(ref_rhs)
    rowscale = np.zeros(n)
    np.maximum.at(rowscale, np.asarray(ref_rows), np.abs(np.asarray(ref_vals)))
    vmax = max(float(np.max(np.abs(rhs_old))), 1e-300)
    scale = np.maximum(np.maximum(np.abs(ref_rhs), np.abs(rhs)), rowscale * vmax)
    scale = np.maximum(scale, 1e-300)
    return float(np.max(np.abs(ref_rhs - rhs) / (1e-12 * scale)))

