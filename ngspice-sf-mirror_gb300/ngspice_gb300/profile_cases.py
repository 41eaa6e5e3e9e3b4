"""Small, self-contained cases for profiling the kernels under ncu.

    python -m ngspice_gb300.profile_cases c1 3p     # the 10k-transistor BSIM4
                                                     # circuit, first 3 ps
    python -m ngspice_gb300.profile_cases gnn 8192  # three training steps of
                                                     # the predictor network

Each case runs once and exits 0 on success (so it can run plainly before
the same command runs under ncu).  Run from the repository root with the
package directory on PYTHONPATH.
"""
from __future__ import annotations

import sys

import numpy as np


def c1(tstop: str = "3p") -> None:
    from . import engine as E, netlists
    text = netlists.random_logic(n_transistors=10000, seed=1, tstop=tstop)
    c = E.Circuit(text, probes=["y0"], outcap=256)
    sec = E.run([c])
    r = c.results()
    print("status", r[E.R_STATUS], "iters", r[E.R_NUMITER], "accepted", r[E.R_ACCEPTED],
          "device_s", round(sec, 3), "launches", E.last_launches())
    if r[E.R_STATUS] != 0:
        raise SystemExit(1)


def gnn(n: int = 8192) -> None:
    from . import gnn as G, predictor
    rng = np.random.default_rng(0)
    nbs = [set() for _ in range(n)]
    for i in range(n):
        for j in rng.integers(max(0, i - 50), min(n, i + 50), 6):
            if int(j) != i:
                nbs[i].add(int(j))
                nbs[int(j)].add(i)
    ptr, idx = [0], []
    for i in range(n):
        idx += sorted(nbs[i])
        ptr.append(len(idx))
    net = G.Net(np.array(ptr, np.int32), np.array(idx, np.int32))
    net.set_params(predictor.init_params(0))
    X = rng.standard_normal((n, G.F_IN)).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    w = np.ones(n, np.float32)
    for _ in range(3):
        loss, _ = net.train_step(X, y, w, 1e-3)
    print("loss", loss)


if __name__ == "__main__":
    case = sys.argv[1] if len(sys.argv) > 1 else "c1"
    arg = sys.argv[2] if len(sys.argv) > 2 else None
    if case == "c1":
        c1(arg or "3p")
    elif case == "gnn":
        gnn(int(arg or 8192))
    else:
        raise SystemExit(f"unknown case {case}")
