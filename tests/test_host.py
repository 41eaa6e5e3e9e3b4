"""CPU: the product library loads, exports its C ABI, and its host compiler
numbers equations and lays out the matrix exactly as the reference does."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden


def declared_symbols():
    names = set()
    for h in ("sharedspice.h", "ngspice_gb300.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"\b(ng[A-Za-z0-9_]+)\s*\(", text))
    return {n for n in names if not n.startswith("ngcomplex")}


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, missing
    from ngspice_gb300 import engine
    assert set(engine.EXPORTS) <= declared_symbols()


@pytest.mark.parametrize("name", ["rc_ladder", "inverter_chain32"])
def test_equation_names_and_pattern_match_reference(built_lib, name):
    from ngspice_gb300 import engine as E
    g = golden(name)
    c = E.Circuit(str(g["netlist"]), host_only=True)
    assert c.names() == list(g["names"])
    cp, ri = c.pattern()
    mine = {(int(ri[p]), j) for j in range(c.n) for p in range(cp[j], cp[j + 1])}
    p0, p1 = g["it_ptr"][0], g["it_ptr"][1]
    ref = set(zip(g["it_rows"][p0:p1].tolist(), g["it_cols"][p0:p1].tolist()))
    assert mine == ref


def test_unsupported_input_is_reported(built_lib):
    from ngspice_gb300 import engine as E
    with pytest.raises(E.EngineError, match="unsupported element"):
        E.Circuit("t\nq1 c b e qmod\n.tran 1n 10n\n.end\n", host_only=True)
    with pytest.raises(E.EngineError, match="no .tran"):
        E.Circuit("t\nr1 a 0 1k\nv1 a 0 1\n.end\n", host_only=True)
    with pytest.raises(E.EngineError, match="shorted VSRC"):
        E.Circuit("t\nv1 a a 1\nr1 a 0 1\n.tran 1n 2n\n.end\n", host_only=True)


def test_bsim4_version_selection(built_lib):
    """Version 4.7 cards select the BSIM4v7 restatement, which numbers and
    lays out the mixed 4.7/4.8 chain as the reference does; its parser
    ignores the 4.8-only model parameters and rejects the 4.8-only instance
    multipliers (bsim4v7/b4v7.c).  Versions before 4.7 select devices the
    GPU load does not have."""
    from ngspice_gb300 import engine as E
    g = golden("v47_chain_mixed")
    c = E.Circuit(str(g["netlist"]), host_only=True)
    assert c.names() == list(g["names"])
    cp, ri = c.pattern()
    mine = {(int(ri[p]), j) for j in range(c.n) for p in range(cp[j], cp[j + 1])}
    p0, p1 = g["it_ptr"][0], g["it_ptr"][1]
    assert mine == set(zip(g["it_rows"][p0:p1].tolist(), g["it_cols"][p0:p1].tolist()))
    deck = ("t\n.model nm nmos level=54 version={v} vth0=0.42 toxe=1.75e-9 {mod}\n"
            "m1 d g 0 0 nm w=200n l=45n {inst}\nvd d 0 1\nvg g 0 1\n.tran 1p 10p\n.end\n")
    E.Circuit(deck.format(v="4.7.0", mod="gidlclamp=-1e-5 idovvdsc=1e-9 ketac=0.1 lketac=0"
                          " rgeomod=0", inst="m=2"), host_only=True)
    E.Circuit(deck.format(v="4.8.3", mod="ketac=0.1", inst="mult_i=2 mult_q=0.5"),
              host_only=True)
    with pytest.raises(E.EngineError, match=r"unknown parameter \(mult_i\)"):
        E.Circuit(deck.format(v="4.7.0", mod="", inst="mult_i=2"), host_only=True)
    with pytest.raises(E.EngineError, match="rgeomod=1"):
        E.Circuit(deck.format(v="4.7", mod="rgeomod=1", inst=""), host_only=True)
    with pytest.raises(E.EngineError, match="versions 4.7.x and 4.8.x"):
        E.Circuit(deck.format(v="4.6.5", mod="", inst=""), host_only=True)


def test_diode_temperature_selectors(built_lib):
    """Diode tlev 0-2 and tlevc 0-1 compile (diotemp.c); other selector
    values are refused with a message."""
    from ngspice_gb300 import engine as E
    deck = ("t\n.model dd d is=1e-14 {sel}\nd1 a 0 dd\nr1 a b 1k\nv1 b 0 1\n"
            ".tran 1n 10n\n.options temp=60\n.end\n")
    for sel in ("tlev=1 tlevc=1 cta=1e-3 ctc=1e-3 tpb=1e-3 tvj=1e-3 ctp=1e-3 tphp=1e-3",
                "tlev=2 gap1=7e-4 gap2=1100 eg=1.1"):
        E.Circuit(deck.format(sel=sel), host_only=True)
    with pytest.raises(E.EngineError, match="tlev 3"):
        E.Circuit(deck.format(sel="tlev=3"), host_only=True)
    with pytest.raises(E.EngineError, match="tlevc 2"):
        E.Circuit(deck.format(sel="tlevc=2"), host_only=True)


def test_run_refuses_host_only_circuit(built_lib):
    from ngspice_gb300 import engine as E
    g = golden("rc_ladder")
    c = E.Circuit(str(g["netlist"]), host_only=True)
    with pytest.raises(E.EngineError, match="without a device"):
        E.run([c])


def test_open_many_reports_the_failing_netlist(built_lib):
    """ngsf_open_many parses every netlist on the host cores before any
    device work, so a bad netlist fails the whole batch on the CPU, naming
    its index; an empty batch is empty."""
    from ngspice_gb300 import engine as E, netlists
    good = netlists.random_logic(n_transistors=40, seed=3, tstop="5p")
    with pytest.raises(E.EngineError, match="netlist 1: short card"):
        E.open_many([good, "* broken\nR1 a\n.tran 1p 2p\n.end\n", good])
    with pytest.raises(E.EngineError, match="netlist 0: unsupported element"):
        E.open_many(["t\nq1 c b e qmod\n.tran 1n 10n\n.end\n"])
    assert E.open_many([]) == []


def test_factor_shape_needs_a_device_circuit(built_lib):
    from ngspice_gb300 import engine as E
    c = E.Circuit(str(golden("rc_ladder")["netlist"]), host_only=True)
    with pytest.raises(E.EngineError, match="host-only"):
        c.set_factor_shape(32, 1024)
    with pytest.raises(E.EngineError, match="host-only"):
        c.wide_info()


@pytest.mark.parametrize("name,blocks", [("mc_1k_50p", 135), ("mc_2k_50p", 133),
                                         ("mc_3k_50p", 137), ("c1_10k_30p", 138)])
def test_block_triangular_analysis_matches_klu(built_lib, name, blocks):
    """SMPpreOrder's analysis (ngsf_smp_preorder): the block upper
    triangular form of the circuit pattern has as many diagonal blocks as
    the reference's klu_analyze reports on the same netlist (driver with
    ORACLE_KLU_STATS=1 on the compiled reference); the voltage sources give
    the singleton blocks, the rest of the circuit one large block."""
    from ngspice_gb300 import engine as E
    g = golden(name)
    c = E.Circuit(str(g["netlist"]), host_only=True)
    nb, big = c.smp_preorder()
    assert nb == blocks
    assert big > c.n // 2


def test_block_triangular_analysis_of_small_decks(built_lib):
    """The analysis on decks whose zero-free diagonal needs augmenting
    paths (voltage-source branches have no diagonal entry): every source's
    node and branch become singleton blocks, the resistive network between
    them one block."""
    from ngspice_gb300 import engine as E
    deck = ("t\nv1 a 0 1\nv2 b a 2\nr1 b c 1k\nr2 c 0 1k\nr3 c d 1k\nc1 d 0 1p\n"
            ".tran 1n 10n\n.end\n")
    c = E.Circuit(deck, host_only=True)
    nb, big = c.smp_preorder()
    # unknowns a, b, c, d, v1#branch, v2#branch: the sources' nodes and
    # branches are singletons, c and d one block
    assert c.n == 6
    assert (nb, big) == (5, 2)
    rc = E.Circuit("t\nv1 a 0 1\nr1 a b 1k\nr2 b 0 1k\n.tran 1n 10n\n.end\n", host_only=True)
    assert rc.smp_preorder() == (3, 1)
