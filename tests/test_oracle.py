"""The CPU oracle against the reference's own outputs (CPU only).

The golden vectors were produced by the reference's emitted C
(tests/golden/make_golden.py); the oracle must reproduce every stage
bit for bit.  When the reference's C is built locally (oracle/_ref), the
oracle is also compared with it on fresh random states.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES
from create_rate_subs_gb300 import synth
from oracle.oracle import Oracle, RefLib, gross_scale, wdot_errors


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_bitexact_vs_golden(case, golden):
    mech, g = golden(case)
    out = Oracle(mech.blob).eval(g["T"], g["P"], g["Y"])
    for k in ("conc", "fwd", "rev", "pm", "wdot", "misc"):
        assert np.array_equal(out[k], g[k]), k


@pytest.mark.parametrize("name,n", [("small", 3000), ("gri53", 3000), ("large561", 1024)])
def test_oracle_bitexact_vs_reference_build(name, n, synth_mech):
    """Every stage of the oracle equals the reference's own emitted C on
    fresh seeded states, for each workload mechanism (the 561-species /
    2539-reaction one included)."""
    if not RefLib.available(name):
        pytest.skip("reference C not built here (python oracle/build_ref.py all %s)" % name)
    mech = synth_mech(name)
    T, P, Y = synth.make_states(mech.n_species, n, seed=99)
    a = Oracle(mech.blob).eval(T, P, Y)
    b = RefLib(name).eval(T, P, Y)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name", ["small", "gri53", "large561"])
def test_reference_build_keeps_its_mechanism_text(name):
    """The reference build of each workload keeps the Chemkin text it was
    emitted from, and on this host the generator still writes that text."""
    import tempfile
    from oracle import build_ref
    files = build_ref.mechanism_files(name)
    if files is None:
        pytest.skip("reference C not built here (python oracle/build_ref.py all %s)" % name)
    fresh = synth.write_mechanism(name, tempfile.mkdtemp(prefix="crs_mech_"))
    for a, b in zip(files, fresh):
        with open(a) as fa, open(b) as fb:
            assert fa.read() == fb.read(), a


def test_oracle_omp_matches_serial(golden):
    mech, g = golden("gri53")
    o = Oracle(mech.blob)
    w, used = o.wdot_omp(g["T"], g["P"], g["Y"], nthreads=2)
    assert used >= 1
    assert np.array_equal(w, g["wdot"])


def test_error_metric_planted_mistake(golden):
    """A mistake planted in an oracle output is caught by the metric."""
    mech, g = golden("gri53")
    G = gross_scale(mech.tables, g["fwd"], g["rev"], g["pm"])
    e0 = wdot_errors(g["wdot"], g["wdot"], G)
    assert e0["scaled"] == 0.0
    w = g["wdot"].copy()
    k, i = 5, 3
    w[k, i] += 1e-9 * G[k, i]
    e1 = wdot_errors(w, g["wdot"], G)
    assert 0.9e-9 < e1["scaled"] < 1.1e-9


# ---- thermo utilities and dydt (rate_subs.py:1396-1776, 1829-2067) -------

def _y_state(g, N):
    return np.concatenate([g["T"][None], g["Y"][: N - 1]], axis=0)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_thermo_and_dydt_bitexact_vs_golden(case, golden):
    mech, g = golden(case)
    o = Oracle(mech.blob)
    for w in ("h", "u", "cv", "cp"):
        assert np.array_equal(o.thermo(w, g["T"]), g["thermo_" + w]), w
    misc, conc = o.conc_rho(g["T"], g["misc"][2], g["Y"])
    assert np.array_equal(misc, g["conc_rho_misc"])
    assert np.array_equal(conc, g["conc_rho"])
    N = mech.n_species
    assert np.array_equal(o.dydt(g["P"], _y_state(g, N)), g["dydt_conp"])


@pytest.mark.parametrize("case", ["gri53", "features"])
def test_oracle_conv_consistent_with_conp(case, golden):
    """Constant volume at the density constant pressure produced: the same
    species rates (the pressure differs only by rounding), and
    dT/dt = -sum(wdot_k u_k mw_k) / (rho cv_avg)."""
    mech, g = golden(case)
    o = Oracle(mech.blob)
    N = mech.n_species
    y = _y_state(g, N)
    rho = g["misc"][2]
    dv = o.dydt(rho, y, conv=True)
    dp = g["dydt_conp"]
    G = gross_scale(mech.tables, g["fwd"], g["rev"], g["pm"])
    mw = mech.tables["sp_mw"]
    scale = G[: N - 1] * mw[: N - 1, None] / rho
    ok = scale > 0
    assert np.max(np.abs(dv[1:] - dp[1:])[ok] / scale[ok]) <= 1e-12
    u, cv = o.thermo("u", g["T"]), o.thermo("cv", g["T"])
    yN = 1.0 - g["Y"][: N - 1].sum(axis=0)
    Yf = np.concatenate([g["Y"][: N - 1], yN[None]], axis=0)
    cv_avg = (cv * Yf).sum(axis=0)
    w = Oracle(mech.blob).eval(g["T"], g["P"], g["Y"])["wdot"]
    sumt = (w * u * mw[:, None])
    dT = -sumt.sum(axis=0) / (rho * cv_avg)
    gross = np.abs(sumt).sum(axis=0) / np.abs(rho * cv_avg)
    assert np.max(np.abs(dv[0] - dT) / np.maximum(gross, 1e-300)) <= 1e-12


@pytest.mark.parametrize("name", ["small", "gri53"])
def test_oracle_dydt_bitexact_vs_reference_build(name, synth_mech):
    from oracle.oracle import RefDydt
    if not RefDydt.available(name):
        pytest.skip("reference dydt not built here (python oracle/build_ref.py all %s)" % name)
    mech = synth_mech(name)
    N = mech.n_species
    T, P, Y = synth.make_states(N, 2000, seed=98)
    y = np.concatenate([T[None], Y[: N - 1]], axis=0)
    assert np.array_equal(Oracle(mech.blob).dydt(P, y), RefDydt(name).dydt(P, y))
