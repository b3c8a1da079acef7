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


@pytest.mark.parametrize("name", ["small", "gri53"])
def test_oracle_bitexact_vs_reference_build(name, synth_mech):
    if not RefLib.available(name):
        pytest.skip("reference C not built here (python oracle/build_ref.py all %s)" % name)
    mech = synth_mech(name)
    T, P, Y = synth.make_states(mech.n_species, 3000, seed=99)
    a = Oracle(mech.blob).eval(T, P, Y)
    b = RefLib(name).eval(T, P, Y)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


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
