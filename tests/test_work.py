"""The algorithmic cost model behind the roofline fractions (CPU only).

work.fp64_slots counts the FP64-pipe work of one state as a lower bound in
FP64 instruction slots; bench.py's roofline divides the time that bound
allows by the measured time, so a kernel that does all the work cannot
score above 1."""
import importlib.util
import os

import pytest

from conftest import REPO
from create_rate_subs_gb300 import work


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_slots_follow_the_tables(synth_mech):
    t = synth_mech("gri53").tables
    R, NREV = int(t["dims"][1]), int(t["dims"][2])
    tile = work.fp64_slots(t, "mixed_tile", 9.0)
    assert tile["parts"]["kc_exponent"] == 6 * int(t["kc_ptr"][NREV])
    assert tile["parts"]["net_rate"] == NREV
    assert tile["parts"]["accumulation"] == int(t["nu_ptr"][R])
    # one T_common group per reaction: the one-state-per-thread kernel forms
    # the Kc exponents in float-float, off the FP64 pipe
    mixed = work.fp64_slots(t, "mixed", 9.0)
    assert "kc_exponent" not in mixed["parts"]
    assert mixed["slots"] == tile["slots"] - tile["parts"]["kc_exponent"]
    rates = work.fp64_slots(t, "rates", 9.0)
    assert rates["slots"] == tile["slots"] - tile["parts"]["accumulation"]
    w = work.work(t)
    full = work.fp64_slots(t, "fp64", 9.0)
    assert full["slots"] == w["flops"] / 2 + 9 * w["transcendentals"]
    # the FP64 split does strictly more FP64 work than the mixed ones
    assert full["slots"] > tile["slots"] > rates["slots"] > 0
    assert tile["slots"] > mixed["slots"] > 0
    with pytest.raises(ValueError):
        work.fp64_slots(t, "fp32", 9.0)


@pytest.mark.parametrize("precision,gemm", [("fp64", False), ("mixed", False), ("mixed_tile", False),
                                            ("rates", True)])
def test_roofline_fraction_is_one_at_the_bound(precision, gemm, synth_mech):
    b = _bench()
    t = synth_mech("gri53").tables
    N = int(t["dims"][0])
    peaks = {"fp64_fma_ops": 5.28e11, "fp64_table_exp": 5.28e11 / 9.2}
    probe = b._roofline(t, precision, 1.0, peaks, N, gemm=gemm)
    bound_ns = max(v for k, v in probe["per_state_ns"].items() if k != "measured")
    at_bound = b._roofline(t, precision, 1e9 / bound_ns, peaks, N, gemm=gemm)
    assert at_bound["frac"] == pytest.approx(1.0, rel=1e-12)
    slower = b._roofline(t, precision, 0.5e9 / bound_ns, peaks, N, gemm=gemm)
    assert slower["frac"] == pytest.approx(0.5, rel=1e-12)
    assert at_bound["exp_price_slots"] == pytest.approx(9.2)


def test_mixed_counts_fp64_kc_with_several_groups(golden):
    """A mechanism whose reactions span several T_common groups keeps the
    FP64 Kc polynomials in the mixed one-state-per-thread kernel, and the
    model counts them."""
    mech, _ = golden("features")
    t = mech.tables
    NREV = int(t["dims"][2])
    assert any(int(t["kc_ptr"][j + 1]) - int(t["kc_ptr"][j]) > 1 for j in range(NREV))
    mixed = work.fp64_slots(t, "mixed", 9.0)
    assert mixed["parts"]["kc_exponent"] == 6 * int(t["kc_ptr"][NREV])
    assert mixed["slots"] == work.fp64_slots(t, "mixed_tile", 9.0)["slots"]
