"""GPU parity: libcrs kernels against the reference's outputs.

Reference values are the golden vectors (produced by the reference's own
emitted C) and, for fresh random states, the CPU oracle, which is pinned
bit-exact to those vectors (tests/test_oracle.py).

Tolerances
* CRS_MODE_FP64_STRICT: concentrations and species-rate sums involve no
  transcendental function and must be bit-identical; fwd / rev / pres_mod
  differ from the host only through exp/log/pow last bits: per-entry
  relative error <= 1e-13; wdot: scaled error <= 1e-12.
* wdot errors use the gross-rate normalisation of oracle.wdot_errors:
  |w - w_ref| / G with G_k = sum_r |nu_kr| (|fwd_r| + |rev_r|) pres_mod_r.
"""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN_CASES
from create_rate_subs_gb300 import _lib, synth
from oracle.oracle import Oracle, gross_scale, wdot_errors

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL_WDOT_FP64 = 1e-12
TOL_STAGE_FP64 = 1e-13
TOL_WDOT_MIXED = 1e-6
# wdot tolerance per mode (scaled error)
TOL = {"fp64_strict": TOL_WDOT_FP64, "fp64": TOL_WDOT_FP64, "mixed": TOL_WDOT_MIXED,
       "fp64_tps": TOL_WDOT_FP64, "mixed_tps": TOL_WDOT_MIXED,
       "fp64_warp": TOL_WDOT_FP64, "mixed_warp": TOL_WDOT_MIXED}


def _rs(mech):
    from create_rate_subs_gb300.rates import RateSubs
    return RateSubs(mech)


def _dev(*arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _relmax(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.abs(a - b)
    s = np.abs(b)
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(s > 0, d / s, d)
    return float(np.max(r)) if r.size else 0.0


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_strict_stages_vs_golden(case, golden):
    mech, g = golden(case)
    rs = _rs(mech)
    T, P, Y = _dev(g["T"], g["P"], g["Y"])
    out = {k: v.cpu().numpy() for k, v in rs.wdot_stages(T, P, Y, "fp64_strict").items()}
    assert np.array_equal(out["conc"], g["conc"])
    assert _relmax(out["fwd"], g["fwd"]) <= TOL_STAGE_FP64
    assert _relmax(out["rev"], g["rev"]) <= TOL_STAGE_FP64
    assert _relmax(out["pm"], g["pm"]) <= TOL_STAGE_FP64
    G = gross_scale(mech.tables, g["fwd"], g["rev"], g["pm"])
    err = wdot_errors(out["wdot"], g["wdot"], G)
    assert err["scaled"] <= TOL_WDOT_FP64, err
    assert rs.status() == (0, 0)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_batched_reference_functions_vs_golden(case, golden):
    """The four reference functions, batched, stage by stage."""
    mech, g = golden(case)
    rs = _rs(mech)
    T, P, Y, C, F, R, PM = _dev(g["T"], g["P"], g["Y"], g["conc"], g["fwd"],
                                g["rev"], g["pm"])
    y_N, mw, rho, conc = rs.eval_conc(T, P, Y)
    assert np.array_equal(conc.cpu().numpy(), g["conc"])
    assert np.array_equal(torch.stack([y_N, mw, rho]).cpu().numpy(), g["misc"])
    fwd, rev = rs.eval_rxn_rates(T, P, C)
    assert _relmax(fwd.cpu().numpy(), g["fwd"]) <= TOL_STAGE_FP64
    assert _relmax(rev.cpu().numpy(), g["rev"]) <= TOL_STAGE_FP64
    pm = rs.get_rxn_pres_mod(T, P, C)
    assert _relmax(pm.cpu().numpy(), g["pm"]) <= TOL_STAGE_FP64
    # spec rates from the reference's own fwd/rev/pm: only + and *, so exact
    w = rs.eval_spec_rates(F, R, PM)
    assert np.array_equal(w.cpu().numpy(), g["wdot"])


@pytest.mark.parametrize("case", ["small", "features"])
def test_per_state_dropin(case, golden):
    """The reference's per-state signatures through crs_bind on a handle
    loaded onto the GPU: they evaluate its host table image and equal the
    reference bit for bit."""
    mech, g = golden(case)
    rs = _rs(mech)
    lib = _lib.load()
    _lib.check(lib.crs_bind(rs.h))
    N, R, NREV, NPM = (int(x) for x in g["dims"])
    dp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    try:
        for i in (0, 5, g["T"].shape[0] - 1):
            y = np.ascontiguousarray(g["Y"][: N - 1, i])
            conc = np.zeros(N)
            yN, mw, rho = (ctypes.c_double(), ctypes.c_double(), ctypes.c_double())
            lib.eval_conc(g["T"][i], g["P"][i], dp(y), ctypes.byref(yN),
                          ctypes.byref(mw), ctypes.byref(rho), dp(conc))
            assert np.array_equal(conc, g["conc"][:, i])
            assert (yN.value, mw.value, rho.value) == tuple(g["misc"][:, i])
            C = np.ascontiguousarray(g["conc"][:, i])
            fwd, rev, pm = np.zeros(R), np.zeros(max(NREV, 1)), np.zeros(max(NPM, 1))
            lib.eval_rxn_rates(g["T"][i], g["P"][i], dp(C), dp(fwd), dp(rev))
            assert np.array_equal(fwd, g["fwd"][:, i])
            assert np.array_equal(rev[:NREV], g["rev"][:, i])
            lib.get_rxn_pres_mod(g["T"][i], g["P"][i], dp(C), dp(pm))
            assert np.array_equal(pm[:NPM], g["pm"][:, i])
            F = np.ascontiguousarray(g["fwd"][:, i])
            Rr = np.ascontiguousarray(g["rev"][:, i]) if NREV else np.zeros(1)
            PMr = np.ascontiguousarray(g["pm"][:, i]) if NPM else np.zeros(1)
            sp = np.zeros(N)
            dyN = ctypes.c_double()
            lib.eval_spec_rates(dp(F), dp(Rr), dp(PMr), dp(sp), ctypes.byref(dyN))
            assert np.array_equal(sp[: N - 1], g["wdot"][: N - 1, i])
            assert dyN.value == g["wdot"][N - 1, i]
    finally:
        lib.crs_bind(None)


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("mode", ["fp64", "mixed", "fp64_tps", "mixed_tps", "fp64_warp", "mixed_warp"])
def test_fast_modes_vs_golden(case, mode, golden):
    """Restructured FP64 and mixed precision against the reference's own
    outputs; the fused kernel's intermediates are checked too."""
    mech, g = golden(case)
    rs = _rs(mech)
    T, P, Y = _dev(g["T"], g["P"], g["Y"])
    out = {k: v.cpu().numpy() for k, v in rs.wdot_stages(T, P, Y, mode).items()}
    G = gross_scale(mech.tables, g["fwd"], g["rev"], g["pm"])
    err = wdot_errors(out["wdot"], g["wdot"], G)
    assert err["scaled"] <= TOL[mode], err
    # concentrations relative to the total concentration: the bath gas
    # inherits the cancellation of y_N = 1 - sum(y), which FP64 summation
    # orders resolve differently
    stage_tol = 1e-13 if mode.startswith("fp64") else 2e-7
    ctot = np.abs(g["conc"]).sum(axis=0)
    assert np.max(np.abs(out["conc"] - g["conc"]) / ctot) <= stage_tol
    assert rs.status() == (0, 0)


@pytest.mark.parametrize("n", [1, 31, 33, 127, 129, 1000])
def test_odd_sizes_and_tails(n, synth_mech):
    mech = synth_mech("gri53")
    T, P, Y = synth.make_states(mech.n_species, n, seed=n)
    ref = Oracle(mech.blob).eval(T, P, Y)
    G = gross_scale(mech.tables, ref["fwd"], ref["rev"], ref["pm"])
    rs = _rs(mech)
    dT, dP, dY = _dev(T, P, Y)
    for mode in ("fp64_strict", "fp64", "mixed", "fp64_tps", "mixed_tps", "fp64_warp", "mixed_warp"):
        w = rs.wdot(dT, dP, dY, mode).cpu().numpy()
        assert wdot_errors(w, ref["wdot"], G)["scaled"] <= TOL[mode], mode


def test_strided_soa(synth_mech):
    """ld > n: states embedded in a wider SoA buffer."""
    mech = synth_mech("small")
    n, ld = 300, 512
    T, P, Y = synth.make_states(mech.n_species, n, seed=3)
    ref = Oracle(mech.blob).eval(T, P, Y)
    G = gross_scale(mech.tables, ref["fwd"], ref["rev"], ref["pm"])
    rs = _rs(mech)
    big = np.zeros((mech.n_species, ld))
    big[:, :n] = Y
    dT, dP, dY = _dev(T, P, big)
    dY = dY[:, :n]
    w = rs.wdot(dT, dP, dY, "fp64_strict").cpu().numpy()
    assert wdot_errors(w, ref["wdot"], G)["scaled"] <= TOL_WDOT_FP64


@pytest.mark.parametrize("mode", ["fp64_strict", "fp64", "mixed", "fp64_tps", "mixed_tps", "fp64_warp", "mixed_warp"])
def test_random_states_gri53(mode, synth_mech):
    mech = synth_mech("gri53")
    n = 1 << 14
    T, P, Y = synth.make_states(mech.n_species, n, seed=1234)
    ref = Oracle(mech.blob).eval(T, P, Y)
    G = gross_scale(mech.tables, ref["fwd"], ref["rev"], ref["pm"])
    rs = _rs(mech)
    dT, dP, dY = _dev(T, P, Y)
    w = rs.wdot(dT, dP, dY, mode).cpu().numpy()
    err = wdot_errors(w, ref["wdot"], G)
    print(mode, err)
    assert err["scaled"] <= TOL[mode], err


def test_nonfinite_inputs_are_counted(synth_mech):
    """A NaN temperature yields non-finite wdot and is reported through the
    status word, not by trapping."""
    mech = synth_mech("small")
    T, P, Y = synth.make_states(mech.n_species, 64, seed=5)
    T[7] = np.nan
    rs = _rs(mech)
    dT, dP, dY = _dev(T, P, Y)
    for mode in ("fp64_strict", "fp64", "mixed", "fp64_tps", "mixed_tps", "fp64_warp", "mixed_warp"):
        rs.reset_status()
        w = rs.wdot(dT, dP, dY, mode).cpu().numpy()
        flags, bad = rs.status()
        assert flags == 0
        assert bad == int(np.sum(~np.isfinite(w))) and bad > 0, mode
        assert np.all(np.isfinite(np.delete(w, 7, axis=1))), mode


def test_argument_errors(synth_mech):
    mech = synth_mech("small")
    rs = _rs(mech)
    lib = _lib.load()
    rc = lib.crs_wdot(rs.h, -1, None, None, None, 0, None, 0, None)
    assert rc == 1
    rc = lib.crs_wdot(rs.h, 10, None, None, None, 5, None, 0, None)
    assert rc == 1
    T, P, Y = _dev(*synth.make_states(mech.n_species, 8, seed=1))
    w = torch.empty((mech.n_species, 8), dtype=torch.float64, device="cuda")
    rc = lib.crs_wdot(rs.h, 8, ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(P.data_ptr()),
                      ctypes.c_void_p(Y.data_ptr()), 8, ctypes.c_void_p(w.data_ptr()), 99, None)
    assert rc == 1


# ---- tensor-core contraction (CRS_MODE_GEMM) and large mechanisms --------

TOL_WDOT_GEMM = 1e-4   # bf16 hi+lo terms (~2^-17 each) summed in fp32


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gemm_mode_vs_golden(case, golden):
    mech, g = golden(case)
    rs = _rs(mech)
    T, P, Y = _dev(g["T"], g["P"], g["Y"])
    w = rs.wdot(T, P, Y, "gemm").cpu().numpy()
    G = gross_scale(mech.tables, g["fwd"], g["rev"], g["pm"])
    err = wdot_errors(w, g["wdot"], G)
    print(case, err)
    assert err["scaled"] <= TOL_WDOT_GEMM, err
    assert rs.status() == (0, 0)


@pytest.mark.parametrize("n", [1, 127, 129, 5000, (1 << 18) + 77])
def test_gemm_mode_sizes_and_chunks(n, synth_mech):
    """Tails of the 128-row tiles and more states than one workspace chunk;
    checked against the FP64 kernel (itself pinned to the oracle)."""
    mech = synth_mech("gri53")
    T, P, Y = synth.make_states(mech.n_species, n, seed=n + 1)
    rs = _rs(mech)
    dT, dP, dY = _dev(T, P, Y)
    ref = rs.wdot_stages(dT, dP, dY, "fp64_strict")
    w = rs.wdot(dT, dP, dY, "gemm").cpu().numpy()
    R = {k: v.cpu().numpy() for k, v in ref.items()}
    G = gross_scale(mech.tables, R["fwd"], R["rev"], R["pm"])
    assert wdot_errors(w, R["wdot"], G)["scaled"] <= TOL_WDOT_GEMM


def test_large_mechanism_all_modes(synth_mech):
    """561 species / 2539 reactions: tables in global memory, warp-per-state
    kernels, and the tensor-core contraction, against the oracle."""
    mech = synth_mech("large561")
    n = 600
    T, P, Y = synth.make_states(mech.n_species, n, seed=21)
    ref = Oracle(mech.blob).eval(T, P, Y)
    G = gross_scale(mech.tables, ref["fwd"], ref["rev"], ref["pm"])
    rs = _rs(mech)
    dT, dP, dY = _dev(T, P, Y)
    for mode, tol in (("fp64", TOL_WDOT_FP64), ("fp64_strict", TOL_WDOT_FP64),
                      ("mixed", TOL_WDOT_MIXED), ("gemm", TOL_WDOT_GEMM)):
        w = rs.wdot(dT, dP, dY, mode).cpu().numpy()
        err = wdot_errors(w, ref["wdot"], G)
        print("large561", mode, err)
        assert err["scaled"] <= tol, (mode, err)
    assert rs.status() == (0, 0)


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("mode,tol", [("mixed_tile", TOL_WDOT_MIXED), ("gemm", 1e-4),
                                      ("fp64_tile", TOL_WDOT_FP64)])
def test_two_pass_modes_vs_golden(case, mode, tol, golden):
    """The two-pass state-tile path (FP64 net rates through HBM, then the
    species sums or the tensor-core contraction) against the reference's
    own outputs, on every golden mechanism: PLOG, Chebyshev, explicit REV,
    several T_common groups and the edge states included."""
    mech, g = golden(case)
    rs = _rs(mech)
    T, P, Y = _dev(g["T"], g["P"], g["Y"])
    w = rs.wdot(T, P, Y, mode).cpu().numpy()
    G = gross_scale(mech.tables, g["fwd"], g["rev"], g["pm"])
    err = wdot_errors(w, g["wdot"], G)
    assert err["scaled"] <= tol, err
    assert rs.status() == (0, 0)


@pytest.mark.parametrize("name", ["gri53", "large561"])
def test_two_pass_matches_oracle_odd_sizes(name, synth_mech):
    """Odd state counts (partial tiles of 32, several chunks for the large
    mechanism) and a batch with ld > n."""
    from oracle.oracle import Oracle
    mech = synth_mech(name)
    rs = _rs(mech)
    N = mech.n_species
    for n in (1, 33, 1000):
        T, P, Y = synth.make_states(N, n, seed=17 + n)
        ref = Oracle(mech.blob).eval(T, P, Y)
        G = gross_scale(mech.tables, ref["fwd"], ref["rev"], ref["pm"])
        ld = n + 7
        Yp = np.zeros((N - 1, ld))
        Yp[:, :n] = Y[: N - 1]
        dT, dP, dY = _dev(T, P, Yp)
        lib = _lib.load()
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for mode, tol in (("mixed_tile", TOL_WDOT_MIXED), ("gemm", 1e-4),
                          ("fp64_tile", TOL_WDOT_FP64)):
            W = torch.full((N, ld), 7.0, dtype=torch.float64, device="cuda")
            _lib.check(lib.crs_wdot(rs.h, n, p(dT), p(dP), p(dY), ld, p(W), _lib.MODES[mode],
                                    st))
            Wh = W.cpu().numpy()
            assert np.all(Wh[:, n:] == 7.0), (name, n, mode)   # padding untouched
            err = wdot_errors(Wh[:, :n], ref["wdot"], G)
            assert err["scaled"] <= tol, (name, n, mode, err)
    assert rs.status() == (0, 0)
