"""Thermo utilities and dydt on the GPU against the reference's outputs.

* eval_h / eval_u / eval_cv / eval_cp and eval_conc_rho: bit-identical to
  the reference's emitted C (golden vectors; crs_dydt.cu is built without
  FMA contraction, in the emitted operand order);
* constant-pressure dydt against the reference's emitted dydt (golden):
  species rows within the wdot tolerance of the mode, scaled by the gross
  rate G_k mw_k / rho; dT/dt within the same tolerance of its gross energy
  scale sum_k |dY_k/dt| |h_k| rho / (rho cp_avg);
* constant volume (the reference's text does not compile) against the CPU
  oracle's restatement;
* the per-state drop-ins eval_h ... dydt through crs_bind.
"""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN_CASES
from create_rate_subs_gb300 import _lib
from oracle.oracle import Oracle, gross_scale

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = {"fp64_strict": 1e-12, "fp64": 1e-12, "mixed": 1e-6}


def _rs(mech):
    from create_rate_subs_gb300.rates import RateSubs
    return RateSubs(mech)


def _d(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _ystate(g, N):
    return np.concatenate([g["T"][None], g["Y"][: N - 1]], axis=0)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_thermo_and_conc_rho_bitexact(case, golden):
    mech, g = golden(case)
    rs = _rs(mech)
    T = _d(g["T"])
    for w, f in (("h", rs.eval_h), ("u", rs.eval_u), ("cv", rs.eval_cv), ("cp", rs.eval_cp)):
        assert np.array_equal(f(T).cpu().numpy(), g["thermo_" + w]), w
    y_N, mw, p, conc = rs.eval_conc_rho(T, _d(g["misc"][2]), _d(g["Y"][: mech.n_species - 1]))
    assert np.array_equal(np.stack([y_N.cpu().numpy(), mw.cpu().numpy(), p.cpu().numpy()]),
                          g["conc_rho_misc"])
    assert np.array_equal(conc.cpu().numpy(), g["conc_rho"])
    assert rs.status() == (0, 0)


def _check_dydt(mech, g, dy, ref, tol, thermo_e, thermo_c):
    N = mech.n_species
    mw = mech.tables["sp_mw"]
    rho = g["misc"][2]
    G = gross_scale(mech.tables, g["fwd"], g["rev"], g["pm"])
    sc = G[: N - 1] * mw[: N - 1, None] / rho
    ok = sc > 0
    assert np.max(np.abs(dy[1:] - ref[1:])[ok] / sc[ok]) <= tol
    yN = 1.0 - g["Y"][: N - 1].sum(axis=0)
    Yf = np.concatenate([g["Y"][: N - 1], yN[None]], axis=0)
    c_avg = (thermo_c * Yf).sum(axis=0)
    gross_T = (G * np.abs(thermo_e) * mw[:, None]).sum(axis=0) / np.abs(rho * c_avg)
    okT = gross_T > 0
    assert np.max(np.abs(dy[0] - ref[0])[okT] / gross_T[okT]) <= tol


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("mode", ["fp64_strict", "fp64", "mixed"])
def test_dydt_conp_vs_reference(case, mode, golden):
    mech, g = golden(case)
    rs = _rs(mech)
    N = mech.n_species
    dy = rs.dydt(_d(g["P"]), _d(_ystate(g, N)), conv=False, mode=mode).cpu().numpy()
    _check_dydt(mech, g, dy, g["dydt_conp"], TOL[mode], g["thermo_h"], g["thermo_cp"])
    assert rs.status()[0] == 0


@pytest.mark.parametrize("case", ["gri53", "features"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_dydt_conv_vs_oracle(case, mode, golden):
    mech, g = golden(case)
    rs = _rs(mech)
    N = mech.n_species
    y = _ystate(g, N)
    rho = g["misc"][2]
    ref = Oracle(mech.blob).dydt(rho, y, conv=True)
    dy = rs.dydt(_d(rho), _d(y), conv=True, mode=mode).cpu().numpy()
    _check_dydt(mech, g, dy, ref, TOL[mode], g["thermo_u"], g["thermo_cv"])


def test_dydt_strided_and_large(synth_mech):
    from create_rate_subs_gb300 import synth
    mech = synth_mech("gri53")
    rs = _rs(mech)
    N, n, ld = mech.n_species, 100_003, 100_096
    T, P, Y = synth.make_states(N, n, seed=4)
    y = torch.zeros((N, ld), dtype=torch.float64, device="cuda")
    y[0, :n] = _d(T)
    y[1:, :n] = _d(Y[: N - 1])
    dy = rs.dydt(_d(P), y[:, :n], mode="fp64")
    ref = Oracle(mech.blob).dydt(P[:2000], np.concatenate([T[None], Y[: N - 1]])[:, :2000])
    got = dy[:, :2000].cpu().numpy()
    scale = np.abs(ref).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(got - ref) / scale) <= 1e-10
    assert np.all(np.isfinite(dy.cpu().numpy()))


def test_per_state_dropins(golden):
    mech, g = golden("gri53")
    rs = _rs(mech)
    lib = _lib.load()
    assert lib.crs_bind(rs.h) == 0
    try:
        N = mech.n_species
        i = 3
        h = np.zeros(N)
        lib.eval_h(float(g["T"][i]), h.ctypes.data)
        assert np.array_equal(h, g["thermo_h"][:, i])
        cp = np.zeros(N)
        lib.eval_cp(float(g["T"][i]), cp.ctypes.data)
        assert np.array_equal(cp, g["thermo_cp"][:, i])
        # dydt per state runs on the host in the reference's order: the
        # reference's emitted constant-pressure dydt bit for bit, and the
        # oracle's constant-volume restatement bit for bit
        ys = _ystate(g, N)
        y = np.ascontiguousarray(ys[:, i])
        dy = np.zeros(N)
        lib.dydt(0.0, float(g["P"][i]), y.ctypes.data, dy.ctypes.data)
        assert np.array_equal(dy, g["dydt_conp"][:, i])
        assert lib.crs_dydt_form(1) == 0
        rho = g["misc"][2]
        lib.dydt(0.0, float(rho[i]), y.ctypes.data, dy.ctypes.data)
        conv = Oracle(mech.blob).dydt(rho, ys, conv=True)
        assert np.array_equal(dy, conv[:, i])
    finally:
        lib.crs_dydt_form(0)
        lib.crs_bind(None)
