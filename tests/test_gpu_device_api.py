"""The reference's per-state functions called from a user's own CUDA kernel.

The CLI's cuda target writes rates.cuh / chem_utils.cuh / dydt.cuh with
__device__ definitions of eval_conc, eval_rxn_rates, get_rxn_pres_mod,
eval_spec_rates and dydt over the mechanism's table image
(include/crs_device.cuh), as the reference's -l cuda output declares them
for its integrator kernels (rate_subs.py:256, 283; create_rate_subs.py:
57-102).  This test writes a small user kernel that calls them one state
per thread, compiles it with nvcc -fmad=false for sm_103a, and checks:

* concentrations equal the reference's golden vectors bit for bit, and
  fwd / rev / pres_mod are within 1e-13 relative (CUDA's exp/log/pow);
* every output equals the batched reference-order kernel
  (CRS_MODE_FP64_STRICT) and its dydt bit for bit: the same arithmetic
  (include/crs_eval.h) under the same rounding rules.
"""
import ctypes
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from create_rate_subs_gb300 import build as crs_build
from create_rate_subs_gb300.create_rate_subs import create_rate_subs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

USER_KERNEL = r'''
#include "rates.cuh"
#include "chem_utils.cuh"
#include "dydt.cuh"

// one state per thread, as an integrator's right-hand-side kernel calls
// the reference's device functions
__global__ void k_user(int n, const double *T, const double *P, const double *Y,
                       double *conc, double *fwd, double *rev, double *pm,
                       double *wdot, double *dy, double *scratch) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double y[NSP], C[NSP], f[NRXN], r[NRXN_REV > 0 ? NRXN_REV : 1];
  double p[NPDEP > 0 ? NPDEP : 1], sp[NSP], ys[NSP], d[NSP];
  for (int k = 0; k < NSP - 1; ++k) y[k] = Y[(long)k * n + i];
  double yN, mw, rho;
  eval_conc(T[i], P[i], y, &yN, &mw, &rho, C);
  eval_rxn_rates(T[i], P[i], C, f, r);
  get_rxn_pres_mod(T[i], P[i], C, p);
  eval_spec_rates(f, r, p, sp, &sp[NSP - 1]);
  ys[0] = T[i];
  for (int k = 0; k < NSP - 1; ++k) ys[k + 1] = y[k];
  dydt(0.0, P[i], ys, d, scratch + (long)i * crs_device_dydt_scratch());
  for (int k = 0; k < NSP; ++k) {
    conc[(long)k * n + i] = C[k];
    wdot[(long)k * n + i] = sp[k];
    dy[(long)k * n + i] = d[k];
  }
  for (int k = 0; k < NRXN; ++k) fwd[(long)k * n + i] = f[k];
  for (int k = 0; k < NRXN_REV; ++k) rev[(long)k * n + i] = r[k];
  for (int k = 0; k < NPDEP; ++k) pm[(long)k * n + i] = p[k];
}

extern "C" int run_user(int n, const double *T, const double *P, const double *Y,
                        double *conc, double *fwd, double *rev, double *pm, double *wdot,
                        double *dy, double *scratch) {
  k_user<<<(n + 127) / 128, 128>>>(n, T, P, Y, conc, fwd, rev, pm, wdot, dy, scratch);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int)e;
}

extern "C" int dydt_scratch(void) { return crs_device_dydt_scratch(); }
'''


def _relmax(a, b):
    d = np.abs(np.asarray(a) - np.asarray(b))
    s = np.abs(np.asarray(b))
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(s > 0, d / s, d)
    return float(np.max(r)) if r.size else 0.0


def _build_user(case, golden_case, tmp):
    """CLI cuda target for the golden mechanism, then the user kernel."""
    g = golden_case
    mp, tp = os.path.join(tmp, "mech.inp"), os.path.join(tmp, "therm.dat")
    with open(mp, "w") as f:
        f.write(str(g["mech_text"]))
    with open(tp, "w") as f:
        f.write(str(g["therm_text"]))
    out = os.path.join(tmp, "out")
    create_rate_subs("cuda", mp, tp, str(g["last_spec"]) or None, out_dir=out)
    src = os.path.join(tmp, "user.cu")
    with open(src, "w") as f:
        f.write(USER_KERNEL)
    lib = os.path.join(tmp, "libuser_%s.so" % case)
    cmd = [crs_build.nvcc()] + crs_build.ARCH + ["-O3", "-fmad=false", "-std=c++17",
                                                  "-Xcompiler", "-fPIC", "-shared", "-I", out,
                                                  "-o", lib, src]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    return ctypes.CDLL(lib)


@pytest.mark.parametrize("case", ["small", "features", "features_lastAR"])
def test_user_kernel_calls_device_functions(case, golden):
    from create_rate_subs_gb300.rates import RateSubs
    mech, g = golden(case)
    tmp = tempfile.mkdtemp(prefix="crs_devapi_")
    try:
        lib = _build_user(case, g, tmp)
        N, R, NREV, NPM = (int(x) for x in g["dims"])
        n = g["T"].shape[0]
        d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        T, P, Y = d(g["T"]), d(g["P"]), d(g["Y"][: N - 1])
        out = {k: torch.zeros((max(rows, 1), n), dtype=torch.float64, device="cuda")
               for k, rows in (("conc", N), ("fwd", R), ("rev", NREV), ("pm", NPM),
                               ("wdot", N), ("dy", N))}
        ns = int(lib.dydt_scratch())
        scratch = torch.zeros(ns * n, dtype=torch.float64, device="cuda")
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        rc = lib.run_user(ctypes.c_int(n), p(T), p(P), p(Y), p(out["conc"]), p(out["fwd"]),
                          p(out["rev"]), p(out["pm"]), p(out["wdot"]), p(out["dy"]),
                          p(scratch))
        assert rc == 0, "user kernel failed with CUDA error %d" % rc
        got = {k: v.cpu().numpy() for k, v in out.items()}
        # against the reference's own outputs
        assert np.array_equal(got["conc"], g["conc"])
        assert _relmax(got["fwd"], g["fwd"]) <= 1e-13
        assert _relmax(got["rev"][:NREV], g["rev"]) <= 1e-13
        assert _relmax(got["pm"][:NPM], g["pm"]) <= 1e-13
        # against the batched reference-order kernel: bit for bit
        rs = RateSubs(mech)
        st = {k: v.cpu().numpy() for k, v in rs.wdot_stages(T, P, Y, "fp64_strict").items()}
        assert np.array_equal(got["conc"], st["conc"])
        assert np.array_equal(got["fwd"], st["fwd"])
        assert np.array_equal(got["rev"][:NREV], st["rev"])
        assert np.array_equal(got["pm"][:NPM], st["pm"])
        assert np.array_equal(got["wdot"], st["wdot"])
        ystate = torch.cat([T[None], Y], dim=0)
        dy_batched = rs.dydt(P, ystate, conv=False, mode="fp64_strict").cpu().numpy()
        assert np.array_equal(got["dy"], dy_batched)
        assert rs.status() == (0, 0)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
