"""The allocation-free entry point crs_wdot_gemm_noalloc.

It exists for callers that cannot allocate device memory while they
evaluate rates (memory pools or frameworks that own every allocation,
embedding runtimes, time-stepping loops that must not block on cudaMalloc).
Through the C ABI it must give what crs_wdot(..., CRS_MODE_GEMM, ...) gives,
within that mode's tolerance, on two calls in a row -- the second call
finds the previous call's data in the shared scratch array.

This file is collected last on purpose, and passes on its own in a fresh
process as well as after every other test.
"""
import ctypes
import tempfile

import numpy as np
import pytest

from create_rate_subs_gb300 import _lib, synth
from create_rate_subs_gb300.mechanism import Mechanism
from oracle.oracle import gross_scale

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL_WDOT_GEMM = 1e-4  # the tensor-core contraction's tolerance (scaled error)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("name,n", [("gri53", 50000), ("large561", 3000)])
def test_noalloc_matches_gemm_mode_twice(name, n):
    from create_rate_subs_gb300.rates import RateSubs
    d = tempfile.mkdtemp(prefix="crs_noalloc_")
    mech = Mechanism.from_chemkin(*synth.write_mechanism(name, d))
    rs = RateSubs(mech)
    lib = _lib.load()
    N = mech.n_species
    T, P, Y = synth.make_states(N, n, seed=99)
    dT, dP, dY = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (T, P, Y[: N - 1]))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = torch.empty((N, n), dtype=torch.float64, device="cuda")
    assert lib.crs_wdot(rs.h, n, _p(dT), _p(dP), _p(dY), n, _p(ref),
                        _lib.MODES["gemm"], stream) == 0, _lib.last_error()
    stages = rs.wdot_stages(dT, dP, dY, "fp64_strict")
    S = {k: v.cpu().numpy() for k, v in stages.items()}
    G = gross_scale(mech.tables, S["fwd"], S["rev"], S["pm"])
    G = np.where(G == 0, 1.0, G)
    want = ref.cpu().numpy()
    for call in range(2):
        out = torch.full((N, n), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.crs_wdot_gemm_noalloc(rs.h, n, _p(dT), _p(dP), _p(dY), n, _p(out), stream)
        assert rc == 0, _lib.last_error()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got)), call
        assert np.max(np.abs(got - want) / G) <= TOL_WDOT_GEMM, call
    assert rs.status() == (0, 0)


def test_noalloc_rejects_bad_arguments():
    from create_rate_subs_gb300.rates import RateSubs
    d = tempfile.mkdtemp(prefix="crs_noalloc_")
    rs = RateSubs(Mechanism.from_chemkin(*synth.write_mechanism("small", d)))
    lib = _lib.load()
    assert lib.crs_wdot_gemm_noalloc(rs.h, -1, None, None, None, 0, None, None) == 1
    assert lib.crs_wdot_gemm_noalloc(rs.h, 10, None, None, None, 10, None, None) == 1
    assert lib.crs_wdot_gemm_noalloc(None, 10, None, None, None, 10, None, None) == 1
