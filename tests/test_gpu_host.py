"""crs_wdot_host: wdot from host arrays, read in place (pinned memory the
device addresses) or chunked over two streams (pageable memory, or
CRS_HOST_STAGED).

Each state is evaluated by the same kernel as crs_wdot, so the results must
be bit-identical to crs_wdot on device copies of the same inputs, for one
chunk, several chunks with a ragged tail, a row stride larger than n, pinned
and pageable host memory, both paths, and every mode.
"""
import ctypes

import numpy as np
import pytest

from create_rate_subs_gb300 import _lib, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def rs(synth_mech):
    from create_rate_subs_gb300.rates import RateSubs
    return RateSubs(synth_mech("gri53"))


def _device_ref(rs, T, P, Y, mode):
    dT, dP, dY = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (T, P, Y))
    return rs.wdot(dT, dP, dY, mode=mode).cpu().numpy()


@pytest.mark.parametrize("n", [1, 1000, (1 << 17) + 77])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_host_matches_device(rs, n, mode):
    N = rs.n_species
    T, P, Y = synth.make_states(N, n, seed=n)
    want = _device_ref(rs, T, P, Y[: N - 1], mode)
    got = rs.wdot_host(T, P, Y, mode=mode)
    assert np.array_equal(got, want)


def test_host_pinned_and_strided(rs):
    N, n, ld = rs.n_species, 70001, 70400
    T, P, Y = synth.make_states(N, n, seed=5)
    want = _device_ref(rs, T, P, Y[: N - 1], "fp64")
    hY = torch.zeros((N, ld), dtype=torch.float64).pin_memory()
    hY[:, :n] = torch.from_numpy(Y)
    hT = torch.from_numpy(T).pin_memory()
    hP = torch.from_numpy(P).pin_memory()
    hW = torch.full((N, ld), float("nan"), dtype=torch.float64).pin_memory()
    lib = _lib.load()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.crs_wdot_host(rs.h, n, p(hT), p(hP), p(hY), ld, p(hW), 0) == 0, _lib.last_error()
    assert np.array_equal(hW[:, :n].numpy(), want)
    assert torch.isnan(hW[:, n:]).all()          # padding columns untouched


def test_host_every_mode(rs):
    N, n = rs.n_species, 3000
    T, P, Y = synth.make_states(N, n, seed=9)
    for mode in _lib.MODES:
        want = _device_ref(rs, T, P, Y[: N - 1], mode)
        assert np.array_equal(rs.wdot_host(T, P, Y, mode=mode), want), mode


def test_host_rejects_bad_arguments(rs):
    lib = _lib.load()
    assert lib.crs_wdot_host(rs.h, -1, None, None, None, 0, None, 0) == 1
    assert lib.crs_wdot_host(rs.h, 10, None, None, None, 10, None, 0) == 1
    assert lib.crs_wdot_host(None, 10, None, None, None, 10, None, 0) == 1
    x = np.zeros(10)
    y = np.zeros((rs.n_species, 10))
    assert lib.crs_wdot_host(rs.h, 10, x.ctypes.data, x.ctypes.data, y.ctypes.data, 5,
                             y.ctypes.data, 0) == 1   # ld < n


def _pinned(T, P, Y, N, ld):
    hT = torch.from_numpy(T).pin_memory()
    hP = torch.from_numpy(P).pin_memory()
    hY = torch.zeros((N - 1, ld), dtype=torch.float64).pin_memory()
    hY[:, : T.shape[0]] = torch.from_numpy(Y[: N - 1])
    hW = torch.full((N, ld), float("nan"), dtype=torch.float64).pin_memory()
    return hT, hP, hY, hW


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("mode", ["fp64", "mixed", "gemm"])
def test_host_pinned_in_place_and_staged(rs, mode, staged):
    """Pinned arrays: read in place by one launch, or (CRS_HOST_STAGED)
    copied through device buffers; both bit-identical to crs_wdot."""
    from create_rate_subs_gb300.rates import HOST_STAGED
    N, n, ld = rs.n_species, (1 << 17) + 333, (1 << 17) + 512
    T, P, Y = synth.make_states(N, n, seed=31)
    want = _device_ref(rs, T, P, Y[: N - 1], mode)
    hT, hP, hY, hW = _pinned(T, P, Y, N, ld)
    lib = _lib.load()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    flag = _lib.MODES[mode] | (HOST_STAGED if staged else 0)
    assert lib.crs_wdot_host(rs.h, n, p(hT), p(hP), p(hY), ld, p(hW), flag) == 0, \
        _lib.last_error()
    assert np.array_equal(hW[:, :n].numpy(), want)
    assert torch.isnan(hW[:, n:]).all()
