"""The mixed kernel's float-float Kc exponent (crs_mixed.cuh KcMix), on CPU.

The kernel evaluates ln(prefactor) + c0 + c1 ln T + T (c2 + T (c3 + T (c4 +
c5 T))) - c6 / T as seven float-float multiply-adds (ff_fma) over
coefficients split into FP32 pairs on the host (crs_fast.cu, kc_mix).  This
test restates that arithmetic in numpy (IEEE float32 operations; each
fmaf as an exact product plus one rounding) and bounds its distance to the
FP64 polynomial of the same tables over T in [300, 3500] K and at
T_common, for every synthetic mechanism: the exponent feeds an FP32
exponential whose own input split is 2^-48 relative, so 1e-10 absolute
leaves two orders of magnitude between this error and anything a rate
notices.  The GPU parity tests check the kernel itself."""
import numpy as np
import pytest

f32 = np.float32


def _split(v):
    h = v.astype(np.float32)
    return h, (v - h.astype(np.float64)).astype(np.float32)


def _fmaf(a, b, c):
    # float32 a * b is exact in float64; one rounding of the sum to float32
    # (a double rounding in rare cases: far below the bound tested)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def _ff_fma(a, b, c):
    """a * b + c on (head, tail) float32 pairs, as ff_fma in the kernel."""
    p = (a[0] * b[0]).astype(np.float32)
    e = _fmaf(a[0], b[0], -p)
    e = _fmaf(a[0], b[1], e)
    e = _fmaf(a[1], b[0], e)
    s = (p + c[0]).astype(np.float32)
    bb = (s - p).astype(np.float32)
    err = ((p - (s - bb)) + (c[0] - bb)).astype(np.float32)
    return s, (err + (e + c[1])).astype(np.float32)


@pytest.mark.parametrize("name", ["small", "gri53", "large561"])
def test_float_float_kc_exponent_matches_fp64(name, synth_mech):
    t = synth_mech(name).tables
    NREV = int(t["dims"][2])
    kptr = np.asarray(t["kc_ptr"])
    assert np.all(np.diff(kptr[: NREV + 1]) <= 1)  # one T_common group: the KcMix path
    lo = np.asarray(t["kc_lo"]).reshape(-1, 7)
    hi = np.asarray(t["kc_hi"]).reshape(-1, 7)
    tmid = np.asarray(t["kc_tmid"])
    lp = np.log(np.asarray(t["kc_pref"][:NREV]))
    rng = np.random.default_rng(7)
    T = np.concatenate([rng.uniform(300.0, 3500.0, 64), np.unique(tmid),
                        np.nextafter(np.unique(tmid), 0.0), np.nextafter(np.unique(tmid), 1e9)])
    logT, invT = np.log(T), 1.0 / T
    Tff, lff, iff = _split(T), _split(logT), _split(invT)
    worst = 0.0
    for j in range(NREV):
        if kptr[j + 1] == kptr[j]:
            continue
        g = kptr[j]
        c = np.where((T <= tmid[g])[:, None], lo[g][None, :], hi[g][None, :])
        c[:, 0] += lp[j]
        h = ((c[:, 5] * T + c[:, 4]) * T + c[:, 3]) * T + c[:, 2]
        ref = h * T + c[:, 0] + c[:, 1] * logT - c[:, 6] * invT
        C = [_split(c[:, q]) for q in range(6)] + [_split(-c[:, 6])]
        v = C[5]
        for q in (4, 3, 2, 0):
            v = _ff_fma(v, Tff, C[q])
        v = _ff_fma(C[1], lff, v)
        v = _ff_fma(C[6], iff, v)
        got = v[0].astype(np.float64) + v[1].astype(np.float64)
        worst = max(worst, float(np.max(np.abs(got - ref))))
    assert worst < 1e-10, worst
