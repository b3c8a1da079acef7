"""Dynamic state scheduling of the one-state-per-thread kernels.

The fp64 and mixed per-thread kernels hand states to warps from a counter
slot that each launch draws from its mechanism handle (256 slots) and that
the launch's last warp puts back to zero.  Which warp evaluates a state does
not change its arithmetic, so every launch must reproduce a one-shot result
bit for bit: many launches in a row (more than the slot count, so every slot
is reused), ragged and tiny batch sizes, and launches on two streams at once.
"""
import numpy as np
import pytest

from create_rate_subs_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def rs(synth_mech):
    from create_rate_subs_gb300.rates import RateSubs
    return RateSubs(synth_mech("gri53"))


def _states(rs, n, seed):
    N = rs.n_species
    T, P, Y = synth.make_states(N, n, seed=seed)
    return tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (T, P, Y[: N - 1]))


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_slots_reused_many_launches(rs, mode):
    n = 20011
    T, P, Y = _states(rs, n, 41)
    want = rs.wdot(T, P, Y, mode=mode).clone()
    out = torch.empty_like(want)
    sizes = [1, 31, 32, 33, 317, 1000, n]
    for it in range(300):               # > 256 slots: every slot is drawn again
        m = sizes[it % len(sizes)]
        out.fill_(float("nan"))
        rs.wdot(T[:m], P[:m], Y[:, :m], mode=mode, out=out[:, :m])
        if it % 37 == 0 or m == n:
            torch.cuda.synchronize()
            assert torch.equal(out[:, :m], want[:, :m]), (it, m)
    torch.cuda.synchronize()
    flags, bad = rs.status()
    assert flags == 0


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_two_streams_at_once(rs, mode):
    n = 1 << 16
    T, P, Y = _states(rs, n, 43)
    want = rs.wdot(T, P, Y, mode=mode).clone()
    outs = [torch.full_like(want, float("nan")) for _ in range(2)]
    streams = [torch.cuda.Stream() for _ in range(2)]
    torch.cuda.synchronize()
    for it in range(20):
        for s, o in zip(streams, outs):
            with torch.cuda.stream(s):
                rs.wdot(T, P, Y, mode=mode, out=o)
    torch.cuda.synchronize()
    for o in outs:
        assert torch.equal(o, want)


def test_inexact_nu_runs_the_warp_kernel(tmp_path):
    """A stoichiometric coefficient whose double has a nonzero low word
    (0.7) cannot use the compact nu lists of the mixed per-thread kernel:
    mixed_tps reports it as unsupported and mixed runs the warp kernel,
    within the mixed tolerance of the oracle."""
    from conftest import load_golden
    from create_rate_subs_gb300 import _lib
    from create_rate_subs_gb300.mechanism import Mechanism
    from create_rate_subs_gb300.rates import RateSubs
    from oracle.oracle import Oracle, gross_scale, wdot_errors
    _, g = load_golden("features")
    text = str(g["mech_text"])
    assert "0.5H2+0.5O2=>OH" in text
    mp, tp = tmp_path / "mech.inp", tmp_path / "therm.dat"
    mp.write_text(text.replace("0.5H2+0.5O2=>OH", "0.7H2+0.3O2=>OH"))
    tp.write_text(str(g["therm_text"]))
    mech = Mechanism.from_chemkin(str(mp), str(tp))
    rs = RateSubs(mech)
    n = 2000
    T, P, Y = synth.make_states(mech.n_species, n, seed=7)
    ref = Oracle(mech.blob).eval(T, P, Y)
    G = gross_scale(mech.tables, ref["fwd"], ref["rev"], ref["pm"])
    dT, dP, dY = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (T, P, Y))
    with pytest.raises(_lib.CRSError) as ei:
        rs.wdot(dT, dP, dY, "mixed_tps")
    assert ei.value.code == 4
    for mode in ("mixed", "fp64"):
        w = rs.wdot(dT, dP, dY, mode).cpu().numpy()
        tol = 1e-6 if mode == "mixed" else 1e-12
        assert wdot_errors(w, ref["wdot"], G)["scaled"] <= tol, mode
