"""The reference's per-state functions on the host (CPU only).

libcrs evaluates eval_conc / eval_rxn_rates / get_rxn_pres_mod /
eval_spec_rates, the thermo utilities and dydt (rate_subs.py:287-290,
761-763, 1124-1127, 1297-1299, 1396-2067) for one state on the calling
thread, over the mechanism's host table image, in the reference's operation
order compiled without contraction.  They must equal the reference's
emitted C bit for bit (the golden vectors), be callable from many threads
at once, and need no GPU: the mechanism is loaded with crs_mech_load_host.
"""
import ctypes
import threading

import numpy as np
import pytest

from conftest import GOLDEN_CASES
from create_rate_subs_gb300 import _lib

dp = lambda a: a.ctypes.data_as(ctypes.c_void_p)


class HostMech(object):
    def __init__(self, mech):
        self.lib = _lib.load()
        self.h = ctypes.c_void_p()
        _lib.check(self.lib.crs_mech_load_host(mech.blob, len(mech.blob), ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.lib.crs_mech_free(self.h)
            self.h = ctypes.c_void_p()


def _dims(g):
    return tuple(int(x) for x in g["dims"])


def _arrays(g):
    """The fixture's arrays read once (an npz file reads lazily and is not
    safe to share between threads)."""
    return {k: g[k] for k in g.files}


def _state_outputs(lib, g, i, bound=None):
    """Every per-state function on golden state i.  bound = None: the
    reference signatures through the binding; else the crs_state_* calls
    on that handle."""
    N, R, NREV, NPM = _dims(g)
    T, P = float(g["T"][i]), float(g["P"][i])
    y = np.ascontiguousarray(g["Y"][: N - 1, i])
    conc = np.zeros(N)
    yN, mw, rho = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    fwd, rev, pm = np.zeros(R), np.zeros(max(NREV, 1)), np.zeros(max(NPM, 1))
    sp, dyN = np.zeros(max(N - 1, 1)), ctypes.c_double()
    F = np.ascontiguousarray(g["fwd"][:, i])
    Rr = np.ascontiguousarray(g["rev"][:, i]) if NREV else np.zeros(1)
    PMr = np.ascontiguousarray(g["pm"][:, i]) if NPM else np.zeros(1)
    th = {w: np.zeros(N) for w in "h u cv cp".split()}
    crho_c = np.zeros(N)
    cr = (ctypes.c_double(), ctypes.c_double(), ctypes.c_double())
    ys = np.ascontiguousarray(np.concatenate([[T], g["Y"][: N - 1, i]]))
    dy = np.zeros(N)
    if bound is None:
        lib.eval_conc(T, P, dp(y), ctypes.byref(yN), ctypes.byref(mw), ctypes.byref(rho),
                      dp(conc))
        lib.eval_rxn_rates(T, P, dp(conc), dp(fwd), dp(rev))
        lib.get_rxn_pres_mod(T, P, dp(conc), dp(pm))
        lib.eval_spec_rates(dp(F), dp(Rr), dp(PMr), dp(sp), ctypes.byref(dyN))
        for w, fn in (("h", lib.eval_h), ("u", lib.eval_u), ("cv", lib.eval_cv),
                      ("cp", lib.eval_cp)):
            fn(T, dp(th[w]))
        lib.eval_conc_rho(T, float(g["misc"][2, i]), dp(y), ctypes.byref(cr[0]),
                          ctypes.byref(cr[1]), ctypes.byref(cr[2]), dp(crho_c))
        lib.dydt(0.0, P, dp(ys), dp(dy))
    else:
        h = bound
        _lib.check(lib.crs_state_eval_conc(h, T, P, dp(y), ctypes.byref(yN), ctypes.byref(mw),
                                           ctypes.byref(rho), dp(conc)))
        _lib.check(lib.crs_state_eval_rxn_rates(h, T, P, dp(conc), dp(fwd), dp(rev)))
        _lib.check(lib.crs_state_get_rxn_pres_mod(h, T, P, dp(conc), dp(pm)))
        _lib.check(lib.crs_state_eval_spec_rates(h, dp(F), dp(Rr), dp(PMr), dp(sp),
                                                 ctypes.byref(dyN)))
        for j, w in enumerate("h u cv cp".split()):
            _lib.check(lib.crs_state_eval_thermo(h, j, T, dp(th[w])))
        _lib.check(lib.crs_state_eval_conc_rho(h, T, float(g["misc"][2, i]), dp(y),
                                               ctypes.byref(cr[0]), ctypes.byref(cr[1]),
                                               ctypes.byref(cr[2]), dp(crho_c)))
        _lib.check(lib.crs_state_dydt(h, 0, P, dp(ys), dp(dy)))
    wdot = np.concatenate([sp[: N - 1], [dyN.value]])
    return dict(conc=conc, misc=np.array([yN.value, mw.value, rho.value]), fwd=fwd,
                rev=rev[:NREV], pm=pm[:NPM], wdot=wdot, th=th, crho=crho_c,
                crho_misc=np.array([c.value for c in cr]), dydt=dy)


def _matches(g, i, o):
    """Names of the outputs of state i that differ from the golden vectors."""
    bad = []
    checks = [("conc", g["conc"][:, i]), ("misc", g["misc"][:, i]), ("fwd", g["fwd"][:, i]),
              ("rev", g["rev"][:, i]), ("pm", g["pm"][:, i]), ("wdot", g["wdot"][:, i]),
              ("crho", g["conc_rho"][:, i]), ("crho_misc", g["conc_rho_misc"][:, i]),
              ("dydt", g["dydt_conp"][:, i])]
    for k, ref in checks:
        if not np.array_equal(o[k], ref):
            bad.append(k)
    for w in ("h", "u", "cv", "cp"):
        if not np.array_equal(o["th"][w], g["thermo_" + w][:, i]):
            bad.append(w)
    return bad


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_reference_signatures_bitexact_vs_golden(case, golden):
    mech, g = golden(case)
    hm = HostMech(mech)
    lib = hm.lib
    _lib.check(lib.crs_bind(hm.h))
    try:
        for i in range(g["T"].shape[0]):
            bad = _matches(g, i, _state_outputs(lib, g, i))
            assert not bad, (case, i, bad)
    finally:
        lib.crs_bind(None)
        hm.close()


@pytest.mark.parametrize("case", ["gri53", "features"])
def test_constant_volume_dydt_equals_the_oracle(case, golden):
    """Constant volume (whose emitted text does not compile in the
    reference) against the oracle's restatement, bit for bit."""
    from oracle.oracle import Oracle
    mech, g = golden(case)
    hm = HostMech(mech)
    N = mech.n_species
    ys = np.concatenate([g["T"][None], g["Y"][: N - 1]], axis=0)
    rho = g["misc"][2]
    want = Oracle(mech.blob).dydt(rho, ys, conv=True)
    try:
        for i in range(g["T"].shape[0]):
            y = np.ascontiguousarray(ys[:, i])
            dy = np.zeros(N)
            _lib.check(hm.lib.crs_state_dydt(hm.h, 1, float(rho[i]), dp(y), dp(dy)))
            assert np.array_equal(dy, want[:, i]), (case, i)
    finally:
        hm.close()


@pytest.mark.parametrize("case", ["gri53", "features"])
def test_explicit_handle_calls_bitexact_vs_golden(case, golden):
    mech, g = golden(case)
    hm = HostMech(mech)
    try:
        for i in range(g["T"].shape[0]):
            bad = _matches(g, i, _state_outputs(hm.lib, g, i, bound=hm.h))
            assert not bad, (case, i, bad)
    finally:
        hm.close()


def test_eight_threads_at_once(golden):
    """Eight threads call the reference signatures on one process-wide
    binding at the same time (ctypes releases the interpreter lock during
    each call); every result stays bit-exact."""
    mech, g = golden("gri53")
    g = _arrays(g)
    hm = HostMech(mech)
    lib = hm.lib
    _lib.check(lib.crs_bind(hm.h))
    n = g["T"].shape[0]
    errors = []
    start = threading.Barrier(8)

    def work(tid):
        try:
            start.wait()
            for rep in range(4):
                for i in range(tid, n, 3):
                    bad = _matches(g, i, _state_outputs(lib, g, i))
                    if bad:
                        errors.append((tid, i, bad))
        except Exception as exc:  # reported below
            errors.append((tid, repr(exc)))

    ts = [threading.Thread(target=work, args=(k,)) for k in range(8)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    lib.crs_bind(None)
    hm.close()
    assert not errors, errors[:5]


def test_thread_bindings_are_per_thread(golden):
    """Two threads, each bound to its own mechanism with crs_bind_thread,
    evaluate concurrently and each gets its own mechanism's results."""
    cases = ("small", "features")
    loaded = {c: (golden(c)[0], _arrays(golden(c)[1])) for c in cases}
    hms = {c: HostMech(loaded[c][0]) for c in cases}
    lib = hms["small"].lib
    lib.crs_bind(None)
    errors = []

    def work(case):
        mech, g = loaded[case]
        try:
            _lib.check(lib.crs_bind_thread(hms[case].h))
            for i in range(min(g["T"].shape[0], 40)):
                bad = _matches(g, i, _state_outputs(lib, g, i))
                if bad:
                    errors.append((case, i, bad))
            lib.crs_bind_thread(None)
        except Exception as exc:
            errors.append((case, repr(exc)))

    ts = [threading.Thread(target=work, args=(c,)) for c in cases]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for hm in hms.values():
        hm.close()
    assert not errors, errors[:5]


def test_freed_mechanism_is_unbound(golden):
    """crs_mech_free removes the handle from the process-wide binding: a
    later call reports that no mechanism is bound instead of reading freed
    memory, and leaves its outputs untouched."""
    mech, g = golden("small")
    hm = HostMech(mech)
    lib = hm.lib
    _lib.check(lib.crs_bind(hm.h))
    hm.close()
    N, R, NREV, _ = _dims(g)
    C = np.ascontiguousarray(g["conc"][:, 0])
    fwd = np.full(R, 7.0)
    rev = np.full(max(NREV, 1), 7.0)
    lib.eval_rxn_rates(float(g["T"][0]), float(g["P"][0]), dp(C), dp(fwd), dp(rev))
    assert "no mechanism bound" in _lib.last_error()
    assert np.all(fwd == 7.0) and np.all(rev == 7.0)


def test_explicit_handle_argument_errors(golden):
    mech, _ = golden("small")
    hm = HostMech(mech)
    lib = hm.lib
    out = np.zeros(64)
    assert lib.crs_state_eval_rxn_rates(None, 1000.0, 1e5, dp(out), dp(out), dp(out)) == 1
    assert lib.crs_state_eval_rxn_rates(hm.h, 1000.0, 1e5, None, dp(out), dp(out)) == 1
    assert lib.crs_state_eval_thermo(hm.h, 7, 1000.0, dp(out)) == 1
    assert lib.crs_state_dydt(hm.h, 2, 1e5, dp(out), dp(out)) == 1
    hm.close()


def test_host_only_handle_refused_by_batched_calls(golden):
    """A mechanism loaded without a GPU has no device tables: the batched
    entry points refuse it before touching a device."""
    mech, _ = golden("small")
    hm = HostMech(mech)
    rc = hm.lib.crs_wdot(hm.h, 4, None, None, None, 4, None, 0, None)
    assert rc == 1 and "no device tables" in _lib.last_error()
    hm.close()


@pytest.mark.parametrize("name,n", [("gri53", 300), ("large561", 24)])
def test_host_functions_bitexact_vs_reference_build(name, n, synth_mech):
    """The per-state host functions (their padded-factor, signed-sum and
    grouped pres_mod paths) on fresh seeded states of the workload
    mechanisms, against the reference's own emitted C for the same states,
    every stage bit for bit."""
    from oracle.oracle import RefLib
    from create_rate_subs_gb300 import synth
    if not RefLib.available(name):
        pytest.skip("reference C not built here (python oracle/build_ref.py all %s)" % name)
    mech = synth_mech(name)
    N, R, NREV, NPM = mech.n_species, mech.n_reactions, mech.n_rev, mech.n_pdep
    T, P, Y = synth.make_states(N, n, seed=2024)
    want = RefLib(name).eval(T, P, Y)
    hm = HostMech(mech)
    lib = hm.lib
    try:
        for i in range(n):
            y = np.ascontiguousarray(Y[: N - 1, i])
            conc = np.zeros(N)
            yN, mw, rho = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
            fwd, rev, pm = np.zeros(R), np.zeros(max(NREV, 1)), np.zeros(max(NPM, 1))
            sp, dyN = np.zeros(N - 1), ctypes.c_double()
            h, Ti, Pi = hm.h, float(T[i]), float(P[i])
            _lib.check(lib.crs_state_eval_conc(h, Ti, Pi, dp(y), ctypes.byref(yN),
                                               ctypes.byref(mw), ctypes.byref(rho), dp(conc)))
            _lib.check(lib.crs_state_eval_rxn_rates(h, Ti, Pi, dp(conc), dp(fwd), dp(rev)))
            _lib.check(lib.crs_state_get_rxn_pres_mod(h, Ti, Pi, dp(conc), dp(pm)))
            _lib.check(lib.crs_state_eval_spec_rates(h, dp(fwd), dp(rev), dp(pm), dp(sp),
                                                     ctypes.byref(dyN)))
            assert np.array_equal(conc, want["conc"][:, i]), (name, i, "conc")
            assert np.array_equal(fwd, want["fwd"][:, i]), (name, i, "fwd")
            assert np.array_equal(rev[:NREV], want["rev"][:, i]), (name, i, "rev")
            assert np.array_equal(pm[:NPM], want["pm"][:, i]), (name, i, "pm")
            wdot = np.concatenate([sp, [dyN.value]])
            assert np.array_equal(wdot, want["wdot"][:, i]), (name, i, "wdot")
    finally:
        hm.close()
