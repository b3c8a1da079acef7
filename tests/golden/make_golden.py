"""Regenerate the golden vectors in tests/golden/ from the reference itself.

For each case below this script writes the mechanism (synthetic, or the
hand-written features.inp), has the reference's own generator emit C for it
(oracle/build_ref.py: a Python 3-patched copy of the reference in a scratch
directory), compiles that C with -O2 -ffp-contract=off and evaluates it on
seeded states plus edge states: every stage of the rates path, the thermo
utilities (eval_h/u/cv/cp, eval_conc_rho) and the constant-pressure dydt
(compiled with -DCONP).  The outputs are stored as
<case>.npz together with the mechanism text, so that the tests can pin the
front end and the oracle without the reference checkout.

Run from the repository root:  python tests/golden/make_golden.py [CASE ...]
(needs the reference checkout; oracle/build_ref.py says where it is looked
for and how to point elsewhere).
"""

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from create_rate_subs_gb300 import chem, synth  # noqa: E402
from oracle import build_ref  # noqa: E402
from oracle.oracle import RefDydt, RefLib  # noqa: E402

# case -> (mechanism source, last_spec, n random states, state seed)
CASES = {
    # the small configuration's 1024 seeded states (+ the edge states)
    "small": ("small", None, 1024, 11),
    "gri53": ("gri53", None, 48, 12),
    "features": ("features", None, 64, 13),
    "features_lastAR": ("features", "AR", 32, 14),
}

_FEATURE_COMPS = {  # name -> (C, H, O, N, Ar), T_common
    "H2": ((0, 2, 0, 0, 0), 1000.0), "O2": ((0, 0, 2, 0, 0), 1000.0),
    "H": ((0, 1, 0, 0, 0), 1000.0), "O": ((0, 0, 1, 0, 0), 1000.0),
    "OH": ((0, 1, 1, 0, 0), 1387.0), "H2O": ((0, 2, 1, 0, 0), 1200.0),
    "N2": ((0, 0, 0, 2, 0), 1000.0), "HO2": ((0, 1, 2, 0, 0), 1200.0),
    "H2O2": ((0, 2, 2, 0, 0), 1000.0), "AR": ((0, 0, 0, 0, 1), 1000.0),
}


def features_thermo(path):
    """Thermo for features.inp: seeded NASA-7 fits, three common
    temperatures (1000, 1200, 1387 K) so reactions get several Kc groups."""
    rng = np.random.default_rng(77)
    out = ["THERMO", "   300.000  1000.000  5000.000"]
    for name, (comp, tmid) in _FEATURE_COMPS.items():
        lo, hi = synth._fit_thermo(rng)
        entry = synth._thermo_entry(name, comp, lo, hi).split("\n")
        l1 = entry[0][:65] + "%8.2f" % tmid
        entry[0] = l1.ljust(79) + "1"
        out.extend(entry)
    out.append("END")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def edge_states(n_species, tmids):
    """States that sit on branch boundaries: T exactly at each T_common
    (the '<=' branch), very low/high T and P, zero and one-hot mass
    fractions, and a mass-fraction sum above one (negative bath gas)."""
    T, P, Y = [], [], []
    base = np.full(n_species, 1.0 / n_species)
    for t in sorted(set(tmids)) + [300.0, 3500.0]:
        T.append(t); P.append(chem.PA); Y.append(base.copy())
    for p in (1e-3 * chem.PA, 1e3 * chem.PA):
        T.append(1500.0); P.append(p); Y.append(base.copy())
    y = base.copy(); y[: n_species // 2] = 0.0; y /= y.sum()
    T.append(1800.0); P.append(chem.PA); Y.append(y)
    y = np.zeros(n_species); y[-1] = 1.0
    T.append(1300.0); P.append(5 * chem.PA); Y.append(y)
    y = np.zeros(n_species); y[0] = 1.0
    T.append(2200.0); P.append(2 * chem.PA); Y.append(y)
    y = base.copy() * 1.3
    T.append(1100.0); P.append(chem.PA); Y.append(y)
    return np.array(T), np.array(P), np.array(Y).T.copy()


def make_case(case):
    src, last, n, seed = CASES[case]
    mdir = os.path.join(REPO, "oracle", "_ref", "_golden_mech", case)
    os.makedirs(mdir, exist_ok=True)
    if src == "features":
        mp = os.path.join(HERE, "features.inp")
        tp = os.path.join(HERE, "features_therm.dat")
        if not os.path.exists(tp):
            features_thermo(tp)
    else:
        mp, tp = synth.write_mechanism(src, mdir)
    name = "golden_" + case
    build_ref.generate(name, mp, tp, last_spec=last)
    build_ref.compile_ref(name)
    ref = RefLib(name)
    N = ref.dims[0]
    with open(os.path.join(build_ref.ref_dir(name), "header.h")) as f:
        names = re.findall(r"^ \* (\d+) (\S+)$", f.read(), re.M)
    names = [x[1] for x in names]
    T, P, Y = synth.make_states(N, n, seed)
    with open(tp) as f:
        tm = sorted({float(l[65:73]) for l in f if l.rstrip().endswith("1")
                     and len(l) > 73 and l[65:73].strip()})
    Te, Pe, Ye = edge_states(N, tm)
    T = np.concatenate([T, Te])
    P = np.concatenate([P, Pe])
    Y = np.concatenate([Y, Ye], axis=1)
    out = ref.eval(T, P, Y)
    # the emitted thermo utilities and constant-pressure dydt on the same
    # states (y = [T, Y_0..Y_{N-2}]); eval_conc_rho at the density that
    # eval_conc returned
    refd = RefDydt(name)
    for w in ("h", "u", "cv", "cp"):
        out["thermo_" + w] = refd.thermo(w, T)
    out["conc_rho_misc"], out["conc_rho"] = refd.conc_rho(T, out["misc"][2], Y)
    out["dydt_conp"] = refd.dydt(P, np.concatenate([T[None], Y[: N - 1]], axis=0))
    with open(mp) as f:
        mech_text = f.read()
    with open(tp) as f:
        therm_text = f.read()
    np.savez_compressed(
        os.path.join(HERE, case + ".npz"),
        mech_text=np.array(mech_text), therm_text=np.array(therm_text),
        last_spec=np.array(last or ""), species=np.array(names),
        dims=np.array(ref.dims, dtype=np.int64), T=T, P=P, Y=Y, **out)
    print(case, "dims", ref.dims, "states", T.shape[0])


if __name__ == "__main__":
    for c in (sys.argv[1:] or CASES):
        make_case(c)
