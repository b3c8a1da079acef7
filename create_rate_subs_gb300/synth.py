"""Seeded synthetic mechanisms and thermochemical states.

The reference ships no mechanism files, so every workload here is generated:
Chemkin text (mechanism + NASA-7 thermo) that the front end -- and the
reference's own generator -- read like any real mechanism, plus random
states in structure-of-arrays layout.

Species: random C/H/O/N formulas (always N2 and AR, so N2 becomes the bath
gas by the reference's default rule).  Thermo: two-range NASA-7 fits of
cp/R = a + b*tanh((T-c)/d) with a~U[2.5,4], b~U[0.5,3], c~U[800,1500] K,
d~U[300,800] K, cp continuous at 1000 K, h298/R~U[-3e4,3e4] K and
s298/R~U[20,40] fixing the integration constants; H and S are continuous at
1000 K.  Reactions: atom-balanced, 1-3 species a side, A log-uniform in
1e6-1e16 (cm-mol-s), beta~U[-2,2], Ea~U[0,50000] cal/mol.  States:
T~U[800,2800] K, P log-uniform in [1,50] atm, Y~Dirichlet(0.5).
"""

import math
from collections import defaultdict

import numpy as np

from . import chem

__all__ = ["CONFIGS", "make_mechanism", "write_mechanism", "make_states"]

# name -> generator arguments for the mechanisms of the workloads.
CONFIGS = {
    # 10 species / 27 reactions over H/O/N/Ar: 5 three-body, 3 Troe.
    "small": dict(n_species=10, n_reactions=27, elements=("H", "O", "N", "AR"),
                  n_thd=5, n_troe=3, n_lind=0, n_sri=0, n_irrev=0, seed=1001),
    # 53 species / 325 reactions over C/H/O/N/Ar.
    "gri53": dict(n_species=53, n_reactions=325,
                  elements=("C", "H", "O", "N", "AR"),
                  n_thd=30, n_troe=25, n_lind=3, n_sri=2, n_irrev=20, seed=2002),
    # 561 species / 2539 reactions: 10% three-body, 5% Troe.
    "large561": dict(n_species=561, n_reactions=2539,
                     elements=("C", "H", "O", "N", "AR"),
                     n_thd=254, n_troe=127, n_lind=0, n_sri=0, n_irrev=156,
                     seed=4004),
}

_ELEM_ORDER = ("C", "H", "O", "N", "AR")
_WT = chem.get_elem_wt()


def _formula(comp):
    parts = []
    for e, n in zip(_ELEM_ORDER, comp):
        if n == 0:
            continue
        parts.append(e if n == 1 else "%s%d" % (e, n))
    return "".join(parts)


def _species_pool(elements, n_species, rng):
    """Unique compositions (C, H, O, N, Ar), ending with N2 and AR.

    A hydrogen/oxygen (and carbon/nitrogen) core is grown by adding random
    sums of two existing species, so that every grown species has at least
    one association channel and elementary exchanges stay plentiful.
    """
    has = set(elements)
    fixed = [(0, 0, 0, 2, 0)]
    if "AR" in has:
        fixed.append((0, 0, 0, 0, 1))
    core = [(0, 1, 0, 0, 0), (0, 0, 1, 0, 0), (0, 1, 1, 0, 0),
            (0, 2, 0, 0, 0), (0, 0, 2, 0, 0), (0, 2, 1, 0, 0),
            (0, 1, 2, 0, 0), (0, 2, 2, 0, 0), (0, 0, 0, 1, 0),
            (0, 0, 1, 1, 0), (0, 1, 0, 1, 0), (0, 0, 2, 1, 0),
            (0, 0, 1, 2, 0), (0, 1, 1, 1, 0), (0, 2, 0, 1, 0)]
    if "C" in has:
        core = core[:8] + [(1, 0, 0, 0, 0), (1, 1, 0, 0, 0), (1, 2, 0, 0, 0),
                           (1, 3, 0, 0, 0), (1, 4, 0, 0, 0), (1, 0, 1, 0, 0),
                           (1, 0, 2, 0, 0), (1, 1, 1, 0, 0), (1, 2, 1, 0, 0)] + core[8:]
    need = n_species - len(fixed)
    comps = core[:need]
    if len(comps) == need:
        return comps + fixed
    lim = (6, 12, 4, 2) if n_species > 300 else (3, 8, 3, 2)
    if "C" not in has:
        lim = (0,) + lim[1:]
    have = set(comps) | set(fixed)
    while len(comps) < need:
        i, j = rng.integers(len(comps)), rng.integers(len(comps))
        c = tuple(a + b for a, b in zip(comps[i], comps[j]))
        if c in have or any(c[k] > lim[k] for k in range(4)) or sum(c) > 12:
            continue
        have.add(c)
        comps.append(c)
    return comps + fixed


def _fit_thermo(rng):
    """NASA-7 (lo, hi) for one species; see the module docstring."""
    a = rng.uniform(2.5, 4.0)
    b = rng.uniform(0.5, 3.0)
    c = rng.uniform(800.0, 1500.0)
    d = rng.uniform(300.0, 800.0)
    h298 = rng.uniform(-3.0e4, 3.0e4)
    s298 = rng.uniform(20.0, 40.0)
    cp = lambda T: a + b * np.tanh((T - c) / d)
    # low range: free quartic fit in tau = T/1000
    Tl = np.linspace(300.0, 1000.0, 71)
    V = np.vander(Tl / 1000.0, 5, increasing=True)
    al, *_ = np.linalg.lstsq(V, cp(Tl), rcond=None)
    lo5 = al / 1000.0 ** np.arange(5)
    cp1000 = float(np.sum(al))
    # high range: cp_hi(T) = cp1000 + sum_j c_j (tau^j - 1), continuous at 1000 K
    Th = np.linspace(1000.0, 5000.0, 161)
    tau = Th / 1000.0
    W = np.stack([tau ** j - 1.0 for j in range(1, 5)], axis=1)
    cj, *_ = np.linalg.lstsq(W, cp(Th) - cp1000, rcond=None)
    ah = np.concatenate([[cp1000 - cj.sum()], cj])
    hi5 = ah / 1000.0 ** np.arange(5)

    def h_poly(p, T):
        return (p[0] * T + p[1] * T ** 2 / 2 + p[2] * T ** 3 / 3
                + p[3] * T ** 4 / 4 + p[4] * T ** 5 / 5)

    def s_poly(p, T):
        return (p[0] * math.log(T) + p[1] * T + p[2] * T ** 2 / 2
                + p[3] * T ** 3 / 3 + p[4] * T ** 4 / 4)

    lo = np.zeros(7)
    hi = np.zeros(7)
    lo[:5] = lo5
    hi[:5] = hi5
    lo[5] = h298 - h_poly(lo5, 298.15)
    lo[6] = s298 - s_poly(lo5, 298.15)
    hi[5] = (h_poly(lo5, 1000.0) + lo[5]) - h_poly(hi5, 1000.0)
    hi[6] = (s_poly(lo5, 1000.0) + lo[6]) - s_poly(hi5, 1000.0)
    return lo, hi


def _thermo_entry(name, comp, lo, hi):
    elems = [(e, n) for e, n in zip(_ELEM_ORDER, comp) if n]
    field = "".join("%-2s%3d" % (e, n) for e, n in elems)
    field = field.ljust(20)
    l1 = "%-18s%-6s%s%s%10.3f%10.3f%8.2f" % (name, "SYNTH", field, "G",
                                              300.0, 5000.0, 1000.0)
    l1 = l1.ljust(79) + "1"
    f = lambda x: "%15.8E" % x
    l2 = "".join(f(x) for x in hi[0:5]).ljust(79) + "2"
    l3 = "".join(f(x) for x in (hi[5], hi[6], lo[0], lo[1], lo[2])).ljust(79) + "3"
    l4 = "".join(f(x) for x in (lo[3], lo[4], lo[5], lo[6])).ljust(79) + "4"
    return "\n".join([l1, l2, l3, l4])


def _side(names):
    counts = defaultdict(int)
    for n in names:
        counts[n] += 1
    out = []
    for n in sorted(counts):
        out.append(n if counts[n] == 1 else "%d%s" % (counts[n], n))
    return "+".join(out)


def make_mechanism(n_species, n_reactions, elements, n_thd, n_troe, n_lind,
                   n_sri, n_irrev, seed):
    """Return (mech_text, thermo_text) for a seeded synthetic mechanism."""
    rng = np.random.default_rng(seed)
    comps = _species_pool(elements, n_species, rng)
    names = [_formula(cmp) for cmp in comps]
    vec = [np.array(cmp, dtype=np.int64) for cmp in comps]
    key = lambda v: tuple(int(x) for x in v)
    singles = defaultdict(list)
    for i, v in enumerate(vec):
        singles[key(v)].append(i)
    pairs = defaultdict(list)
    reactive = [i for i in range(len(comps)) if names[i] not in ("N2", "AR")]
    for ii, i in enumerate(reactive):
        for j in reactive[ii:]:
            pairs[key(vec[i] + vec[j])].append((i, j))

    seen = set()
    rxns = []   # (lhs idx tuple, rhs idx tuple)

    def canon(l, r):
        return (tuple(sorted(l)), tuple(sorted(r)))

    def try_add(l, r):
        if not l or not r:
            return False
        c = canon(l, r)
        if c[0] == c[1] or c in seen or (c[1], c[0]) in seen:
            return False
        seen.add(c)
        rxns.append(c)
        return True

    def assoc():
        """A + B <=> AB (for three-body and fall-off reactions)."""
        for _ in range(2000):
            k = reactive[rng.integers(len(reactive))]
            cands = pairs.get(key(vec[k]), [])
            if not cands:
                continue
            i, j = cands[rng.integers(len(cands))]
            if rng.random() < 0.5:
                if try_add((i, j), (k,)):
                    return True
            elif try_add((k,), (i, j)):
                return True
        raise RuntimeError("could not place an association reaction")

    def elementary():
        for _ in range(5000):
            nl = 2 if rng.random() < 0.85 else int(rng.choice([1, 3]))
            l = tuple(reactive[rng.integers(len(reactive))] for _ in range(nl))
            tot = sum((vec[i] for i in l), np.zeros(5, dtype=np.int64))
            mode = rng.random()
            if mode < 0.7:
                cands = pairs.get(key(tot), [])
                if cands:
                    r = cands[rng.integers(len(cands))]
                    if try_add(l, r):
                        return True
            elif mode < 0.85:
                cands = singles.get(key(tot), [])
                cands = [c for c in cands if c in reactive]
                if cands and try_add(l, (cands[rng.integers(len(cands))],)):
                    return True
            else:
                p = reactive[rng.integers(len(reactive))]
                rem = tot - vec[p]
                if (rem < 0).any():
                    continue
                cands = pairs.get(key(rem), [])
                if cands:
                    q = cands[rng.integers(len(cands))]
                    if try_add(l, (p,) + tuple(q)):
                        return True
        raise RuntimeError("could not place an elementary reaction")

    kinds = (["thd"] * n_thd + ["troe"] * n_troe + ["lind"] * n_lind
             + ["sri"] * n_sri)
    n_elem = n_reactions - len(kinds)
    kinds += ["elem"] * n_elem
    order = rng.permutation(len(kinds))
    kinds = [kinds[i] for i in order]
    elem_slots = [i for i, k in enumerate(kinds) if k == "elem"]
    irrev = set(rng.choice(elem_slots, size=n_irrev, replace=False).tolist()) if n_irrev else set()

    lines = []
    bath = [i for i in range(len(comps))]
    for idx, kind in enumerate(kinds):
        if kind == "elem":
            elementary()
        else:
            assoc()
        l, r = rxns[-1]
        ln, rn = [names[i] for i in l], [names[i] for i in r]
        A = 10.0 ** rng.uniform(6.0, 16.0)
        b = rng.uniform(-2.0, 2.0)
        E = rng.uniform(0.0, 50000.0)
        arrow = "=>" if idx in irrev else "<=>"
        if kind == "elem":
            eq = _side(ln) + arrow + _side(rn)
        elif kind == "thd":
            eq = _side(ln) + "+M" + arrow + _side(rn) + "+M"
            A /= 10.0 ** rng.uniform(0.0, 2.0)
        else:
            eq = _side(ln) + "(+M)" + arrow + _side(rn) + "(+M)"
        lines.append("%-40s %13.6E %8.3f %10.1f" % (eq, A, b, E))
        if kind in ("thd", "troe", "lind", "sri"):
            if kind != "thd":
                A0 = A * 10.0 ** rng.uniform(1.0, 7.0)
                b0 = rng.uniform(-2.0, 2.0)
                E0 = rng.uniform(0.0, 25000.0)
                lines.append("    LOW / %13.6E %8.3f %10.1f /" % (A0, b0, E0))
            if kind == "troe":
                alpha = rng.uniform(0.1, 0.9)
                t3 = rng.uniform(50.0, 500.0)
                t1 = rng.uniform(500.0, 5000.0)
                if rng.random() < 0.5:
                    t2 = rng.uniform(2000.0, 10000.0)
                    lines.append("    TROE / %.4f %.2f %.2f %.2f /" % (alpha, t3, t1, t2))
                else:
                    lines.append("    TROE / %.4f %.2f %.2f /" % (alpha, t3, t1))
            elif kind == "sri":
                a = rng.uniform(0.1, 2.0)
                bb = rng.uniform(100.0, 1000.0)
                c = rng.uniform(500.0, 3000.0)
                if rng.random() < 0.5:
                    d = rng.uniform(0.5, 2.0)
                    e = rng.uniform(-0.5, 0.5)
                    lines.append("    SRI / %.4f %.2f %.2f %.4f %.4f /" % (a, bb, c, d, e))
                else:
                    lines.append("    SRI / %.4f %.2f %.2f /" % (a, bb, c))
            n_eff = int(rng.integers(2, min(7, len(bath)) + 1))
            who = rng.choice(bath, size=n_eff, replace=False)
            effs = " ".join("%s/%.2f/" % (names[i], rng.uniform(0.5, 12.0))
                            for i in sorted(who))
            lines.append("    " + effs)

    therm = ["THERMO", "   300.000  1000.000  5000.000"]
    for name, cmp in zip(names, comps):
        lo, hi = _fit_thermo(rng)
        therm.append(_thermo_entry(name, cmp, lo, hi))
    therm.append("END")

    used_elems = [e for e in _ELEM_ORDER if e in elements]
    mech = ["ELEMENTS", " ".join(used_elems), "END", "SPECIES"]
    for k in range(0, len(names), 8):
        mech.append(" ".join(names[k:k + 8]))
    mech += ["END", "REACTIONS"] + lines + ["END", ""]
    return "\n".join(mech), "\n".join(therm) + "\n"


def write_mechanism(config, directory):
    """Write <config>.inp and <config>_therm.dat into ``directory``;
    return (mech_path, therm_path)."""
    import os
    args = CONFIGS[config] if isinstance(config, str) else config
    name = config if isinstance(config, str) else "mech"
    mech, therm = make_mechanism(**args)
    os.makedirs(directory, exist_ok=True)
    mp = os.path.join(directory, name + ".inp")
    tp = os.path.join(directory, name + "_therm.dat")
    with open(mp, "w") as f:
        f.write(mech)
    with open(tp, "w") as f:
        f.write(therm)
    return mp, tp


def make_states(n_species, n_states, seed, t_range=(800.0, 2800.0),
                p_atm=(1.0, 50.0)):
    """(T[n], P[n] in Pa, Y[n_species, n]) in structure-of-arrays layout.

    T ~ U[t_range], P log-uniform over ``p_atm`` atmospheres, each state's
    mass fractions ~ Dirichlet(0.5).  Row ``n_species-1`` of Y is the bath
    gas; the evaluation reads rows 0..n_species-2 and infers the last.
    """
    rng = np.random.default_rng(seed)
    T = rng.uniform(t_range[0], t_range[1], n_states)
    P = np.exp(rng.uniform(math.log(p_atm[0]), math.log(p_atm[1]), n_states)) * chem.PA
    g = rng.standard_gamma(0.5, size=(n_species, n_states))
    Y = g / g.sum(axis=0, keepdims=True)
    return T, P, np.ascontiguousarray(Y)
