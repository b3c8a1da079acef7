"""Chemkin mechanism and NASA-7 thermo reader.

A from-scratch reader with the semantics of create_rate_subs'
``mech_interpret.read_mech`` / ``read_thermo`` (mech_interpret.py:52-712 and
715-863): the same sections, reaction syntax, auxiliary keywords and unit
conversions, so that the parsed records (and hence the tables built from
them) are the ones the reference would print into its emitted code.

Behaviour that is deliberately different (none of it changes the records of
a well-formed mechanism):

* errors raise :class:`MechanismError` instead of printing and calling
  ``sys.exit(1)`` (mech_interpret.py:147-155, 660-664, 700-710);
* a thermo file that ends without ``END`` before every species was found
  stops at end of file (the reference loops forever there,
  mech_interpret.py:776-782);
* atomic-weight overrides in ``ELEMENTS`` apply to this parse only (the
  reference mutates a module-level dict, mech_interpret.py:49, 184-186);
* the REV split locates the reaction by identity rather than by attribute
  equality (mech_interpret.py:677).
"""

import copy
import math
import re

import numpy as np

from . import chem

__all__ = ["read_mech", "read_thermo", "MechanismError",
           "act_energy_fact", "pre_units", "act_energy_units"]


class MechanismError(ValueError):
    """A mechanism or thermo file that cannot be interpreted."""


# Units accepted on the REACTIONS line (mech_interpret.py:30-36).
pre_units = ["moles", "molecules"]
act_energy_units = ["kelvins", "evolts", "cal/mole", "joules/kmole",
                    "kcal/mole", "joules/mole", "kjoules/mole"]

# Activation energy -> activation temperature [K] (mech_interpret.py:39-46).
act_energy_fact = {
    "kelvins": 1.0,
    "evolts": 11595.,
    "cal/mole": 4.184 / chem.RU_JOUL,
    "kcal/mole": 4184. / chem.RU_JOUL,
    "joules/mole": 1. / chem.RU_JOUL,
    "kjoules/mole": 1000.0 / chem.RU_JOUL,
    "joules/kmole": 1. / (chem.RU_JOUL * 1000.),
}

_BLANK = re.compile(r"^\s*$")
_COMMENT = re.compile(r"^\s*!")

# Three-letter prefixes of auxiliary reaction lines
# (mech_interpret.py:467-652); anything else is an efficiency list.
_AUX = ("dup", "rev", "low", "hig", "tro", "sri", "che", "pch", "tch", "plo")


def _skip(line):
    return bool(_BLANK.search(line) or _COMMENT.search(line))


def _coeffs(line):
    """Numbers of an auxiliary line 'KEY / a b c /' (slashes, commas)."""
    return line.replace("/", " ").replace(",", " ").split()


def _pull_falloff_marker(side):
    """Strip a '(+M)' / '(+SP)' marker from one side of an equation.

    Returns (side_without_marker, found, species_or_M).  Parentheses that
    do not open with '+' belong to species names and are skipped, as are
    literal '(+)' groups (mech_interpret.py:247-283).
    """
    rest = side
    while "(" in rest:
        i1 = rest.find("(")
        i2 = rest.find(")")
        inner = rest[i1 + 1:i2].strip()
        if inner == "+":
            rest = rest[i2 + 1:]
        elif inner[:1] == "+":
            who = rest[i1 + 1:i2].replace("+", " ").strip()
            off = side.find(rest)
            return side[:off + i1] + side[off + i2 + 1:], True, who
        else:
            rest = rest[i2 + 1:]
    return side, False, ""


def _split_side(side):
    """Split one side on '+' into stripped terms (mech_interpret.py:285-309).

    Empty pieces mean a species name ended in '+'; a piece ending in '('
    followed by one starting with ')' is a species with '(+)' in its name.
    """
    parts = side.split("+")
    while "" in parts:
        k = parts.index("")
        parts[k - 1] = parts[k - 1] + "+"
        del parts[k]
    k = 0
    while k < len(parts) - 1:
        if parts[k].endswith("(") and parts[k + 1].startswith(")"):
            parts[k] = parts[k] + "+" + parts[k + 1]
            del parts[k + 1]
        k += 1
    return parts


def _side_species(side):
    """Parse one equation side -> (names, nus, has_M) (mech_interpret.py:311-339).

    A leading number is the stoichiometric coefficient: int unless it
    contains '.', in which case float.  Repeated species are merged.
    """
    names, nus, has_m = [], [], False
    for term in _split_side(side):
        term = term.strip()
        if term[:1].isdigit():
            i = 0
            for i in range(len(term)):
                if term[i:i + 1].isalpha():
                    break
            num = term[:i]
            nu = float(num) if "." in num else int(num)
            term = term[i:].strip()
        else:
            nu = 1
        if term.lower() == "m":
            has_m = True
            continue
        if term in names:
            nus[names.index(term)] += nu
        else:
            names.append(term)
            nus.append(nu)
    return names, nus, has_m


def _parse_reaction(line, units_A, units_E):
    """One reaction line -> ReacInfo (mech_interpret.py:199-465)."""
    toks = line.split()
    if len(toks) < 4:
        raise MechanismError("reaction line needs an equation and A, b, E: "
                             + line)
    try:
        A = float(toks[-3])
        b = float(toks[-2])
        E = float(toks[-1])
    except ValueError:
        raise MechanismError("bad Arrhenius coefficients on: " + line)
    # The equation ends where the A literal first occurs (the reference
    # uses line.index of that token).
    eq = line[:line.index(toks[-3])].strip()

    if "<=>" in eq:
        k = eq.index("<=>")
        rev, lhs, rhs = True, eq[:k].strip(), eq[k + 3:].strip()
    elif "=>" in eq:
        k = eq.index("=>")
        rev, lhs, rhs = False, eq[:k].strip(), eq[k + 2:].strip()
    else:
        k = eq.index("=")
        rev, lhs, rhs = True, eq[:k].strip(), eq[k + 1:].strip()

    thd = pdep = False
    pdep_sp = ""
    for which in (0, 1):
        side = lhs if which == 0 else rhs
        side, found, who = _pull_falloff_marker(side)
        if found:
            pdep = True
            if who.lower() == "m":
                thd, pdep_sp = True, ""
            else:
                pdep_sp = who
        if which == 0:
            lhs = side
        else:
            rhs = side

    reac, reac_nu, m1 = _side_species(lhs)
    prod, prod_nu, m2 = _side_species(rhs)
    thd = thd or m1 or m2
    # '(+M)' fall-off is not a '+M' third-body reaction (mech_interpret.py:436-439).
    if pdep:
        thd = False

    E *= act_energy_fact[units_E]
    if units_A == "moles":
        order = sum(reac_nu)
        if thd:
            A /= 1000. ** order
        else:
            A /= 1000. ** (order - 1.)

    rxn = chem.ReacInfo(rev, reac, reac_nu, prod, prod_nu, A, b, E)
    rxn.thd_body = thd
    rxn.pdep = pdep
    if pdep:
        rxn.pdep_sp = pdep_sp
    return rxn


def _parse_aux(line, rxn, units_A, units_E, state):
    """Auxiliary line for the last reaction (mech_interpret.py:467-652)."""
    key = line[0:3].lower()
    if key == "dup":
        rxn.dup = True
    elif key in ("rev", "low", "hig"):
        t = _coeffs(line)
        p1, p2, p3 = float(t[1]), float(t[2]), float(t[3])
        p3 *= act_energy_fact[units_E]
        if key == "rev":
            if units_A == "moles":
                order = sum(rxn.prod_nu)
                p1 /= 1000. ** order if rxn.thd_body else 1000. ** (order - 1.)
            if p1 != 0.0:
                rxn.rev_par.extend([p1, p2, p3])
            else:
                rxn.rev = False
        elif key == "low":
            if units_A == "moles":
                p1 /= 1000. ** sum(rxn.reac_nu)
            rxn.low.extend([p1, p2, p3])
        else:
            if units_A == "moles":
                p1 /= 1000. ** (sum(rxn.reac_nu) - 2.)
            rxn.high.extend([p1, p2, p3])
    elif key == "tro":
        t = _coeffs(line)
        rxn.troe = True
        rxn.troe_par.extend(float(x) for x in t[1:4])
        if len(t) > 4:
            rxn.troe_par.append(float(t[4]))
    elif key == "sri":
        t = _coeffs(line)
        rxn.sri = True
        rxn.sri_par.extend(float(x) for x in t[1:4])
        if len(t) > 4:
            rxn.sri_par.extend([float(t[4]), float(t[5])])
    elif key == "che":
        rxn.cheb = True
        t = line.replace("/", " ").split()
        if state["cheb_open"]:
            rxn.cheb_par.extend(float(x) for x in t[1:])
        else:
            state["cheb_open"] = True
            rxn.pdep = False
            rxn.cheb_n_temp = int(t[1])
            rxn.cheb_n_pres = int(t[2])
            rxn.cheb_par = [float(x) for x in t[3:]]
    elif key == "pch":
        t = line.replace("/", " ").split()
        rxn.cheb_plim = [float(t[1]) * chem.PA, float(t[2]) * chem.PA]
        if len(t) > 5 and t[3].lower() == "tcheb":
            rxn.cheb_tlim = [float(t[4]), float(t[5])]
    elif key == "tch":
        t = line.replace("/", " ").split()
        rxn.cheb_tlim = [float(t[1]), float(t[2])]
        if len(t) > 5 and t[3].lower() == "pcheb":
            rxn.cheb_plim = [float(t[4]) * chem.PA, float(t[5]) * chem.PA]
    elif key == "plo":
        t = line.replace("/", " ").split()
        if not rxn.plog:
            rxn.plog = True
            rxn.pdep = False
            rxn.plog_par = []
        pars = [float(x) for x in t[1:5]]
        pars[0] *= 101325.0
        pars[3] *= act_energy_fact[units_E]
        if units_A == "moles":
            pars[1] /= 1000. ** (sum(rxn.reac_nu) - 1.)
        rxn.plog_par.append(pars)
    else:
        t = line.replace("/", " ").split()
        if len(t) % 2:
            raise MechanismError("efficiency line needs name/value pairs: "
                                 + line)
        for i in range(0, len(t), 2):
            rxn.thd_body_eff.append([t[i], float(t[i + 1])])


def read_mech(mech_filename, therm_filename=None):
    """Read a Chemkin mechanism -> (elems, specs, reacs).

    Same contract as mech_interpret.py:52-712: species keep file order,
    reactions keep file order with explicit-REV reactions split into two
    irreversible ones, thermo data comes from a THERMO section in the
    mechanism or from ``therm_filename``.
    """
    elems, specs, reacs = [], [], []
    elem_wt = chem.get_elem_wt()
    key = ""
    units_E, units_A = "cal/mole", "moles"
    state = {"cheb_open": False}
    have_thermo_section = False

    with open(mech_filename, "r") as f:
        lines = f.readlines()

    for raw in lines:
        if _skip(raw):
            continue
        line = raw
        k = line.find("!")
        if k > 0:
            line = line[:k]

        head = line[0:4].lower()
        if head in ("elem", "spec"):
            key = head
            toks = line.split()
            if len(toks) > 1:
                line = line[line.index(toks[1]):]
            else:
                continue
        elif head == "reac":
            key = "reac"
            units_E, units_A = "cal/mole", "moles"
            for u in line.split()[1:]:
                ul = u.lower()
                if ul in pre_units:
                    units_A = ul
                elif ul in act_energy_units:
                    units_E = ul
                else:
                    raise MechanismError(
                        "unsupported units on REACTION line: %r (choose "
                        "from %s and %s)" % (u, pre_units, act_energy_units))
            if units_A == "molecules":
                raise NotImplementedError("Molecules units not supported.")
            continue
        elif head == "ther":
            have_thermo_section = True
            read_thermo(mech_filename, elems, specs, elem_wt)
            continue
        elif line[0:3].lower() == "end":
            key = ""
            continue

        line = line.strip()
        if key == "elem":
            last = ""
            for tok in line.replace("/", " ").split():
                if tok.isalpha():
                    if tok[0:3] == "end":
                        continue
                    if tok not in elems:
                        elems.append(tok)
                    last = tok
                else:
                    elem_wt[last.lower()] = float(tok)
        elif key == "spec":
            names = {sp.name for sp in specs}
            for tok in line.split():
                if tok[0:3] == "end":
                    continue
                if tok not in names:
                    specs.append(chem.SpecInfo(tok))
                    names.add(tok)
        elif key == "reac":
            if "=" in line:
                state["cheb_open"] = False
                reacs.append(_parse_reaction(line, units_A, units_E))
            else:
                if not reacs:
                    raise MechanismError("auxiliary line before any "
                                         "reaction: " + line)
                _parse_aux(line, reacs[-1], units_A, units_E, state)

    # Chebyshev bookkeeping (mech_interpret.py:654-671).
    for i, rxn in enumerate(reacs):
        if rxn.cheb:
            n, m = rxn.cheb_n_temp, rxn.cheb_n_pres
            if len(rxn.cheb_par) != n * m:
                raise MechanismError("incorrect number of CHEB coefficients "
                                     "in reaction %d" % i)
            if units_A == "moles":
                order = sum(rxn.reac_nu)
                rxn.cheb_par[0] += math.log10(0.001 ** (order - 1.))
            rxn.cheb_par = np.reshape(rxn.cheb_par, (n, m))

    # Explicit reverse parameters: split into two irreversible reactions
    # (mech_interpret.py:673-693).
    out = []
    for rxn in reacs:
        out.append(rxn)
        if rxn.rev_par:
            back = copy.deepcopy(rxn)
            rxn.rev = False
            rxn.rev_par = []
            back.A, back.b, back.E = back.rev_par[0], back.rev_par[1], back.rev_par[2]
            back.rev = False
            back.rev_par = []
            back.prod, back.prod_nu = rxn.reac[:], rxn.reac_nu[:]
            back.reac, back.reac_nu = rxn.prod[:], rxn.prod_nu[:]
            out.append(back)
    reacs = out

    if any(not sp.mw for sp in specs):
        if therm_filename:
            read_thermo(therm_filename, elems, specs, elem_wt)
        elif not have_thermo_section:
            raise MechanismError("no thermo file specified, but species "
                                 "missing data")
    missing = [sp.name for sp in specs if not sp.mw]
    if missing:
        raise MechanismError("missing thermo data for " + ", ".join(missing))
    return elems, specs, reacs


def _fields(text, width):
    return [text[i:i + width] for i in range(0, len(text), width)]


def read_thermo(filename, elems, specs, elem_wt=None):
    """Fill ``mw``, ``elem``, ``Trange``, ``lo``, ``hi`` of ``specs`` from a
    fixed-column NASA-7 thermo file (mech_interpret.py:715-863).

    Columns: name 0:18 (cut at the first blank), element/count pairs in
    5-character fields over 24:44, temperatures 45:73 (low, high[, common]);
    lines 2-4 carry 15-character coefficients: hi[0:5]; hi[5:7], lo[0:3];
    lo[3:7].  The first entry of a species wins.
    """
    if elem_wt is None:
        elem_wt = chem.get_elem_wt()
    by_name = {sp.name: sp for sp in specs}
    with open(filename, "r") as f:
        lines = f.readlines()
    n = len(lines)
    i = 0
    while i < n:
        line = lines[i]
        i += 1
        if _skip(line):
            continue
        if "thermo" in line.lower():
            break
    else:
        raise MechanismError("no THERMO line in " + filename)

    t_common = None
    if i < n:
        toks = lines[i].split()
        if toks and toks[0][0:1].isdigit():
            t_common = [float(x) for x in toks]
            i += 1

    while i < n:
        line = lines[i]
        i += 1
        if line[0:3].lower() == "end":
            break
        if _skip(line):
            continue
        name = line[0:18].strip()
        if name.find(" ") > 0:
            name = name[:name.find(" ")]
        sp = by_name.get(name)
        if sp is None or sp.mw:
            i += 3
            continue
        for fld in _fields(line[24:44], 5):
            e = fld[0:2].strip()
            if e == "" or e == "0":
                continue
            cnt = int(float(fld[2:].strip()))
            sp.elem.append([e, cnt])
            try:
                sp.mw += cnt * elem_wt[e.lower()]
            except KeyError:
                raise MechanismError("unknown element %r in species %s"
                                     % (e, name))
        temps = [float(x) for x in line[45:73].split()]
        if len(temps) == 3:
            t_com = temps[2]
        elif t_common is not None:
            t_com = t_common[1]
        else:
            raise MechanismError("no common temperature for species " + name)
        sp.Trange = [temps[0], t_com, temps[1]]
        if i + 3 > n:
            raise MechanismError("truncated thermo entry for " + name)
        c2 = _fields(lines[i][0:75], 15)
        c3 = _fields(lines[i + 1][0:75], 15)
        c4 = _fields(lines[i + 2][0:75], 15)
        i += 3
        sp.hi[0:5] = [float(x) for x in c2[0:5]]
        sp.hi[5], sp.hi[6] = float(c3[0]), float(c3[1])
        sp.lo[0:3] = [float(x) for x in c3[2:5]]
        sp.lo[3:7] = [float(x) for x in c4[0:4]]
        if all(s.mw != 0.0 for s in specs):
            break
    return None
