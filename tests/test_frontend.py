"""Front end: Chemkin reader, species order, tables (CPU only)."""
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from create_rate_subs_gb300 import chem, mech_interpret, synth, tables
from create_rate_subs_gb300.mechanism import Mechanism, choose_last_species


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_species_order_matches_reference(case, golden):
    """The species order equals the one the reference printed in header.h
    (create_rate_subs.py:399-403) -- bit-exact indexing."""
    mech, g = golden(case)
    assert mech.names == [str(s) for s in g["species"]]
    assert (mech.n_species, mech.n_reactions, mech.n_rev, mech.n_pdep) == \
        tuple(int(x) for x in g["dims"])


def _write(text, suffix):
    fd, p = tempfile.mkstemp(suffix=suffix)
    with os.fdopen(fd, "w") as f:
        f.write(text)
    return p


THERMO = None


def _thermo(names_comps):
    rng = np.random.default_rng(3)
    out = ["THERMO", "   300.000  1000.000  5000.000"]
    for name, comp in names_comps:
        lo, hi = synth._fit_thermo(rng)
        out.append(synth._thermo_entry(name, comp, lo, hi))
    out.append("END")
    return "\n".join(out) + "\n"


BASIC = [("H2", (0, 2, 0, 0, 0)), ("O2", (0, 0, 2, 0, 0)), ("H", (0, 1, 0, 0, 0)),
         ("O", (0, 0, 1, 0, 0)), ("OH", (0, 1, 1, 0, 0)), ("H2O", (0, 2, 1, 0, 0)),
         ("N2", (0, 0, 0, 2, 0)), ("AR", (0, 0, 0, 0, 1))]


def _mech(reactions, units=""):
    return ("ELEMENTS\nH O N AR\nEND\nSPECIES\nH2 O2 H O OH H2O N2 AR\nEND\n"
            "REACTIONS %s\n%s\nEND\n" % (units, reactions))


def _parse(reactions, units=""):
    mp = _write(_mech(reactions, units), ".inp")
    tp = _write(_thermo(BASIC), ".dat")
    return mech_interpret.read_mech(mp, tp)


def test_units_and_orders():
    """A conversion by reaction order, E by the unit factor
    (mech_interpret.py:39-46, 441-455)."""
    _, _, r = _parse("H+O2<=>O+OH 1.0E+14 0.0 1000.0\n"
                     "2O+M<=>O2+M 1.0E+16 -0.5 0.0\n"
                     "H+O2(+M)<=>HO2(+M) 1.0E+12 0.5 0.0\n LOW/1.0E+18 -1.0 0.0/\n"
                     .replace("HO2", "H2O"))
    assert r[0].A == 1.0e14 / 1000.0
    assert r[0].E == 1000.0 * (4.184 / chem.RU_JOUL)
    assert r[1].thd_body and not r[1].pdep
    assert r[1].A == 1.0e16 / 1000.0 ** 2
    assert r[2].pdep and not r[2].thd_body and r[2].pdep_sp == ""
    assert r[2].A == 1.0e12 / 1000.0
    assert r[2].low[0] == 1.0e18 / 1000.0 ** 2
    _, _, rk = _parse("H+O2<=>O+OH 1.0E+14 0.0 1000.0", units="KELVINS")
    assert rk[0].E == 1000.0


def test_rev_split_and_duplicate_merge():
    """Explicit REV becomes two irreversible reactions (mech_interpret.py:
    673-693); repeated species merge their coefficients."""
    _, _, r = _parse("H+O2<=>O+OH 1.0E+14 0.0 1000.0\n REV / 2.0E+13 0.1 500.0 /\n"
                     "H+H+O2=>H2+O2 1.0E+10 0 0")
    assert len(r) == 3
    assert not r[0].rev and not r[1].rev
    assert r[1].reac == ["O", "OH"] and r[1].prod == ["H", "O2"]
    assert r[1].A == 2.0e13 / 1000.0 and r[1].b == 0.1
    assert r[2].reac == ["H", "O2"] and r[2].reac_nu == [2, 1]


def test_named_collider_and_efficiencies():
    _, _, r = _parse("H+OH(+H2O)<=>H2O(+H2O) 1.0E+13 0.0 0.0\n LOW/1.0E+18 -1.0 0.0/\n"
                     "2H+M<=>H2+M 1.0E+18 -1.0 0.0\n H2/2.5/ H2O/12.0/ AR/1.0/")
    assert r[0].pdep and r[0].pdep_sp == "H2O"
    assert r[1].thd_body_eff == [["H2", 2.5], ["H2O", 12.0], ["AR", 1.0]]


def test_errors():
    with pytest.raises(mech_interpret.MechanismError):
        _parse("H+O2<=>O+OH 1.0E+14 0.0 1000.0", units="FURLONGS")
    mp = _write(_mech("H+O2<=>O+OH 1.0E+14 0.0 1000.0"), ".inp")
    with pytest.raises(mech_interpret.MechanismError):
        mech_interpret.read_mech(mp, None)
    tp = _write(_thermo(BASIC[:-1]), ".dat")   # AR missing
    with pytest.raises(mech_interpret.MechanismError):
        mech_interpret.read_mech(mp, tp)


def test_last_species_rules():
    """User choice, else N2/Ar/He by name and exact weight, else the last
    (create_rate_subs.py:466-512)."""
    _, specs, _ = _parse("H+O2<=>O+OH 1.0E+14 0.0 1000.0")
    assert specs[choose_last_species(specs)].name == "N2"
    assert specs[choose_last_species(specs, "ar")].name == "AR"
    assert specs[choose_last_species(specs, "XX")].name == "N2"
    specs[6].mw += 1e-9  # N2 no longer matches the exact weight
    assert specs[choose_last_species(specs)].name == "AR"


def test_table_roundings():
    """Troe constants are taken as printed with %.8e, SRI a/b/c/e with 6
    significant digits (rate_subs.py:968-1037)."""
    mech, _ = load_golden("features")
    t = mech.tables
    troe = [p for p in range(mech.n_pdep) if t["pm_form"][p] == tables.FORM_TROE]
    for p in troe:
        for v in t["pm_troe"][p]:
            assert v == float("%.8e" % v)
    sri = [p for p in range(mech.n_pdep) if t["pm_form"][p] == tables.FORM_SRI]
    assert sri
    for p in sri:
        for v in t["pm_sri"][p][[0, 1, 2, 4]]:
            assert v == float("{:.6}".format(v))


def test_blob_roundtrip(golden):
    mech, _ = golden("gri53")
    back = tables.unpack(mech.blob)
    for k, v in mech.tables.items():
        assert np.array_equal(np.asarray(v).ravel(), np.asarray(back[k]).ravel()), k


def test_synthetic_counts(synth_mech):
    """Workload mechanisms have the sizes their names promise."""
    for name, (N, R, NREV, NPM) in (("small", (10, 27, 27, 8)),
                                    ("gri53", (53, 325, 305, 60))):
        m = synth_mech(name)
        assert (m.n_species, m.n_reactions, m.n_rev, m.n_pdep) == (N, R, NREV, NPM)
        assert m.names[-1] == "N2"


def test_atom_balance(synth_mech):
    """Every synthetic reaction conserves atoms."""
    m = synth_mech("gri53")
    _, E = m.element_matrix()
    t = m.tables
    for r in range(m.n_reactions):
        s = np.zeros(E.shape[0])
        for e in range(t["nu_ptr"][r], t["nu_ptr"][r + 1]):
            s += E[:, t["nu_sp"][e]] * t["nu_val"][e]
        assert np.all(s == 0), r


def test_states_layout():
    T, P, Y = synth.make_states(7, 100, seed=1)
    assert T.shape == (100,) and P.shape == (100,) and Y.shape == (7, 100)
    assert np.allclose(Y.sum(axis=0), 1.0)
    assert T.min() >= 800 and T.max() <= 2800
    assert P.min() >= chem.PA * 0.999 and P.max() <= 50 * chem.PA * 1.001
