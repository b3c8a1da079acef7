"""Physical constants, element weights and the species/reaction records.

These records are what the Chemkin front end produces and what the table
builder consumes.  Field names and units follow create_rate_subs'
``chem_utilities.py`` so that code written against the reference's objects
keeps working:

* constants: chem_utilities.py:17-25 (``RU`` J/(kmol K), ``PA`` Pa, ...)
* element weights [kg/kmol]: chem_utilities.py:47-95
* ``ReacInfo``: chem_utilities.py:98-211 (A in m/kmol/s units, ``E`` stored
  as an activation temperature in K)
* ``SpecInfo``: chem_utilities.py:214-248 (NASA-7 ``lo``/``hi`` arrays,
  ``Trange`` = [T_low, T_common, T_high])
"""

import numpy as np

__all__ = ["RU", "RU_JOUL", "RUC", "AVAG", "PA", "get_elem_wt",
           "ReacInfo", "SpecInfo"]

# Universal gas constant [J/(kmol K)] and friends (chem_utilities.py:17-25).
RU = 8314.4621
RU_JOUL = 8.3144621
RUC = RU / 4.18400
AVAG = 6.0221367e23
# One standard atmosphere [Pa].
PA = 101325.0

# Atomic weights [kg/kmol] by lower-case element symbol.  The numbers are the
# reference's table (chem_utilities.py:59-94); they fix every molecular
# weight and therefore every concentration, so they must be identical.
_ELEM_WT = (
    ("h", 1.00794), ("he", 4.00260), ("li", 6.93900), ("be", 9.01220),
    ("b", 10.81100), ("c", 12.0110), ("n", 14.00674), ("o", 15.99940),
    ("f", 18.99840), ("ne", 20.18300), ("na", 22.98980), ("mg", 24.31200),
    ("al", 26.98150), ("si", 28.08600), ("p", 30.97380), ("s", 32.06400),
    ("cl", 35.45300), ("ar", 39.94800), ("k", 39.10200), ("ca", 40.08000),
    ("sc", 44.95600), ("ti", 47.90000), ("v", 50.94200), ("cr", 51.99600),
    ("mn", 54.93800), ("fe", 55.84700), ("co", 58.93320), ("ni", 58.71000),
    ("cu", 63.54000), ("zn", 65.37000), ("ga", 69.72000), ("ge", 72.59000),
    ("as", 74.92160), ("se", 78.96000), ("br", 79.90090), ("kr", 83.80000),
    ("rb", 85.47000), ("sr", 87.62000), ("y", 88.90500), ("zr", 91.22000),
    ("nb", 92.90600), ("mo", 95.94000), ("tc", 99.00000), ("ru", 101.07000),
    ("rh", 102.90500), ("pd", 106.40000), ("ag", 107.87000),
    ("cd", 112.40000), ("in", 114.82000), ("sn", 118.69000),
    ("sb", 121.75000), ("te", 127.60000), ("i", 126.90440),
    ("xe", 131.30000), ("cs", 132.90500), ("ba", 137.34000),
    ("la", 138.91000), ("ce", 140.12000), ("pr", 140.90700),
    ("nd", 144.24000), ("pm", 145.00000), ("sm", 150.35000),
    ("eu", 151.96000), ("gd", 157.25000), ("tb", 158.92400),
    ("dy", 162.50000), ("ho", 164.93000), ("er", 167.26000),
    ("tm", 168.93400), ("yb", 173.04000), ("lu", 174.99700),
    ("hf", 178.49000), ("ta", 180.94800), ("w", 183.85000),
    ("re", 186.20000), ("os", 190.20000), ("ir", 192.20000),
    ("pt", 195.09000), ("au", 196.96700), ("hg", 200.59000),
    ("tl", 204.37000), ("pb", 207.19000), ("bi", 208.98000),
    ("po", 210.00000), ("at", 210.00000), ("rn", 222.00000),
    ("fr", 223.00000), ("ra", 226.00000), ("ac", 227.00000),
    ("th", 232.03800), ("pa", 231.00000), ("u", 238.03000),
    ("np", 237.00000), ("pu", 242.00000), ("am", 243.00000),
    ("cm", 247.00000), ("bk", 249.00000), ("cf", 251.00000),
    ("es", 254.00000), ("fm", 253.00000), ("d", 2.01410),
    ("e", 5.48578e-4),
)


def get_elem_wt():
    """Fresh dict {element symbol (lower case): atomic weight [kg/kmol]}.

    Same contract as chem_utilities.py:47-95.  A new dict is returned on each
    call so that atomic-weight overrides in one mechanism's ELEMENTS section
    cannot leak into the next parse.
    """
    return dict(_ELEM_WT)


class _Record(object):
    """Attribute-wise equality, as chem_utilities.py:28-44 provides."""

    def __eq__(self, other):
        if type(self) is not type(other):
            return False
        a, b = self.__dict__, other.__dict__
        if a.keys() != b.keys():
            return False
        for k, v in a.items():
            w = b[k]
            if isinstance(v, np.ndarray) or isinstance(w, np.ndarray):
                if not np.array_equal(np.asarray(v), np.asarray(w)):
                    return False
            elif v != w:
                return False
        return True

    def __ne__(self, other):
        return not self.__eq__(other)

    __hash__ = None


class ReacInfo(_Record):
    """One reaction (fields of chem_utilities.py:155-211).

    ``A`` is in kmol/m^3/s units after the parser's conversion, ``b`` is the
    temperature exponent, ``E`` the activation temperature [K].  ``reac`` /
    ``prod`` hold species names until the species order is fixed, then
    indices.  ``thd_body`` marks ``+M`` reactions, ``pdep`` ``(+M)`` or
    ``(+SP)`` fall-off reactions; ``low``/``high`` hold [A, b, E] of the
    other pressure limit; ``troe_par``/``sri_par`` the broadening constants.
    """

    def __init__(self, rev, reactants, reac_nu, products, prod_nu, A, b, E):
        self.reac = reactants
        self.reac_nu = reac_nu
        self.prod = products
        self.prod_nu = prod_nu
        self.A = A
        self.b = b
        self.E = E
        self.rev = rev
        self.rev_par = []
        self.dup = False
        self.thd_body = False
        self.thd_body_eff = []
        self.pdep = False
        self.pdep_sp = ''
        self.low = []
        self.high = []
        self.troe = False
        self.troe_par = []
        self.sri = False
        self.sri_par = []
        self.cheb = False
        self.cheb_n_temp = 0
        self.cheb_n_pres = 0
        self.cheb_plim = [0.001 * PA, 100. * PA]
        self.cheb_tlim = [300., 2500.]
        self.cheb_par = None
        self.plog = False
        self.plog_par = None


class SpecInfo(_Record):
    """One species (fields of chem_utilities.py:236-248)."""

    def __init__(self, name):
        self.name = name
        self.elem = []
        self.mw = 0.0
        self.hi = np.zeros(7)
        self.lo = np.zeros(7)
        self.Trange = [300.0, 1000.0, 5000.0]
