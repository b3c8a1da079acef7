"""A parsed, ordered mechanism and its tables.

``Mechanism.from_chemkin`` runs the same front-end steps as the reference's
``create_rate_subs`` (create_rate_subs.py:466-526): parse, pick the bath gas
(user choice, else the first of N2/Ar/He matched by name *and* exact
molecular weight, else the last species), move it to the end, and replace
species names by indices.  The tables built from the result are what the
sm_103a library evaluates.
"""

import copy
import logging

from . import chem
from .mech_interpret import read_mech
from .tables import build_tables, pack
from .utils import get_species_mappings, reassign_species_lists

__all__ = ["Mechanism", "choose_last_species"]

log = logging.getLogger("create_rate_subs_gb300")


def choose_last_species(specs, last_spec=None):
    """Index of the species to move last (create_rate_subs.py:466-512)."""
    if last_spec is not None:
        want = last_spec.lower().strip()
        for i, sp in enumerate(specs):
            if sp.name.lower() == want:
                return i
        log.warning("user specified last species %s not found in mechanism;"
                    " attempting to find a default species", last_spec)
    wt = chem.get_elem_wt()
    for name, mw in (("N2", wt["n"] * 2.), ("Ar", wt["ar"]), ("He", wt["he"])):
        for i, sp in enumerate(specs):
            if name.lower() == sp.name.lower() and mw == sp.mw:
                return i
    log.warning("neither a user specified nor a default last species was "
                "found; using the last species %s", specs[-1].name)
    return len(specs) - 1


class Mechanism(object):
    """Species in evaluation order, reactions with index-based species lists,
    and the packed tables.

    Attributes: ``elems``, ``specs`` (ordered ``SpecInfo``), ``reacs``
    (``ReacInfo`` with integer species), ``fwd_spec_mapping`` (original index
    of each ordered species), ``names``.
    """

    def __init__(self, elems, specs, reacs, last_spec=None):
        specs = list(specs)
        reacs = copy.deepcopy(list(reacs))
        last = choose_last_species(specs, last_spec)
        fwd, _ = get_species_mappings(len(specs), last)
        specs = [specs[i] for i in fwd]
        reassign_species_lists(reacs, specs)
        self.elems = list(elems)
        self.specs = specs
        self.reacs = reacs
        self.fwd_spec_mapping = fwd
        self._tables = None
        self._blob = None

    @classmethod
    def from_chemkin(cls, mech_filename, therm_filename=None, last_spec=None):
        elems, specs, reacs = read_mech(mech_filename, therm_filename)
        return cls(elems, specs, reacs, last_spec)

    @property
    def names(self):
        return [sp.name for sp in self.specs]

    @property
    def n_species(self):
        return len(self.specs)

    @property
    def n_reactions(self):
        return len(self.reacs)

    @property
    def n_rev(self):
        return sum(1 for r in self.reacs if r.rev)

    @property
    def n_pdep(self):
        return sum(1 for r in self.reacs if r.thd_body or r.pdep)

    @property
    def tables(self):
        if self._tables is None:
            self._tables = build_tables(self.specs, self.reacs)
        return self._tables

    @property
    def blob(self):
        """Packed tables, the input of ``crs_mech_load``."""
        if self._blob is None:
            self._blob = pack(self.tables)
        return self._blob

    def element_matrix(self, elements=None):
        """(n_elements, n_species) atom counts, for conservation checks."""
        import numpy as np
        if elements is None:
            elements = []
            for sp in self.specs:
                for e, _ in sp.elem:
                    if e.lower() not in [x.lower() for x in elements]:
                        elements.append(e)
        idx = {e.lower(): i for i, e in enumerate(elements)}
        m = np.zeros((len(elements), len(self.specs)))
        for j, sp in enumerate(self.specs):
            for e, n in sp.elem:
                m[idx[e.lower()], j] += n
        return elements, m
