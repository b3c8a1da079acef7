"""Species bookkeeping shared by the front end and the table builder.

Same contracts as create_rate_subs' ``utils.py``:
``get_species_mappings`` (utils.py:40-60), ``get_nu`` (utils.py:63-79),
``reassign_species_lists`` (utils.py:199-212), ``is_integer``
(utils.py:215-228), ``create_dir`` (utils.py:125-144).
"""

import errno
import os

__all__ = ["get_species_mappings", "get_nu", "reassign_species_lists",
           "is_integer", "create_dir", "langs"]

# Output targets of the CLI.  'c'/'cuda'/'fortran'/'matlab' are the
# reference's (utils.py:14); 'gb300' writes the table blob and headers for
# the sm_103a library.
langs = ["c", "cuda", "fortran", "matlab", "gb300"]


def get_species_mappings(num_specs, last_species):
    """(fwd_map, back_map) that move species ``last_species`` to the end.

    ``fwd_map[i]`` is the original index of new species ``i``;
    ``back_map[j]`` is the new index of original species ``j``.
    """
    fwd = [i for i in range(num_specs) if i != last_species] + [last_species]
    back = [0] * num_specs
    for new, old in enumerate(fwd):
        back[old] = new
    return fwd, back


def get_nu(isp, rxn):
    """Net stoichiometric coefficient of species ``isp`` in ``rxn``
    (products minus reactants; 0 if it does not take part)."""
    in_p = isp in rxn.prod
    in_r = isp in rxn.reac
    if in_p and in_r:
        nu = rxn.prod_nu[rxn.prod.index(isp)] - rxn.reac_nu[rxn.reac.index(isp)]
        return 0 if nu == 0 else nu
    if in_p:
        return rxn.prod_nu[rxn.prod.index(isp)]
    if in_r:
        return -rxn.reac_nu[rxn.reac.index(isp)]
    return 0


def reassign_species_lists(reacs, specs):
    """Replace species names in reactions by their index in ``specs``."""
    index = {sp.name: i for i, sp in enumerate(specs)}
    for rxn in reacs:
        rxn.reac = [index[s] for s in rxn.reac]
        rxn.prod = [index[s] for s in rxn.prod]
        rxn.thd_body_eff = [(index[t[0]], t[1]) for t in rxn.thd_body_eff]
        if rxn.pdep_sp:
            rxn.pdep_sp = index[rxn.pdep_sp]


def is_integer(val):
    """True when ``val`` has an integral value, int or float."""
    try:
        return float(val).is_integer()
    except (TypeError, ValueError, OverflowError):
        return False


def create_dir(path):
    """mkdir -p."""
    try:
        os.makedirs(path)
    except OSError as exc:
        if exc.errno != errno.EEXIST:
            raise
