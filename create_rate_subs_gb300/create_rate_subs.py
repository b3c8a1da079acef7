"""Command line and driver: the reference's ``create_rate_subs`` entry point.

    python -m create_rate_subs_gb300 -l gb300 -i mech.dat [-t therm.dat] [-ls N2]

Same options as the reference's CLI (create_rate_subs.py:560-593):
``-l/--lang``, ``-i/--input``, ``-t/--thermo``, ``-ls/--last_species``,
output in ``./out/``.  Differences, all deliberate:

* ``-ls`` is honoured (the reference parses it and then drops it,
  create_rate_subs.py:593);
* instead of unrolled source, every target writes the mechanism tables
  (``out/mech.crs``, loaded by ``crs_mech_load_file``) and headers that
  declare the reference's four per-state functions, implemented by libcrs:
  ``c`` -> header.h, chem_utils.h, rates.h; ``cuda`` -> the same with .cuh
  names; ``gb300`` -> both sets;
* ``fortran`` and ``matlab`` are refused (the reference itself marks them
  incomplete, create_rate_subs.py:459-460).
"""

import argparse
import os
import sys

from .mech_interpret import MechanismError
from .mechanism import Mechanism
from .utils import create_dir, langs

__all__ = ["create_rate_subs", "main"]


def _header(mech):
    lines = ["/* Species of the mechanism, in evaluation order (the bath gas last). */",
             "#ifndef CRS_MECH_HEADER", "#define CRS_MECH_HEADER", "",
             "/** Number of species."]
    for i, name in enumerate(mech.names):
        lines.append(" * %d %s" % (i, name))
    lines += [" */", "#define NSP %d" % mech.n_species,
              "/** Number of variables. NN = NSP + 1 (temperature). */",
              "#define NN %d" % (mech.n_species + 1),
              "#define NRXN %d" % mech.n_reactions,
              "#define NREV %d" % mech.n_rev,
              "#define NPDEP %d" % mech.n_pdep, "", "#endif", ""]
    return "\n".join(lines)


def _decls(kind):
    if kind == "chem_utils":
        body = ("void eval_conc (const double, const double, const double*, "
                "double*, double*, double*, double*);\n")
    else:
        body = ("void eval_rxn_rates (const double, const double, const double*, "
                "double*, double*);\n"
                "void eval_spec_rates (const double*, const double*, const double*, "
                "double*, double*);\n"
                "void get_rxn_pres_mod (const double, const double, const double*, "
                "double*);\n")
    guard = "CRS_%s_HEAD" % kind.upper()
    return ("#ifndef %s\n#define %s\n\n#include \"header.h\"\n\n"
            "/* Implemented by libcrs (include/crs.h) on the GPU.  Load out/mech.crs\n"
            " * with crs_mech_load_file and select it with crs_bind first. */\n"
            "#ifdef __cplusplus\nextern \"C\" {\n#endif\n%s"
            "#ifdef __cplusplus\n}\n#endif\n\n#endif\n" % (guard, guard, body))


def create_rate_subs(lang, mech_name, therm_name=None, last_spec=None,
                     out_dir="./out/"):
    """Parse, order and write tables + headers; returns the Mechanism."""
    lang = lang.lower()
    if lang not in langs:
        raise ValueError("language needs to be one of: %s" % ", ".join(langs))
    if lang in ("fortran", "matlab"):
        raise NotImplementedError("Fortran and Matlab targets are not provided")
    if mech_name.endswith((".cti", ".xml")):
        raise NotImplementedError("Cantera input is not supported (cantera is "
                                  "not available and its reader used an "
                                  "obsolete API)")
    mech = Mechanism.from_chemkin(mech_name, therm_name, last_spec)
    create_dir(out_dir)
    with open(os.path.join(out_dir, "mech.crs"), "wb") as f:
        f.write(mech.blob)
    exts = {"c": [".h"], "cuda": [".cuh"], "gb300": [".h", ".cuh"]}[lang]
    for ext in exts:
        with open(os.path.join(out_dir, "header" + ext), "w") as f:
            f.write(_header(mech))
        with open(os.path.join(out_dir, "chem_utils" + ext), "w") as f:
            f.write(_decls("chem_utils").replace('"header.h"', '"header%s"' % ext))
        with open(os.path.join(out_dir, "rates" + ext), "w") as f:
            f.write(_decls("rates").replace('"header.h"', '"header%s"' % ext))
    return mech


def main(argv=None):
    ap = argparse.ArgumentParser(
        description="Generates mechanism tables for the GB300 species and "
                    "reaction rate library.")
    ap.add_argument("-l", "--lang", type=str, choices=langs, required=True,
                    help="Target: c, cuda (headers for the reference's "
                         "function names) or gb300 (both).")
    ap.add_argument("-i", "--input", type=str, required=True,
                    help="Input mechanism filename (e.g., mech.dat).")
    ap.add_argument("-t", "--thermo", type=str, default=None,
                    help="Thermodynamic database filename (e.g., therm.dat), "
                         "or nothing if in mechanism.")
    ap.add_argument("-ls", "--last_species", required=False, type=str,
                    default=None,
                    help="The name of the species to set as the last in the "
                         "mechanism. If not specified, defaults to the first "
                         "of N2, AR, and HE in the mechanism.")
    args = ap.parse_args(argv)
    try:
        mech = create_rate_subs(args.lang, args.input, args.thermo,
                                args.last_species)
    except (MechanismError, NotImplementedError, ValueError, OSError) as exc:
        print("Error: %s" % exc, file=sys.stderr)
        return 1
    print("%d species, %d reactions (%d reversible, %d pressure-dependent); "
          "tables in ./out/mech.crs" % (mech.n_species, mech.n_reactions,
                                        mech.n_rev, mech.n_pdep))
    return 0
