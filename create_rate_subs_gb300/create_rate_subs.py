"""Command line and driver: the reference's ``create_rate_subs`` entry point.

    python -m create_rate_subs_gb300 -l gb300 -i mech.dat [-t therm.dat] [-ls N2]

Same options as the reference's CLI (create_rate_subs.py:560-593):
``-l/--lang``, ``-i/--input``, ``-t/--thermo``, ``-ls/--last_species``,
output in ``./out/``.  Differences, all deliberate:

* ``-ls`` is honoured (the reference parses it and then drops it,
  create_rate_subs.py:593);
* instead of unrolled source, every target writes the mechanism tables
  (``out/mech.crs``, loaded by ``crs_mech_load_file``) and headers for the
  reference's per-state functions:
  ``c`` -> header.h, chem_utils.h, rates.h, dydt.h: host declarations,
  implemented by libcrs (crs.h; bind the loaded tables with crs_bind);
  ``cuda`` -> header.cuh, chem_utils.cuh, rates.cuh, dydt.cuh: __device__
  definitions (include/crs_device.cuh) over the mechanism's table image,
  written as mech_image.cuh, with the headers they include copied beside
  them, so that a user's kernel calls them per thread as it calls the
  reference's emitted CUDA; ``gb300`` -> both sets;
* ``fortran`` and ``matlab`` are refused (the reference itself marks them
  incomplete, create_rate_subs.py:459-460).
"""

import argparse
import os
import shutil
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
              "/** Reactions, reversible reactions, pres_mod entries. */",
              "#define NRXN %d" % mech.n_reactions,
              "#define NRXN_REV %d" % mech.n_rev,
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
            "/* Implemented by libcrs (include/crs.h) on the host, reentrant.  Load\n"
            " * out/mech.crs with crs_mech_load_file or crs_mech_load_host and select\n"
            " * it with crs_bind (or crs_bind_thread) first. */\n"
            "#ifdef __cplusplus\nextern \"C\" {\n#endif\n%s"
            "#ifdef __cplusplus\n}\n#endif\n\n#endif\n" % (guard, guard, body))


def _dydt_decls():
    return ("#ifndef CRS_DYDT_HEAD\n#define CRS_DYDT_HEAD\n\n#include \"header.h\"\n\n"
            "/* Implemented by libcrs (include/crs.h) on the host: constant pressure\n"
            " * unless crs_dydt_form(1) selects constant volume. */\n"
            "#ifdef __cplusplus\nextern \"C\" {\n#endif\n"
            "void dydt (const double, const double, const double*, double*);\n"
            "#ifdef __cplusplus\n}\n#endif\n\n#endif\n")


def table_image(blob):
    """(image bytes, layout int32 words) of a mechanism blob, built by
    libcrs on the host (crs_mech_image)."""
    import ctypes
    from . import _lib
    lib = _lib.load()
    sizes = (ctypes.c_size_t * 2)()
    _lib.check(lib.crs_mech_image(blob, len(blob), None, 0, None, 0, sizes))
    img = ctypes.create_string_buffer(int(sizes[0]))
    lay = (ctypes.c_int32 * int(sizes[1]))()
    _lib.check(lib.crs_mech_image(blob, len(blob), img, sizes[0], lay, sizes[1], sizes))
    return img.raw[: int(sizes[0])], list(lay)


def _image_header(mech):
    """mech_image.cuh: the table image as a __device__ array and its
    layout as a __constant__ crs::ImgLayout (crs_tables.h), for
    crs_device.cuh."""
    img, lay = table_image(mech.blob)
    if len(img) % 8:
        img = img + b"\0" * (8 - len(img) % 8)
    words = [int.from_bytes(img[i:i + 8], "little") for i in range(0, len(img), 8)]
    out = ["/* Table image of the mechanism (%d species, %d reactions) for the per-state"
           % (mech.n_species, mech.n_reactions),
           " * device functions of crs_device.cuh; written by create_rate_subs_gb300. */",
           "#ifndef CRS_MECH_IMAGE_CUH", "#define CRS_MECH_IMAGE_CUH", "",
           "#include \"crs_tables.h\"", "",
           "#define CRS_MECH_IMAGE_DEFINED 1",
           "#define CRS_MECH_NSP %d" % mech.n_species,
           "#define CRS_MECH_NRXN %d" % mech.n_reactions,
           "#define CRS_MECH_NREV %d" % mech.n_rev,
           "#define CRS_MECH_NPDEP %d" % mech.n_pdep, "",
           "static __device__ __align__(16) const unsigned long long crs_mech_image_words[%d] = {"
           % len(words)]
    for i in range(0, len(words), 6):
        out.append("  " + ", ".join("0x%016xull" % w for w in words[i:i + 6]) + ",")
    out.append("};")
    out.append("#define crs_mech_image "
               "(reinterpret_cast<const unsigned char *>(crs_mech_image_words))")
    out.append("static __constant__ crs::ImgLayout crs_mech_layout = {")
    for i in range(0, len(lay), 12):
        out.append("  " + ", ".join(str(v) for v in lay[i:i + 12]) + ",")
    out += ["};", "", "#endif", ""]
    return "\n".join(out)


def _device_header(guard):
    return ("#ifndef %s\n#define %s\n\n#include \"header.cuh\"\n"
            "#include \"mech_image.cuh\"\n#include \"crs_device.cuh\"\n\n#endif\n"
            % (guard, guard))


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
    if lang in ("c", "gb300"):
        files = {"header.h": _header(mech), "chem_utils.h": _decls("chem_utils"),
                 "rates.h": _decls("rates"), "dydt.h": _dydt_decls()}
        for name, text in files.items():
            with open(os.path.join(out_dir, name), "w") as f:
                f.write(text)
    if lang in ("cuda", "gb300"):
        files = {"header.cuh": _header(mech), "mech_image.cuh": _image_header(mech),
                 "chem_utils.cuh": _device_header("CRS_CHEM_UTILS_CUH"),
                 "rates.cuh": _device_header("CRS_RATES_CUH"),
                 "dydt.cuh": _device_header("CRS_DYDT_CUH")}
        for name, text in files.items():
            with open(os.path.join(out_dir, name), "w") as f:
                f.write(text)
        inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                           "include")
        for name in ("crs_tables.h", "crs_eval.h", "crs_device.cuh"):
            shutil.copy(os.path.join(inc, name), os.path.join(out_dir, name))
    return mech


def main(argv=None):
    ap = argparse.ArgumentParser(
        description="Generates mechanism tables for the GB300 species and "
                    "reaction rate library.")
    ap.add_argument("-l", "--lang", type=str, choices=langs, required=True,
                    help="Target: c (host declarations, implemented by "
                         "libcrs), cuda (device definitions over the "
                         "mechanism's table image) or gb300 (both).")
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
