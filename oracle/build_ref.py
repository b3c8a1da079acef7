"""Build the reference's own C for a mechanism (TEST INFRASTRUCTURE).

Recipe, two steps:

``generate``  (needs the reference checkout: the directory named by the
    environment variable CRS_REFERENCE, default /root/reference)
    Copies the reference's five Python modules into a scratch directory,
    applies the minimal Python 3 patch (``except Exception, e`` ->
    ``as e`` and ``iteritems`` in chem_utilities.py; ``range`` ->
    ``list(range(...))`` for the species maps in utils.py; ``xrange`` ->
    ``range`` in create_rate_subs.py), runs the reference's
    ``create_rate_subs('c', mech, therm)`` in a scratch working directory
    and copies the emitted ``chem_utils.c``, ``rxn_rates.c``,
    ``rxn_rates_pres_mod.c``, ``spec_rates.c``, ``dydt.c`` and their headers into
    ``oracle/_ref/<name>/``, with the mechanism text they were emitted from
    in ``oracle/_ref/<name>/_mech/`` (``mechanism_files``).  Nothing is
    written to the reference checkout.

``compile``  (needs only ``oracle/_ref/<name>/`` and ``oracle/ref_harness.c``)
    Compiles the emitted files with the batch driver into
    ``oracle/_ref/<name>/libref.so`` (``-O2 -ffp-contract=off -fopenmp``:
    the parity build, states spread over threads) and ``libref_omp.so`` (``-O3 -fopenmp``: the timed CPU baseline),
    and the emitted ``dydt.c`` (constant pressure, ``-DCONP``) with
    ``ref_dydt_harness.c`` into ``libref_dydt.so``.

``oracle/_ref/`` is git-ignored; the emitted sources travel with the
working tree so that ``compile`` can run on another host.

Usage: python oracle/build_ref.py {generate,compile,all} NAME [NAME ...]
       python oracle/build_ref.py available   (exit 0 when the checkout exists)
       (NAME is a key of create_rate_subs_gb300.synth.CONFIGS)
"""

import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout that ``generate`` reads (never written).
REFERENCE = os.environ.get("CRS_REFERENCE", "/root/reference")
EMITTED = ("chem_utils.c", "rxn_rates.c", "rxn_rates_pres_mod.c",
           "spec_rates.c", "header.h", "rates.h", "chem_utils.h", "dydt.c",
           "dydt.h")

_PATCHES = {
    "chem_utilities.py": [("except Exception, e:", "except Exception as e:"),
                          (".iteritems()", ".items()")],
    "utils.py": [("fwd_species_map = range(num_specs)",
                  "fwd_species_map = list(range(num_specs))"),
                 ("back_species_map = range(num_specs)",
                  "back_species_map = list(range(num_specs))")],
    "create_rate_subs.py": [("xrange(", "range(")],
}


def ref_dir(name):
    return os.path.join(REF_OUT, name)


def generate(name, mech_path, therm_path, reference=None, last_spec=None):
    """Emit the reference's C for one mechanism into oracle/_ref/<name>/."""
    reference = reference or REFERENCE
    if not os.path.isdir(reference):
        raise FileNotFoundError("reference checkout not found: " + reference)
    mech_path = os.path.abspath(mech_path)
    therm_path = os.path.abspath(therm_path) if therm_path else None
    with tempfile.TemporaryDirectory(prefix="crs_refgen_") as tmp:
        src = os.path.join(tmp, "src")
        os.makedirs(src)
        for fn in ("chem_utilities.py", "create_rate_subs.py",
                   "mech_interpret.py", "rate_subs.py", "utils.py"):
            with open(os.path.join(reference, fn)) as f:
                text = f.read()
            for old, new in _PATCHES.get(fn, []):
                if old not in text:
                    raise RuntimeError("patch target %r missing in %s" % (old, fn))
                text = text.replace(old, new)
            with open(os.path.join(src, fn), "w") as f:
                f.write(text)
        work = os.path.join(tmp, "work")
        os.makedirs(work)
        code = ("import sys, warnings\n"
                "warnings.simplefilter('ignore')\n"
                "sys.path.insert(0, %r)\n"
                "import create_rate_subs as crs\n"
                "crs.create_rate_subs('c', %r, %r, %r)\n"
                % (src, mech_path, therm_path, last_spec))
        res = subprocess.run([sys.executable, "-c", code], cwd=work,
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference generator failed:\n" + res.stdout
                               + res.stderr)
        out = os.path.join(work, "out")
        dst = ref_dir(name)
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        os.makedirs(dst)
        for fn in EMITTED:
            p = os.path.join(out, fn)
            if os.path.exists(p):
                shutil.copy(p, dst)
        with open(os.path.join(dst, "generator.log"), "w") as f:
            f.write(res.stdout + res.stderr)
        # the mechanism text the C was emitted from: tests and the bench
        # parse this same text, so that they compare functions of one input
        mdir = os.path.join(dst, "_mech")
        os.makedirs(mdir)
        shutil.copy(mech_path, mdir)
        if therm_path:
            shutil.copy(therm_path, mdir)
    return dst


def mechanism_files(name):
    """(mech_path, therm_path) of the text the emitted C of ``name`` was
    generated from, or None when that build is absent.

    The synthetic generator fits NASA-7 polynomials with LAPACK least
    squares, whose last bits differ between BLAS builds (x86 and Arm), and a
    coefficient printed with nine digits can then round the other way: a text
    regenerated on another host may differ from the one the reference's C
    encodes.  Comparisons against ``RefLib(name)`` therefore parse this
    file."""
    mdir = os.path.join(ref_dir(name), "_mech")
    mp = os.path.join(mdir, name + ".inp")
    tp = os.path.join(mdir, name + "_therm.dat")
    if os.path.exists(mp) and os.path.exists(tp):
        return mp, tp
    return None


def _max_index(text, array):
    idx = [int(m) for m in re.findall(re.escape(array) + r"\[(\d+)\]", text)]
    return max(idx) + 1 if idx else 0


def dims(name):
    """(NSP, NR, NREV, NPM) read from the emitted files themselves."""
    d = ref_dir(name)
    with open(os.path.join(d, "header.h")) as f:
        nsp = int(re.search(r"#define NSP (\d+)", f.read()).group(1))
    with open(os.path.join(d, "rxn_rates.c")) as f:
        rr = f.read()
    nr = _max_index(rr, "fwd_rxn_rates")
    nrev = _max_index(rr, "rev_rxn_rates")
    npm = 0
    p = os.path.join(d, "rxn_rates_pres_mod.c")
    if os.path.exists(p):
        with open(p) as f:
            npm = _max_index(f.read(), "pres_mod")
    return nsp, nr, nrev, npm


def _cc(args, cwd):
    res = subprocess.run(args, cwd=cwd, capture_output=True, text=True)
    return res.returncode, res.stdout + res.stderr


def compile_ref(name, opt_parity=None, opt_fast=None):
    """Build libref.so (parity) and libref_omp.so (timed) for one name.

    Straight-line files of several MB (thousands of reactions) compile with
    -O1 / -O2 to keep the build within a minute or two."""
    d = ref_dir(name)
    big = os.path.getsize(os.path.join(d, "rxn_rates.c")) > 1_000_000
    opt_parity = opt_parity or ("-O1" if big else "-O2")
    opt_fast = opt_fast or ("-O2" if big else "-O3")
    nsp, nr, nrev, npm = dims(name)
    srcs = ["chem_utils.c", "rxn_rates.c", "spec_rates.c"]
    if npm:
        srcs.append("rxn_rates_pres_mod.c")
    harness = os.path.join(HERE, "ref_harness.c")
    defs = ["-DCRS_NSP=%d" % nsp, "-DCRS_NR=%d" % nr,
            "-DCRS_NREV=%d" % nrev, "-DCRS_NPM=%d" % npm]
    base = ["gcc", "-shared", "-fPIC", "-I", d] + defs
    # the parity build evaluates states on OpenMP threads (per-state
    # arithmetic unchanged), so that tests can pin millions of states
    jobs = [(base + [opt_parity, "-ffp-contract=off", "-fopenmp", "-o", "libref.so"]
             + srcs + [harness, "-lm"]),
            (base + [opt_fast, "-fopenmp", "-o", "libref_omp.so"]
             + srcs + [harness, "-lm"])]
    if os.path.exists(os.path.join(d, "dydt.c")):
        # the emitted constant-pressure dydt (its CONV branch does not compile)
        jobs.append(base + ["-DCONP", opt_parity, "-ffp-contract=off", "-o",
                            "libref_dydt.so"] + srcs
                    + ["dydt.c", os.path.join(HERE, "ref_dydt_harness.c"), "-lm"])
    procs = [subprocess.Popen(j, cwd=d, stdout=subprocess.PIPE,
                              stderr=subprocess.STDOUT, text=True)
             for j in jobs]
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s" % (" ".join(j), out))
    return os.path.join(d, "libref.so"), os.path.join(d, "libref_omp.so")


def have_sources(name):
    d = ref_dir(name)
    return all(os.path.exists(os.path.join(d, f))
               for f in ("chem_utils.c", "rxn_rates.c", "spec_rates.c",
                         "header.h"))


def reference_available():
    """True when the reference checkout that ``generate`` reads exists."""
    return os.path.isdir(REFERENCE)


def main(argv):
    if len(argv) == 2 and argv[1] == "available":
        return 0 if reference_available() else 1
    if len(argv) < 3 or argv[1] not in ("generate", "compile", "all"):
        print(__doc__)
        return 2
    sys.path.insert(0, REPO)
    from create_rate_subs_gb300 import synth
    for name in argv[2:]:
        if argv[1] in ("generate", "all"):
            tmpdir = tempfile.mkdtemp(prefix="crs_mech_")
            mp, tp = synth.write_mechanism(name, tmpdir)
            generate(name, mp, tp)
            shutil.rmtree(tmpdir)
        if argv[1] in ("compile", "all"):
            print(compile_ref(name))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
