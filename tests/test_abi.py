"""libcrs: it builds, loads, exports every symbol that the C-ABI headers in
include/ (the *.h files with an extern "C" block: crs.h, crs_probe.h)
declare and rejects bad input before touching a GPU (CPU only).  The C++
headers beside them (crs_tables.h, crs_eval.h, crs_device.cuh) hold inline
code that a user's program compiles, not library symbols."""
import ctypes
import glob
import os
import re

import pytest

from conftest import REPO
from create_rate_subs_gb300 import _lib, tables


def header_functions(name=None):
    paths = ([os.path.join(REPO, "include", name)] if name
             else sorted(glob.glob(os.path.join(REPO, "include", "*.h"))))
    fns = set()
    for p in paths:
        with open(p) as f:
            text = f.read()
        if 'extern "C"' not in text:
            continue
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        fns |= set(re.findall(r"\b(\w+)\s*\([^;{]*\)\s*;", text)) - {"defined"}
    return sorted(fns)


def test_header_lists_the_reference_signatures():
    fns = header_functions("crs.h")
    for name in ("eval_conc", "eval_rxn_rates", "get_rxn_pres_mod",
                 "eval_spec_rates", "crs_wdot", "crs_mech_load"):
        assert name in fns


def test_library_exports_every_header_symbol():
    lib = _lib.load()
    fns = header_functions()
    assert "crs_probe_peaks" in fns          # include/crs_probe.h is read too
    assert "crs_state_dydt" in fns and "crs_mech_load_host" in fns
    missing = [f for f in fns if not hasattr(lib, f)]
    assert not missing, missing


def test_bad_blob_rejected_without_gpu():
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.crs_mech_load(b"NOTABLOB" + b"\0" * 64, 72, ctypes.byref(h))
    assert rc == 2
    assert "magic" in _lib.last_error()
    rc = lib.crs_mech_load(None, 0, ctypes.byref(h))
    assert rc == 1


def test_corrupt_index_rejected(golden):
    """A species index out of range in the tables is refused at load time,
    so no kernel can index outside its arrays."""
    mech, _ = golden("small")
    t = dict(mech.tables)
    t["nu_sp"] = t["nu_sp"].copy()
    t["nu_sp"][0] = 999
    blob = tables.pack(t)
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.crs_mech_load(blob, len(blob), ctypes.byref(h)) == 2
    assert "nu species" in _lib.last_error()


def test_per_state_call_without_binding_sets_error():
    lib = _lib.load()
    lib.crs_bind(None)
    out = (ctypes.c_double * 40)()
    lib.eval_rxn_rates(1000.0, 101325.0, out, out, out)
    assert "no mechanism bound" in _lib.last_error()


@pytest.mark.parametrize("case", ["small", "gri53", "features", "features_lastAR"])
def test_inspect_builds_every_table_image(case, golden):
    """crs_mech_inspect builds the device table image on the host (every
    blob section and derived table placed, the staged ranges inside the
    image) for every golden mechanism, PLOG and Chebyshev included."""
    mech, _ = golden(case)
    lib = _lib.load()
    out = (ctypes.c_int64 * 6)()
    assert lib.crs_mech_inspect(mech.blob, len(mech.blob), out) == 0, _lib.last_error()
    image, fp64_staged, mixed_staged = out[0], out[1], out[2]
    assert image > 0 and 0 < fp64_staged <= image and 0 < mixed_staged <= image
    assert image % 16 == 0


def test_inspect_large_mechanism(synth_mech):
    mech = synth_mech("large561")
    lib = _lib.load()
    out = (ctypes.c_int64 * 6)()
    assert lib.crs_mech_inspect(mech.blob, len(mech.blob), out) == 0, _lib.last_error()
    # the 561-species tables do not fit in shared memory: the warp kernels
    # read them through L1 (the per-thread kernels are refused at launch)
    assert out[0] > 227 * 1024


@pytest.mark.parametrize("name", ["small", "gri53"])
def test_mixed_kc_section_is_last_and_outside_strict_staging(name, synth_mech):
    """The mixed kernel's float-float Kc polynomials (128 B per reversible
    reaction) are the image's last section: every other section keeps its
    offset, and the strict kernel stages only the bytes before them
    (crs_mech_inspect out[5] = those bytes + its per-thread columns)."""
    mech = synth_mech(name)
    lib = _lib.load()
    out = (ctypes.c_int64 * 6)()
    assert lib.crs_mech_inspect(mech.blob, len(mech.blob), out) == 0, _lib.last_error()
    strict_staged = out[5] - 2 * mech.n_species * 128 * 8
    assert strict_staged % 16 == 0
    assert out[0] - strict_staged == 128 * mech.n_rev + 16  # the section + its 16 B pad
