"""The command line: same options as the reference, tables + headers out."""
import ctypes
import os
import re

import pytest

from conftest import GOLDEN
from create_rate_subs_gb300 import _lib, tables
from create_rate_subs_gb300.create_rate_subs import main

MECH = os.path.join(GOLDEN, "features.inp")
THERM = os.path.join(GOLDEN, "features_therm.dat")


def _run(tmp_path, *args):
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        return main(list(args))
    finally:
        os.chdir(cwd)


def test_gb300_target_writes_tables_and_headers(tmp_path):
    assert _run(tmp_path, "-l", "gb300", "-i", MECH, "-t", THERM) == 0
    out = tmp_path / "out"
    for f in ("mech.crs", "header.h", "rates.h", "chem_utils.h", "header.cuh",
              "rates.cuh", "chem_utils.cuh"):
        assert (out / f).exists(), f
    blob = (out / "mech.crs").read_bytes()
    t = tables.unpack(blob)
    assert [int(x) for x in t["dims"][:4]] == [10, 26, 18, 8]
    info = (ctypes.c_int64 * 6)()
    assert _lib.load().crs_mech_inspect(blob, len(blob), info) == 0
    names = re.findall(r"^ \* \d+ (\S+)$", (out / "header.h").read_text(), re.M)
    assert names[-1] == "N2"
    assert "void eval_rxn_rates (const double, const double, const double*, double*, double*);" \
        in (out / "rates.h").read_text()


def test_last_species_is_honoured(tmp_path):
    assert _run(tmp_path, "-l", "c", "-i", MECH, "-t", THERM, "-ls", "AR") == 0
    names = re.findall(r"^ \* \d+ (\S+)$", (tmp_path / "out" / "header.h").read_text(), re.M)
    assert names[-1] == "AR"
    assert not (tmp_path / "out" / "header.cuh").exists()


def test_refusals(tmp_path):
    assert _run(tmp_path, "-l", "fortran", "-i", MECH, "-t", THERM) == 1
    assert _run(tmp_path, "-l", "c", "-i", str(tmp_path / "missing.inp")) == 1
    assert _run(tmp_path, "-l", "c", "-i", "mech.cti") == 1
    with pytest.raises(SystemExit):
        _run(tmp_path, "-l", "java", "-i", MECH)


def test_cuda_target_image_round_trip(tmp_path):
    """The cuda target's mech_image.cuh holds exactly the table image and
    layout libcrs builds for the mechanism (crs_mech_image), and the
    headers it includes are written beside it."""
    import numpy as np
    from create_rate_subs_gb300.create_rate_subs import table_image
    assert _run(tmp_path, "-l", "cuda", "-i", MECH, "-t", THERM) == 0
    out = tmp_path / "out"
    for f in ("mech.crs", "header.cuh", "mech_image.cuh", "rates.cuh", "chem_utils.cuh",
              "dydt.cuh", "crs_device.cuh", "crs_eval.h", "crs_tables.h"):
        assert (out / f).exists(), f
    assert not (out / "rates.h").exists()
    text = (out / "mech_image.cuh").read_text()
    words = [int(w, 16) for w in re.findall(r"0x([0-9a-f]{16})ull", text)]
    img = b"".join(w.to_bytes(8, "little") for w in words)
    lay_block = text.split("crs_mech_layout = {")[1].split("};")[0]
    lay = [int(v) for v in re.findall(r"-?\d+", lay_block)]
    ref_img, ref_lay = table_image((out / "mech.crs").read_bytes())
    assert img[: len(ref_img)] == ref_img and not any(img[len(ref_img):])
    assert lay == ref_lay
    assert np.int32(lay[6]) == len(ref_img)  # ImgLayout.bytes


def test_cuda_target_compiles_into_a_user_kernel(tmp_path):
    """A kernel that calls the reference's per-state functions from the cuda
    target's headers compiles for sm_103a (nvcc cross-compiles; no GPU)."""
    import shutil
    import subprocess
    from create_rate_subs_gb300 import build as crs_build
    try:
        nvcc = crs_build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    assert _run(tmp_path, "-l", "cuda", "-i", MECH, "-t", THERM) == 0
    src = tmp_path / "user.cu"
    src.write_text(
        '#include "rates.cuh"\n#include "chem_utils.cuh"\n#include "dydt.cuh"\n'
        "__global__ void k(const double *T, const double *P, const double *Y, double *w,\n"
        "                  double *dy, double *scratch) {\n"
        "  const int i = threadIdx.x;\n"
        "  double y[NSP], C[NSP], f[NRXN], r[NRXN_REV], p[NPDEP], ys[NSP];\n"
        "  for (int k = 0; k < NSP - 1; ++k) y[k] = Y[k * 32 + i];\n"
        "  double yN, mw, rho;\n"
        "  eval_conc(T[i], P[i], y, &yN, &mw, &rho, C);\n"
        "  eval_rxn_rates(T[i], P[i], C, f, r);\n"
        "  get_rxn_pres_mod(T[i], P[i], C, p);\n"
        "  eval_spec_rates(f, r, p, w + i * NSP, w + i * NSP + NSP - 1);\n"
        "  ys[0] = T[i];\n"
        "  for (int k = 0; k < NSP - 1; ++k) ys[k + 1] = y[k];\n"
        "  dydt(0.0, P[i], ys, dy + i * NSP, scratch + i * crs_device_dydt_scratch());\n"
        "}\n")
    res = subprocess.run([nvcc] + crs_build.ARCH + ["-std=c++17", "-fmad=false", "-I",
                                                    str(tmp_path / "out"), "-c", str(src),
                                                    "-o", str(tmp_path / "user.o")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
