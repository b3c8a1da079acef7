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


def test_c_target_drop_in_from_a_c_program(tmp_path, golden):
    """The c target's headers with libcrs behind them, used the way an
    integrator uses the reference's emitted C: a C program (gcc, OpenMP)
    includes out/header.h, rates.h and chem_utils.h, binds the mechanism
    loaded from out/mech.crs and calls the four per-state functions by the
    reference's names from several threads; every output equals the
    reference's golden vectors bit for bit."""
    import shutil
    import subprocess
    import numpy as np
    from conftest import REPO
    from create_rate_subs_gb300 import build as crs_build
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    mech, g = golden("features")
    assert _run(tmp_path, "-l", "c", "-i", MECH, "-t", THERM) == 0
    out = tmp_path / "out"
    N, R, NREV, NPM = (int(x) for x in g["dims"][:4])
    n = g["T"].shape[0]
    np.ascontiguousarray(g["T"]).tofile(str(tmp_path / "T.bin"))
    np.ascontiguousarray(g["P"]).tofile(str(tmp_path / "P.bin"))
    np.ascontiguousarray(g["Y"][: N - 1].T).tofile(str(tmp_path / "Y.bin"))  # per state
    src = tmp_path / "drop_in.c"
    src.write_text(r"""
#include <stdio.h>
#include <stdlib.h>
#include "crs.h"
#include "header.h"
#include "rates.h"
#include "chem_utils.h"

static void *slurp(const char *f, size_t *sz) {
  FILE *fp = fopen(f, "rb");
  if (!fp) exit(2);
  fseek(fp, 0, SEEK_END);
  *sz = (size_t)ftell(fp);
  fseek(fp, 0, SEEK_SET);
  void *b = malloc(*sz);
  if (fread(b, 1, *sz, fp) != *sz) exit(2);
  fclose(fp);
  return b;
}

int main(void) {
  size_t sb, st, sp_, sy;
  void *blob = slurp("out/mech.crs", &sb);
  double *T = slurp("T.bin", &st), *P = slurp("P.bin", &sp_), *Y = slurp("Y.bin", &sy);
  const int n = (int)(st / sizeof(double));
  crs_mech *m = NULL;
  if (crs_mech_load_host(blob, sb, &m) != CRS_OK) return 3;
  if (crs_bind(m) != CRS_OK) return 3;
  double *o = malloc(sizeof(double) * (size_t)n * (NSP + NRXN + NRXN_REV + NPDEP + NSP));
  const size_t w = NSP + NRXN + NRXN_REV + NPDEP + NSP;
#pragma omp parallel for schedule(static, 1)
  for (int i = 0; i < n; ++i) {
    double *conc = o + (size_t)i * w, *fwd = conc + NSP, *rev = fwd + NRXN;
    double *pm = rev + NRXN_REV, *sp = pm + NPDEP;
    double y_N, mw, rho;
    eval_conc(T[i], P[i], Y + (size_t)i * (NSP - 1), &y_N, &mw, &rho, conc);
    eval_rxn_rates(T[i], P[i], conc, fwd, rev);
    get_rxn_pres_mod(T[i], P[i], conc, pm);
    eval_spec_rates(fwd, rev, pm, sp, &sp[NSP - 1]);
  }
  FILE *fo = fopen("out.bin", "wb");
  fwrite(o, sizeof(double), (size_t)n * w, fo);
  fclose(fo);
  crs_bind(NULL);
  crs_mech_free(m);
  return 0;
}
""")
    libdir = os.path.dirname(crs_build.build())
    exe = tmp_path / "drop_in"
    cc = subprocess.run([gcc, "-O2", "-fopenmp", "-I", str(out), "-I", os.path.join(REPO, "include"),
                         str(src), "-L", libdir, "-lcrs", "-Wl,-rpath," + libdir, "-o", str(exe)],
                        capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr[-2000:]
    env = dict(os.environ, OMP_NUM_THREADS="4")
    run = subprocess.run([str(exe)], cwd=str(tmp_path), env=env, capture_output=True, text=True)
    assert run.returncode == 0, (run.returncode, run.stderr[-2000:])
    w = N + R + NREV + NPM + N
    o = np.fromfile(str(tmp_path / "out.bin")).reshape(n, w).T
    assert np.array_equal(o[:N], g["conc"])
    assert np.array_equal(o[N:N + R], g["fwd"])
    assert np.array_equal(o[N + R:N + R + NREV], g["rev"])
    assert np.array_equal(o[N + R + NREV:N + R + NREV + NPM], g["pm"])
    assert np.array_equal(o[N + R + NREV + NPM:], g["wdot"])
