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
