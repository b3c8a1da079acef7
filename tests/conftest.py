"""Shared fixtures: golden cases, mechanisms, the oracle."""
import os
import sys
import tempfile

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")
GOLDEN_CASES = ("small", "gri53", "features", "features_lastAR")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def load_golden(case):
    """(Mechanism, npz) for a golden case; the mechanism text is taken from
    the fixture itself."""
    from create_rate_subs_gb300.mechanism import Mechanism
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    d = tempfile.mkdtemp(prefix="crs_golden_")
    mp, tp = os.path.join(d, "mech.inp"), os.path.join(d, "therm.dat")
    with open(mp, "w") as f:
        f.write(str(g["mech_text"]))
    with open(tp, "w") as f:
        f.write(str(g["therm_text"]))
    last = str(g["last_spec"]) or None
    return Mechanism.from_chemkin(mp, tp, last), g


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(case):
        if case not in cache:
            cache[case] = load_golden(case)
        return cache[case]
    return get


@pytest.fixture(scope="session")
def synth_mech():
    """Mechanism objects of the synthetic workloads, by name.  Where the
    reference's emitted C of a workload is built, the mechanism is parsed
    from the text that C was generated from (oracle.build_ref.
    mechanism_files), so that comparisons with RefLib see one mechanism on
    every host."""
    from create_rate_subs_gb300 import synth
    from create_rate_subs_gb300.mechanism import Mechanism
    from oracle import build_ref
    cache = {}

    def get(name):
        if name not in cache:
            files = build_ref.mechanism_files(name)
            if files is None:
                d = tempfile.mkdtemp(prefix="crs_mech_")
                files = synth.write_mechanism(name, d)
            cache[name] = Mechanism.from_chemkin(*files)
        return cache[name]
    return get


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
