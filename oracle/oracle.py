"""ctypes front for the CPU oracle and the reference's emitted C.

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / --impl reference legs import this module.  Nothing in the
create_rate_subs_gb300 package may import it.

* ``Oracle(blob)``: the table-driven restatement (crs_oracle.c), built with
  ``gcc -O2 -ffp-contract=off -fopenmp`` into oracle/liboracle.so.
* ``RefLib(name)``: the reference's emitted C for synthetic mechanism
  ``name``, compiled by oracle/build_ref.py into oracle/_ref/<name>/.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "crs_oracle.c")

_dp = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64
THERMO = {"h": 0, "u": 1, "cv": 2, "cp": 3}


def build(force=False):
    """Compile liboracle.so if missing or older than its source."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC",
           "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True, cwd=HERE)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


class _Batch(object):
    """Common batch helpers over a C library with *_eval / *_wdot_omp."""

    def _outs(self, n, want):
        N, R, NREV, NPM = self.dims[:4]
        shapes = dict(conc=N, fwd=R, rev=NREV, pm=NPM, wdot=N, misc=3)
        return {k: (np.zeros((max(shapes[k], 1), n)) if k in want else None)
                for k in shapes}

    def eval(self, T, P, Y, want=("conc", "fwd", "rev", "pm", "wdot", "misc")):
        """All stages for SoA states; Y has >= N-1 rows of n states."""
        T = np.ascontiguousarray(T, dtype=np.float64)
        P = np.ascontiguousarray(P, dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        n = T.shape[0]
        o = self._outs(n, want)
        rc = self._eval(_i64(n), _ptr(T), _ptr(P), _ptr(Y), _i64(n),
                        _ptr(o["conc"]), _ptr(o["fwd"]), _ptr(o["rev"]),
                        _ptr(o["pm"]), _ptr(o["wdot"]), _ptr(o["misc"]))
        if rc != 0:
            raise RuntimeError("oracle eval failed (%d)" % rc)
        N, R, NREV, NPM = self.dims[:4]
        trim = dict(conc=N, fwd=R, rev=NREV, pm=NPM, wdot=N, misc=3)
        return {k: v[:trim[k]] for k, v in o.items() if v is not None}

    def wdot_omp(self, T, P, Y, nthreads=0, out=None):
        n = T.shape[0]
        if out is None:
            out = np.zeros((self.dims[0], n))
        used = self._omp(_i64(n), _ptr(T), _ptr(P), _ptr(Y), _i64(n),
                         _ptr(out), ctypes.c_int(nthreads))
        return out, used


class Oracle(_Batch):
    """Table-driven FP64 restatement of the emitted code."""

    def __init__(self, blob):
        build()
        self.lib = ctypes.CDLL(LIB)
        L = self.lib
        L.oracle_load.argtypes = [ctypes.c_char_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_void_p)]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_dims.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
        L.oracle_eval.argtypes = [ctypes.c_void_p, _i64, _dp, _dp, _dp, _i64,
                                  _dp, _dp, _dp, _dp, _dp, _dp]
        L.oracle_wdot_omp.argtypes = [ctypes.c_void_p, _i64, _dp, _dp, _dp,
                                      _i64, _dp, ctypes.c_int]
        h = ctypes.c_void_p()
        rc = L.oracle_load(blob, len(blob), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("oracle_load failed (%d)" % rc)
        self.h = h
        d = (ctypes.c_int64 * 5)()
        L.oracle_dims(h, d)
        self.dims = tuple(int(x) for x in d)
        self._eval = lambda *a: L.oracle_eval(self.h, *a)
        self._omp = lambda *a: L.oracle_wdot_omp(self.h, *a)
        L.oracle_dydt_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, _i64, _dp, _dp,
                                        _i64, _dp]
        L.oracle_thermo_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, _i64, _dp,
                                          _i64, _dp]
        L.oracle_conc_rho_batch.argtypes = [ctypes.c_void_p, _i64, _dp, _dp, _dp,
                                            _i64, _dp, _dp]

    def dydt(self, p_or_rho, y, conv=False):
        """dy (N, n) for y (N, n) = [T; Y_0..Y_{N-2}]: constant pressure
        (p_or_rho = P) or constant volume (p_or_rho = rho)."""
        p = np.ascontiguousarray(p_or_rho, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        n = p.shape[0]
        dy = np.zeros((self.dims[0], n))
        rc = self.lib.oracle_dydt_batch(self.h, int(bool(conv)), n, _ptr(p), _ptr(y), n,
                                        _ptr(dy))
        if rc != 0:
            raise RuntimeError("oracle dydt failed (%d)" % rc)
        return dy

    def thermo(self, which, T):
        """which: 'h', 'u', 'cv', 'cp' -> (N, n) at temperatures T."""
        T = np.ascontiguousarray(T, dtype=np.float64)
        out = np.zeros((self.dims[0], T.shape[0]))
        rc = self.lib.oracle_thermo_batch(self.h, THERMO[which], T.shape[0], _ptr(T),
                                          T.shape[0], _ptr(out))
        if rc != 0:
            raise RuntimeError("oracle thermo failed (%d)" % rc)
        return out

    def conc_rho(self, T, rho, Y):
        """(misc (3, n): y_N, mw_avg, pres; conc (N, n)) from density."""
        T = np.ascontiguousarray(T, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        n = T.shape[0]
        misc, conc = np.zeros((3, n)), np.zeros((self.dims[0], n))
        rc = self.lib.oracle_conc_rho_batch(self.h, n, _ptr(T), _ptr(rho), _ptr(Y), n,
                                            _ptr(misc), _ptr(conc))
        if rc != 0:
            raise RuntimeError("oracle conc_rho failed (%d)" % rc)
        return misc, conc

    def __del__(self):
        try:
            self.lib.oracle_free(self.h)
        except Exception:
            pass


class RefLib(_Batch):
    """The reference's emitted C for one synthetic mechanism."""

    def __init__(self, name, omp=False):
        d = os.path.join(HERE, "_ref", name)
        path = os.path.join(d, "libref_omp.so" if omp else "libref.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = L = ctypes.CDLL(path)
        L.ref_dims.argtypes = [ctypes.POINTER(ctypes.c_int64)]
        L.ref_eval.argtypes = [_i64, _dp, _dp, _dp, _i64, _dp, _dp, _dp, _dp,
                               _dp, _dp]
        L.ref_wdot_omp.argtypes = [_i64, _dp, _dp, _dp, _i64, _dp, ctypes.c_int]
        dd = (ctypes.c_int64 * 4)()
        L.ref_dims(dd)
        self.dims = tuple(int(x) for x in dd)
        self._eval = L.ref_eval
        self._omp = L.ref_wdot_omp

    @staticmethod
    def available(name, omp=False):
        return os.path.exists(os.path.join(
            HERE, "_ref", name, "libref_omp.so" if omp else "libref.so"))


class RefDydt(object):
    """The reference's emitted dydt (constant pressure) and thermo
    utilities for one mechanism (oracle/_ref/<name>/libref_dydt.so)."""

    def __init__(self, name):
        path = os.path.join(HERE, "_ref", name, "libref_dydt.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = L = ctypes.CDLL(path)
        L.refd_dydt.argtypes = [_i64, _dp, _dp, _i64, _dp]
        L.refd_thermo.argtypes = [ctypes.c_int, _i64, _dp, _i64, _dp]
        L.refd_conc_rho.argtypes = [_i64, _dp, _dp, _dp, _i64, _dp, _dp]
        self.N = RefLib(name).dims[0]

    @staticmethod
    def available(name):
        return os.path.exists(os.path.join(HERE, "_ref", name, "libref_dydt.so"))

    def dydt(self, P, y):
        P = np.ascontiguousarray(P, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        dy = np.zeros((self.N, P.shape[0]))
        if self.lib.refd_dydt(P.shape[0], _ptr(P), _ptr(y), P.shape[0], _ptr(dy)) != 0:
            raise RuntimeError("refd_dydt failed")
        return dy

    def thermo(self, which, T):
        T = np.ascontiguousarray(T, dtype=np.float64)
        out = np.zeros((self.N, T.shape[0]))
        if self.lib.refd_thermo(THERMO[which], T.shape[0], _ptr(T), T.shape[0],
                                _ptr(out)) != 0:
            raise RuntimeError("refd_thermo failed")
        return out

    def conc_rho(self, T, rho, Y):
        T = np.ascontiguousarray(T, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        n = T.shape[0]
        misc, conc = np.zeros((3, n)), np.zeros((self.N, n))
        if self.lib.refd_conc_rho(n, _ptr(T), _ptr(rho), _ptr(Y), n, _ptr(misc),
                                  _ptr(conc)) != 0:
            raise RuntimeError("refd_conc_rho failed")
        return misc, conc


def nu_abs_matrix(blob_tables):
    """Dense (N, R) matrix of |nu_kr|, the net stoichiometric coefficients
    of the tables' species-rate lists (rate_subs.py:1183-1216)."""
    t = blob_tables
    N, R = int(t["dims"][0]), int(t["dims"][1])
    M = np.zeros((N, R))
    ptr, sp, val = t["nu_ptr"], t["nu_sp"], t["nu_val"]
    for r in range(R):
        for e in range(ptr[r], ptr[r + 1]):
            M[sp[e], r] += abs(val[e])
    return M


def gross_scale(blob_tables, fwd, rev, pm, nu_abs=None):
    """G[k, i] = sum_r |nu_kr| (|fwd_r| + |rev_r|) * pm_r: the scale of the
    terms summed into wdot_k, used to normalise errors where fwd and rev
    cancel.  nu_abs: nu_abs_matrix(blob_tables), when the caller keeps it."""
    t = blob_tables
    R = int(t["dims"][1])
    rev_idx = np.asarray(t["rev_idx"][:R])
    pm_idx = np.asarray(t["pm_idx"][:R])
    g = np.abs(fwd)
    has_rev = rev_idx >= 0
    if np.any(has_rev):
        g[has_rev] += np.abs(rev[rev_idx[has_rev]])
    has_pm = pm_idx >= 0
    if np.any(has_pm):
        g[has_pm] *= np.abs(pm[pm_idx[has_pm]])
    M = nu_abs if nu_abs is not None else nu_abs_matrix(t)
    return M @ g


def wdot_errors(w, w_ref, G):
    """Error report for one result against an FP64 reference.

    Returns dict with
      ``scaled``: max |w - w_ref| / G (G = gross-rate scale), the headline
                  relative error; it stays meaningful where fwd ~ rev;
      ``scaled_rms``: RMS of the same ratio;
      ``rel_wellcond``: max |w - w_ref| / |w_ref| over entries with
                  |w_ref| >= 1e-3 G (cancellation at most 1000x);
      ``rel_1e8``: the same over |w_ref| >= 1e-8 G.
    Entries with G == 0 (species untouched) must match exactly.
    """
    w = np.asarray(w, dtype=np.float64)
    d = np.abs(w - w_ref)
    G = np.asarray(G)
    zero = G == 0
    if np.any(d[zero] != 0):
        return dict(scaled=float("inf"), scaled_rms=float("inf"),
                    rel_wellcond=float("inf"), rel_1e8=float("inf"))
    Gs = np.where(zero, 1.0, G)
    s = d / Gs
    out = dict(scaled=float(np.max(s)) if s.size else 0.0,
               scaled_rms=float(np.sqrt(np.mean(s ** 2))) if s.size else 0.0)
    for key, thr in (("rel_wellcond", 1e-3), ("rel_1e8", 1e-8)):
        m = (~zero) & (np.abs(w_ref) >= thr * G)
        out[key] = float(np.max(d[m] / np.abs(w_ref[m]))) if np.any(m) else 0.0
    return out
