"""Batched evaluation of the reference's rate functions on the GPU.

``RateSubs`` is the Python face of libcrs.  It mirrors the four functions
create_rate_subs emits (rate_subs.py:1297-1299, 287-290, 761-763,
1124-1127) -- same names, same arguments, same units -- but each call
evaluates a whole batch of states held on the GPU:

* ``eval_conc(T, P, Y)``          -> (y_N, mw_avg, rho, conc)
* ``eval_rxn_rates(T, P, C)``     -> (fwd, rev)
* ``get_rxn_pres_mod(T, P, C)``   -> pres_mod
* ``eval_spec_rates(fwd, rev, pres_mod)`` -> wdot (row N-1 = dy_N)
* ``wdot(T, P, Y, mode)``         -> the fused hot path
* ``eval_h/u/cv/cp(T)``, ``eval_conc_rho(T, rho, Y)``, ``dydt(P or rho,
  y, conv)`` -> the thermo utilities and ODE right-hand side
  (rate_subs.py:1396-2067)

Arrays are torch CUDA tensors in structure-of-arrays layout: ``T`` and ``P``
have shape (n,), ``Y`` shape (N-1, n) or (N, n) (only the first N-1 rows
are read), per-species / per-reaction outputs shape (rows, n).  Calls are
ordered on torch's current CUDA stream.

``wdot_host`` runs the same evaluation from host arrays (numpy or CPU
tensors) through crs_wdot_host, copies included and overlapped.
"""

import ctypes

import numpy as np

from . import _lib
from .mechanism import Mechanism

HOST_STAGED = 0x100   # crs_wdot_host: chunks through device buffers (CRS_HOST_STAGED)

__all__ = ["RateSubs"]


def _torch():
    import torch
    return torch


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class RateSubs(object):
    """A mechanism staged on the current CUDA device."""

    def __init__(self, mech, device=None):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("RateSubs needs a CUDA device")
        self.lib = _lib.load()
        self.mech = mech if isinstance(mech, Mechanism) else None
        blob = mech.blob if isinstance(mech, Mechanism) else bytes(mech)
        self.device = torch.device("cuda", torch.cuda.current_device()
                                   if device is None else device)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.crs_mech_load(blob, len(blob), ctypes.byref(h)))
        self.h = h
        d = (ctypes.c_int64 * 5)()
        _lib.check(self.lib.crs_mech_dims(h, d))
        self.n_species, self.n_reactions, self.n_rev, self.n_pdep, _ = (int(x) for x in d)

    @classmethod
    def from_chemkin(cls, mech_filename, therm_filename=None, last_spec=None):
        return cls(Mechanism.from_chemkin(mech_filename, therm_filename, last_spec))

    def close(self):
        if getattr(self, "h", None):
            self.lib.crs_mech_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- helpers ---------------------------------------------------------
    def _stream(self):
        return ctypes.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

    def _check_states(self, T, P, Y=None, rows=None):
        torch = _torch()
        for name, a in (("T", T), ("P", P)):
            if a.dtype != torch.float64 or a.dim() != 1 or not a.is_cuda:
                raise ValueError("%s must be a 1-D float64 CUDA tensor" % name)
            if a.stride(0) != 1:
                raise ValueError("%s must be contiguous" % name)
        n = T.shape[0]
        if P.shape[0] != n:
            raise ValueError("T and P differ in length")
        ld = n
        if Y is not None:
            if Y.dtype != torch.float64 or Y.dim() != 2 or not Y.is_cuda:
                raise ValueError("Y must be a 2-D float64 CUDA tensor (species, n)")
            if Y.shape[1] != n or Y.stride(1) != 1:
                raise ValueError("Y must be (species, n) with unit state stride")
            if Y.shape[0] < (rows if rows is not None else self.n_species - 1):
                raise ValueError("Y has too few species rows")
            ld = Y.stride(0)
        return n, ld

    def _out(self, rows, n):
        torch = _torch()
        return torch.empty((max(rows, 0), n), dtype=torch.float64, device=self.device)

    # -- the reference's functions, batched ------------------------------
    def eval_conc(self, T, P, Y):
        n, ld = self._check_states(T, P, Y)
        torch = _torch()
        conc = self._out(self.n_species, n)
        if ld != n:
            Y = Y[: self.n_species - 1].contiguous()
        misc = torch.empty((3, n), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.crs_eval_conc_batch(
            self.h, n, _ptr(T), _ptr(P), _ptr(Y), n, _ptr(misc[0]), _ptr(misc[1]),
            _ptr(misc[2]), _ptr(conc), self._stream()))
        return misc[0], misc[1], misc[2], conc

    def eval_rxn_rates(self, T, P, C):
        n, _ = self._check_states(T, P, C, rows=self.n_species)
        C = C.contiguous()
        fwd = self._out(self.n_reactions, n)
        rev = self._out(self.n_rev, n)
        _lib.check(self.lib.crs_eval_rxn_rates_batch(
            self.h, n, _ptr(T), _ptr(P), _ptr(C), n, _ptr(fwd),
            _ptr(rev) if self.n_rev else None, self._stream()))
        return fwd, rev

    def get_rxn_pres_mod(self, T, P, C):
        n, _ = self._check_states(T, P, C, rows=self.n_species)
        C = C.contiguous()
        pm = self._out(self.n_pdep, n)
        if self.n_pdep:
            _lib.check(self.lib.crs_get_rxn_pres_mod_batch(
                self.h, n, _ptr(T), _ptr(P), _ptr(C), n, _ptr(pm), self._stream()))
        return pm

    def eval_spec_rates(self, fwd, rev, pres_mod):
        n = fwd.shape[1]
        fwd = fwd.contiguous()
        rev = rev.contiguous() if rev is not None else None
        pres_mod = pres_mod.contiguous() if pres_mod is not None else None
        w = self._out(self.n_species, n)
        _lib.check(self.lib.crs_eval_spec_rates_batch(
            self.h, n, _ptr(fwd), _ptr(rev) if self.n_rev else None,
            _ptr(pres_mod) if self.n_pdep else None, n, _ptr(w), self._stream()))
        return w

    # -- thermo utilities and the ODE right-hand side (rate_subs.py:1396-2067)
    def _thermo(self, which, T):
        torch = _torch()
        if T.dtype != torch.float64 or T.dim() != 1 or not T.is_cuda or T.stride(0) != 1:
            raise ValueError("T must be a contiguous 1-D float64 CUDA tensor")
        n = T.shape[0]
        out = self._out(self.n_species, n)
        _lib.check(self.lib.crs_eval_thermo_batch(self.h, n, _ptr(T), n, which, _ptr(out),
                                                  self._stream()))
        return out

    def eval_h(self, T):
        """Species enthalpies h (N, n) [J/kg]."""
        return self._thermo(0, T)

    def eval_u(self, T):
        """Species internal energies u (N, n) [J/kg]."""
        return self._thermo(1, T)

    def eval_cv(self, T):
        """Species cv (N, n) [J/(kg K)]."""
        return self._thermo(2, T)

    def eval_cp(self, T):
        """Species cp (N, n) [J/(kg K)]."""
        return self._thermo(3, T)

    def eval_conc_rho(self, T, rho, Y):
        """(y_N, mw_avg, pres, conc) from density, as eval_conc_rho."""
        n, ld = self._check_states(T, rho, Y)
        torch = _torch()
        misc = torch.empty((3, n), dtype=torch.float64, device=self.device)
        conc = self._out(self.n_species, n)
        _lib.check(self.lib.crs_eval_conc_rho_batch(
            self.h, n, _ptr(T), _ptr(rho), _ptr(Y), ld, _ptr(misc[0]), _ptr(misc[1]),
            _ptr(misc[2]), _ptr(conc), self._stream()))
        return misc[0], misc[1], misc[2], conc

    def dydt(self, p_or_rho, y, conv=False, mode="fp64", out=None):
        """dy (N, n) for the emitted state vector y (N, n) = [T; Y_0..Y_{N-2}]:
        constant pressure (p_or_rho = P) or constant volume (conv=True,
        p_or_rho = rho); wdot from `mode`."""
        torch = _torch()
        if y.dtype != torch.float64 or y.dim() != 2 or not y.is_cuda or y.stride(1) != 1:
            raise ValueError("y must be a (species, n) float64 CUDA tensor")
        n = y.shape[1]
        if y.shape[0] != self.n_species or p_or_rho.shape != (n,):
            raise ValueError("y must be (N, n) and p_or_rho (n,)")
        p = p_or_rho.contiguous()
        ld = y.stride(0)
        if out is None:
            out = torch.empty((self.n_species, ld), dtype=torch.float64,
                              device=self.device)[:, :n]
        elif out.stride(0) != ld or out.stride(1) != 1:
            raise ValueError("out must have the row stride of y")
        _lib.check(self.lib.crs_dydt(self.h, n, _ptr(p), _ptr(y), ld, _ptr(out),
                                     int(bool(conv)), _lib.MODES[mode], self._stream()))
        return out

    # -- fused hot path ----------------------------------------------------
    def wdot(self, T, P, Y, mode="fp64", out=None):
        """wdot (N, n) for every state, one launch."""
        n, ld = self._check_states(T, P, Y)
        if out is None:
            out = self._out(self.n_species, n)
            ldw = n
        else:
            ldw = out.stride(0)
        if ldw != ld:
            Y = Y[: self.n_species - 1].contiguous() if ld != n else Y
            if ldw != n:
                raise ValueError("out must be (species, n) contiguous")
            ld = n
        _lib.check(self.lib.crs_wdot(self.h, n, _ptr(T), _ptr(P), _ptr(Y), ld,
                                     _ptr(out), _lib.MODES[mode], self._stream()))
        return out

    def wdot_stages(self, T, P, Y, mode="fp64_strict"):
        """wdot plus conc, fwd, rev, pres_mod from the fused kernel."""
        n, ld = self._check_states(T, P, Y)
        if ld != n:
            Y = Y[: self.n_species - 1].contiguous()
        o = dict(wdot=self._out(self.n_species, n), conc=self._out(self.n_species, n),
                 fwd=self._out(self.n_reactions, n), rev=self._out(self.n_rev, n),
                 pm=self._out(self.n_pdep, n))
        _lib.check(self.lib.crs_wdot_stages(
            self.h, n, _ptr(T), _ptr(P), _ptr(Y), n, _ptr(o["wdot"]), _ptr(o["conc"]),
            _ptr(o["fwd"]), _ptr(o["rev"]) if self.n_rev else None,
            _ptr(o["pm"]) if self.n_pdep else None, _lib.MODES[mode], self._stream()))
        return o

    def wdot_host(self, T, P, Y, mode="fp64", out=None, staged=False):
        """wdot (N, n) from host arrays, through crs_wdot_host.  T, P: (n,),
        Y: (>= N-1, n) float64 numpy arrays or CPU torch tensors; out: same
        kinds, (N, n).  Pinned CPU tensors (all four) are read and written
        in place by one launch over the host link; other arrays, or
        staged=True, pass through the GPU in chunks on two streams, copies
        overlapping kernels.  Returns out (a numpy array when allocated
        here)."""
        torch = _torch()

        def host(a, name, shape0=None):
            if isinstance(a, torch.Tensor):
                if a.is_cuda or a.dtype != torch.float64:
                    raise ValueError("%s must be a float64 CPU tensor" % name)
                if a.stride(-1) != 1:
                    raise ValueError("%s must have unit state stride" % name)
                return a, a.data_ptr(), (a.stride(0) if a.dim() == 2 else 1)
            a = np.asarray(a)
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                a = np.ascontiguousarray(a, dtype=np.float64)
            return a, a.ctypes.data, (a.shape[1] if a.ndim == 2 else 1)

        T, pT, _ = host(T, "T")
        P, pP, _ = host(P, "P")
        Y, pY, ld = host(Y, "Y")
        n = T.shape[0]
        if P.shape[0] != n or Y.shape[1] != n or Y.shape[0] < self.n_species - 1:
            raise ValueError("shapes: T (n,), P (n,), Y (>= N-1, n)")
        if out is None:
            out = np.empty((self.n_species, n))
        out, pW, ldw = host(out, "out")
        if tuple(out.shape) != (self.n_species, n) or ldw != ld:
            raise ValueError("out must be (N, n) with the same row stride as Y")
        with torch.cuda.device(self.device):
            _lib.check(self.lib.crs_wdot_host(self.h, n, ctypes.c_void_p(pT),
                                              ctypes.c_void_p(pP), ctypes.c_void_p(pY), ld,
                                              ctypes.c_void_p(pW),
                                              _lib.MODES[mode] | (HOST_STAGED if staged else 0)))
        return out

    def status(self):
        """(flag bits, count of non-finite wdot values) since the last reset."""
        out = (ctypes.c_int32 * 2)()
        _lib.check(self.lib.crs_status(self.h, self._stream(), out))
        return int(out[0]), int(out[1])

    def reset_status(self):
        _lib.check(self.lib.crs_status_reset(self.h, self._stream()))
