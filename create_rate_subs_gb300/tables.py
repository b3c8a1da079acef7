"""Mechanism tables: what the reference prints as literals, as arrays.

create_rate_subs bakes every mechanism constant into unrolled source.  This
module computes the same constants -- with the same host-side arithmetic and
the same decimal rounding of the printed literals -- and stores them as flat
arrays that one table-driven kernel walks for any mechanism.

Where each table comes from in the reference:

* rate constants ``rxn_rate_const``: rate_subs.py:20-135.  Kinds:
  CONST (``A``), EXP (``exp(logA + b*logT - Ta/T)``), NEGEXP
  (``A*exp(b*logT - Ta/T)``, A<0), POW (``A*T*...*T``, A<0 with integral b
  and no E, or an ``int`` b).  ``logA`` is ``math.log(A)``, printed %.16e.
* PLOG (rate_subs.py:444-485): per pressure point a rate row; the branch
  thresholds are the pressures as printed with %.4e, the interpolation
  uses ``math.log(P)`` and the log spacing (printed %.16e, exact).
* Chebyshev (rate_subs.py:136-223): the coefficients and the reduced
  temperature / pressure constants as printed with %.8e.
* Kc groups: rate_subs.py:513-662 (per reaction, species coefficients summed
  on the host and grouped by T_common; prefactor ``(PA/RU)**sum_nu``).
* pressure modification: rate_subs.py:881-1064 (efficiencies as ``eff-1``,
  Troe constants rounded to %.8e, SRI a/b/c/e rounded to 6 significant
  digits and d to %.8e, the ``d*T**e`` factor only when d != 1 and e != 0).
* species rates: rate_subs.py:1158-1226 (net nu per reaction, zero skipped).
* concentrations: rate_subs.py:1295-1391 (``1/mw`` printed %.16e).

The arrays are packed into a self-describing little-endian blob (see
``pack``) that ``crs_mech_load`` in the C library reads.
"""

import math
import struct

import numpy as np

from . import chem
from .utils import get_nu, is_integer

__all__ = ["RATE_CONST", "RATE_EXP", "RATE_NEGEXP", "RATE_POW", "RATE_PLOG", "RATE_CHEB",
           "PM_THD", "PM_FALL_LOW", "PM_FALL_HIGH",
           "FORM_LINDEMANN", "FORM_TROE", "FORM_SRI",
           "build_tables", "pack", "unpack", "BLOB_MAGIC"]

RATE_CONST, RATE_EXP, RATE_NEGEXP, RATE_POW = 0, 1, 2, 3
RATE_PLOG, RATE_CHEB = 4, 5
CHEB_MAX = 16  # most Chebyshev temperature terms the kernels accept
PM_THD, PM_FALL_LOW, PM_FALL_HIGH = 0, 1, 2
FORM_LINDEMANN, FORM_TROE, FORM_SRI = 0, 1, 2

BLOB_MAGIC = b"CRSMECH1"
BLOB_VERSION = 1


def _fmt8(x):
    """A constant as printed with '%.8e' (rate_subs.py:968-991)."""
    return float("{:.8e}".format(x))


def _fmt6(x):
    """A constant as printed with '{:.6}' (rate_subs.py:1020-1037)."""
    return float("{:.6}".format(x))


def rate_record(A, b, E):
    """(kind, npow, A, logA, b, Ta) for one Arrhenius triple.

    Follows the branch structure of rxn_rate_const (rate_subs.py:60-135).
    """
    if A > 0:
        logA = math.log(A)
        if not E and not b:
            return (RATE_CONST, 0, A, logA, 0.0, 0.0)
        if not E and isinstance(b, int):
            return (RATE_POW, max(b, 0), A, logA, 0.0, 0.0)
        return (RATE_EXP, 0, A, logA, float(b), float(E))
    if A < 0:
        if not E and not b:
            return (RATE_CONST, 0, A, 0.0, 0.0, 0.0)
        if not E and is_integer(b):
            return (RATE_POW, max(int(b), 0), A, 0.0, 0.0, 0.0)
        return (RATE_NEGEXP, 0, A, 0.0, float(b), float(E))
    raise NotImplementedError("A == 0 rate constant (the reference raises "
                              "here too, rate_subs.py:132-133)")


def _kc_arrays(sp, nu, factor):
    """Seven Kc coefficients of one species times nu*factor
    (rate_subs.py:370-391; same Python arithmetic, same order)."""
    out = []
    for a in (sp.lo, sp.hi):
        w = nu * factor
        base = [a[6], a[0], a[0] - 1.0, a[1] / 2.0, a[2] / 6.0, a[3] / 12.0,
                a[4] / 20.0, a[5]]
        vals = [base[0] - base[1]] + base[2:]
        out.append([x * w for x in vals])
    return out[0], out[1]


def _kc_groups(rxn, specs):
    """Ordered [(T_mid, lo[7], hi[7])] and sum_nu for one reversible
    reaction (rate_subs.py:513-591): products (net nu) first, then
    reactants absent from the products, grouped by T_common in first-seen
    order."""
    groups = {}
    order = []
    sum_nu = 0

    def add(tmid, lo, hi):
        if tmid not in groups:
            groups[tmid] = (lo, hi)
            order.append(tmid)
        else:
            glo, ghi = groups[tmid]
            groups[tmid] = ([lo[i] + glo[i] for i in range(7)],
                            [hi[i] + ghi[i] for i in range(7)])

    for i, p in enumerate(rxn.prod):
        if p in rxn.reac:
            nu = rxn.prod_nu[i] - rxn.reac_nu[rxn.reac.index(p)]
        else:
            nu = rxn.prod_nu[i]
        if nu == 0:
            continue
        sum_nu += nu
        sp = specs[p]
        lo, hi = _kc_arrays(sp, nu, 1.0)
        add(sp.Trange[1], lo, hi)
    for i, r in enumerate(rxn.reac):
        if r in rxn.prod:
            continue
        nu = rxn.reac_nu[i]
        sum_nu -= nu
        sp = specs[r]
        lo, hi = _kc_arrays(sp, nu, -1.0)
        add(sp.Trange[1], lo, hi)
    return [(t, groups[t][0], groups[t][1]) for t in order], sum_nu


def _stoich(names, nus):
    sp = list(names)
    nu = [float(v) for v in nus]
    nint = [int(v) if is_integer(v) else -1 for v in nus]
    return sp, nu, nint


def build_tables(specs, reacs):
    """Arrays for an ordered mechanism (species indices already assigned).

    Returns a dict name -> numpy array.  See the module docstring for the
    reference lines each table restates.
    """
    N, R = len(specs), len(reacs)
    t = {}
    t["sp_mw"] = np.array([sp.mw for sp in specs], dtype=np.float64)
    t["sp_inv_mw"] = np.array([1.0 / sp.mw for sp in specs], dtype=np.float64)
    t["sp_tmid"] = np.array([sp.Trange[1] for sp in specs], dtype=np.float64)
    t["sp_lo"] = np.array([np.asarray(sp.lo, dtype=np.float64) for sp in specs]).reshape(N, 7)
    t["sp_hi"] = np.array([np.asarray(sp.hi, dtype=np.float64) for sp in specs]).reshape(N, 7)

    rates = []          # rows: (kind, npow, A, logA, b, Ta)
    rx = ([], [], [], [0])
    px = ([], [], [], [0])
    rev_idx, pm_idx = [], []
    kc_ptr, kc_tmid, kc_lo, kc_hi, kc_pref, kc_dnu = [0], [], [], [], [], []
    nu_ptr, nu_sp, nu_val = [0], [], []
    pm = dict(rxn=[], kind=[], form=[], sp=[], eff_ptr=[0], eff_sp=[],
              eff_val=[], k0=[], kinf=[], troe=[], troe_t2=[], sri=[],
              sri_de=[])
    n_rev = n_pm = 0

    rate_aux = []
    plog = dict(ptr=[0], p=[], lp=[], dlp=[], row=[])
    cheb = dict(ptr=[0], nt=[], np=[], par=[], tp=[])
    plog_pending = []
    for r, rxn in enumerate(reacs):
        if rxn.plog:
            rates.append((RATE_PLOG, 0, 0.0, 0.0, 0.0, 0.0))
            rate_aux.append(len(plog["ptr"]) - 1)
            pts = list(rxn.plog_par)
            for i, (P, A, b, E) in enumerate(pts):
                plog["p"].append(float("{:.4e}".format(P)))
                plog["lp"].append(math.log(P))
                plog["dlp"].append(math.log(pts[i + 1][0]) - math.log(P)
                                   if i + 1 < len(pts) else 1.0)
                plog_pending.append((A, b, E))
            plog["ptr"].append(len(plog["p"]))
        elif rxn.cheb:
            nt, npr = int(rxn.cheb_n_temp), int(rxn.cheb_n_pres)
            if nt < 2 or npr < 2 or nt > CHEB_MAX:
                raise NotImplementedError(
                    "reaction %d: Chebyshev needs 2..%d temperature and >= 2 "
                    "pressure terms (the emitted code indexes terms 0 and 1)"
                    % (r, CHEB_MAX))
            rates.append((RATE_CHEB, 0, 0.0, 0.0, 0.0, 0.0))
            rate_aux.append(len(cheb["nt"]))
            par = np.asarray(rxn.cheb_par, dtype=np.float64).reshape(nt, npr)
            cheb["par"].extend(_fmt8(float(x)) for x in par.ravel())
            cheb["ptr"].append(len(cheb["par"]))
            cheb["nt"].append(nt)
            cheb["np"].append(npr)
            t0, t1 = rxn.cheb_tlim
            p0, p1 = rxn.cheb_plim
            cheb["tp"].append([_fmt8(1.0 / t0 + 1.0 / t1), _fmt8(1.0 / t1 - 1.0 / t0),
                               _fmt8(math.log10(p0) + math.log10(p1)),
                               _fmt8(math.log10(p1) - math.log10(p0))])
        else:
            rates.append(rate_record(rxn.A, rxn.b, rxn.E))
            rate_aux.append(-1)
    # the PLOG pressure points' own Arrhenius rows follow the reactions' rows
    for (A, b, E) in plog_pending:
        plog["row"].append(len(rates))
        rates.append(rate_record(A, b, E))
        rate_aux.append(-1)
    for r, rxn in enumerate(reacs):
        for (names, nus, dst) in ((rxn.reac, rxn.reac_nu, rx),
                                  (rxn.prod, rxn.prod_nu, px)):
            sp, nu, nint = _stoich(names, nus)
            dst[0].extend(sp)
            dst[1].extend(nu)
            dst[2].extend(nint)
            dst[3].append(len(dst[0]))

        if rxn.rev:
            if rxn.rev_par:
                raise NotImplementedError("explicit REV parameters must be "
                                          "split by the parser")
            rev_idx.append(n_rev)
            n_rev += 1
            groups, sum_nu = _kc_groups(rxn, specs)
            for tmid, lo, hi in groups:
                kc_tmid.append(tmid)
                kc_lo.append(lo)
                kc_hi.append(hi)
            kc_ptr.append(len(kc_tmid))
            kc_pref.append((chem.PA / chem.RU) ** sum_nu)
            kc_dnu.append(float(sum_nu))
        else:
            rev_idx.append(-1)

        if rxn.thd_body or rxn.pdep:
            pm_idx.append(n_pm)
            n_pm += 1
            pm["rxn"].append(r)
            effs = [(int(s), e - 1.0) for s, e in rxn.thd_body_eff if e != 1.0]
            if rxn.thd_body:
                pm["kind"].append(PM_THD)
                pm["form"].append(FORM_LINDEMANN)
                pm["sp"].append(-1)
                pm["k0"].append(-1)
                pm["kinf"].append(-1)
            else:
                if rxn.low:
                    pm["kind"].append(PM_FALL_LOW)
                    rates.append(rate_record(*rxn.low))
                    rate_aux.append(-1)
                    pm["k0"].append(len(rates) - 1)
                    pm["kinf"].append(r)
                elif rxn.high:
                    pm["kind"].append(PM_FALL_HIGH)
                    rates.append(rate_record(*rxn.high))
                    rate_aux.append(-1)
                    pm["k0"].append(r)
                    pm["kinf"].append(len(rates) - 1)
                else:
                    raise ValueError("reaction %d: fall-off reaction needs a "
                                     "LOW or HIGH line" % r)
                if rxn.pdep_sp == '' or rxn.pdep_sp is None:
                    pm["sp"].append(-1)
                else:
                    pm["sp"].append(int(rxn.pdep_sp))
                    # a named collider uses no efficiencies (rate_subs.py:920-930)
                    effs = []
                if rxn.troe:
                    pm["form"].append(FORM_TROE)
                elif rxn.sri:
                    pm["form"].append(FORM_SRI)
                else:
                    pm["form"].append(FORM_LINDEMANN)
            for s, v in effs:
                pm["eff_sp"].append(s)
                pm["eff_val"].append(v)
            pm["eff_ptr"].append(len(pm["eff_sp"]))

            troe = [0.0] * 5
            has_t2 = 0
            if rxn.pdep and rxn.troe:
                a = rxn.troe_par
                troe[0] = _fmt8(1.0 - a[0])
                troe[1] = _fmt8(a[1]) if a[1] > 0.0 else -_fmt8(abs(a[1]))
                troe[2] = _fmt8(a[0])
                troe[3] = _fmt8(a[2]) if a[2] > 0.0 else -_fmt8(abs(a[2]))
                if len(a) == 4 and a[3] != 0.0:
                    has_t2 = 1
                    troe[4] = _fmt8(a[3]) if a[3] > 0.0 else -_fmt8(abs(a[3]))
            pm["troe"].append(troe)
            pm["troe_t2"].append(has_t2)
            sri = [0.0] * 5
            has_de = 0
            if rxn.pdep and rxn.sri and not rxn.troe:
                a = rxn.sri_par
                sri[0] = _fmt6(a[0])
                sri[1] = _fmt6(a[1]) if a[1] > 0.0 else -_fmt6(abs(a[1]))
                sri[2] = _fmt6(a[2]) if a[2] > 0.0 else -_fmt6(abs(a[2]))
                if len(a) == 5 and a[3] != 1.0 and a[4] != 0.0:
                    has_de = 1
                    sri[3] = _fmt8(a[3])
                    sri[4] = _fmt6(a[4])
            pm["sri"].append(sri)
            pm["sri_de"].append(has_de)
        else:
            pm_idx.append(-1)

        for k in sorted(set(rxn.reac + rxn.prod)):
            nu = get_nu(k, rxn)
            if nu == 0.0:
                continue
            nu_sp.append(k)
            nu_val.append(float(nu))
        nu_ptr.append(len(nu_sp))

    i32 = lambda v: np.asarray(v, dtype=np.int32)
    f64 = lambda v: np.asarray(v, dtype=np.float64)
    t["dims"] = np.array([N, R, n_rev, n_pm, len(rates)], dtype=np.int64)
    t["rate_kind"] = i32([x[0] for x in rates])
    t["rate_npow"] = i32([x[1] for x in rates])
    t["rate_par"] = f64([x[2:] for x in rates]).reshape(len(rates), 4)
    t["rate_aux"] = i32(rate_aux)
    t["plog_ptr"], t["plog_row"] = i32(plog["ptr"]), i32(plog["row"])
    t["plog_p"], t["plog_lp"], t["plog_dlp"] = f64(plog["p"]), f64(plog["lp"]), f64(plog["dlp"])
    t["cheb_ptr"], t["cheb_nt"], t["cheb_np"] = i32(cheb["ptr"]), i32(cheb["nt"]), i32(cheb["np"])
    t["cheb_par"] = f64(cheb["par"])
    t["cheb_tp"] = f64(cheb["tp"]).reshape(len(cheb["nt"]), 4)
    t["rx_ptr"], t["rx_sp"], t["rx_nu"], t["rx_nint"] = i32(rx[3]), i32(rx[0]), f64(rx[1]), i32(rx[2])
    t["px_ptr"], t["px_sp"], t["px_nu"], t["px_nint"] = i32(px[3]), i32(px[0]), f64(px[1]), i32(px[2])
    t["rev_idx"] = i32(rev_idx)
    t["kc_ptr"] = i32(kc_ptr)
    t["kc_tmid"] = f64(kc_tmid)
    t["kc_lo"] = f64(kc_lo).reshape(len(kc_tmid), 7)
    t["kc_hi"] = f64(kc_hi).reshape(len(kc_tmid), 7)
    t["kc_pref"] = f64(kc_pref)
    t["kc_dnu"] = f64(kc_dnu)
    t["pm_idx"] = i32(pm_idx)
    t["pm_rxn"] = i32(pm["rxn"])
    t["pm_kind"] = i32(pm["kind"])
    t["pm_form"] = i32(pm["form"])
    t["pm_sp"] = i32(pm["sp"])
    t["pm_eff_ptr"] = i32(pm["eff_ptr"])
    t["pm_eff_sp"] = i32(pm["eff_sp"])
    t["pm_eff_val"] = f64(pm["eff_val"])
    t["pm_k0"] = i32(pm["k0"])
    t["pm_kinf"] = i32(pm["kinf"])
    t["pm_troe"] = f64(pm["troe"]).reshape(n_pm, 5)
    t["pm_troe_t2"] = i32(pm["troe_t2"])
    t["pm_sri"] = f64(pm["sri"]).reshape(n_pm, 5)
    t["pm_sri_de"] = i32(pm["sri_de"])
    t["nu_ptr"] = i32(nu_ptr)
    t["nu_sp"] = i32(nu_sp)
    t["nu_val"] = f64(nu_val)
    t["names"] = np.frombuffer("\n".join(sp.name for sp in specs).encode(),
                               dtype=np.uint8).copy()
    return t


# ---------------------------------------------------------------------------
# Blob: "CRSMECH1", u32 version, u32 n_sections, then n_sections directory
# entries {char name[24]; u32 dtype; u32 pad; u64 count; u64 offset}, then
# the payloads, each 64-byte aligned.  dtype: 1=f64, 2=i32, 3=i64, 4=u8.
# ---------------------------------------------------------------------------
_DT = {np.dtype(np.float64): 1, np.dtype(np.int32): 2,
       np.dtype(np.int64): 3, np.dtype(np.uint8): 4}
_DT_INV = {v: k for k, v in _DT.items()}
_ENTRY = struct.Struct("<24sIIQQ")


def pack(tables):
    names = sorted(tables)
    head = 16 + _ENTRY.size * len(names)
    off = (head + 63) // 64 * 64
    entries, chunks = [], []
    for name in names:
        arr = np.ascontiguousarray(tables[name])
        code = _DT[arr.dtype]
        raw = arr.tobytes()
        entries.append(_ENTRY.pack(name.encode().ljust(24, b"\0"), code, 0,
                                   arr.size, off))
        chunks.append((off, raw))
        off = (off + len(raw) + 63) // 64 * 64
    buf = bytearray(off)
    buf[0:16] = BLOB_MAGIC + struct.pack("<II", BLOB_VERSION, len(names))
    for i, e in enumerate(entries):
        buf[16 + i * _ENTRY.size:16 + (i + 1) * _ENTRY.size] = e
    for o, raw in chunks:
        buf[o:o + len(raw)] = raw
    return bytes(buf)


def unpack(blob):
    """Inverse of ``pack`` (flat arrays; 2-D tables are reshaped)."""
    if blob[:8] != BLOB_MAGIC:
        raise ValueError("not a mechanism blob")
    ver, n = struct.unpack_from("<II", blob, 8)
    if ver != BLOB_VERSION:
        raise ValueError("unsupported blob version %d" % ver)
    out = {}
    for i in range(n):
        name, code, _, count, off = _ENTRY.unpack_from(blob, 16 + i * _ENTRY.size)
        dt = _DT_INV[code]
        out[name.rstrip(b"\0").decode()] = np.frombuffer(
            blob, dtype=dt, count=count, offset=off).copy()
    for name, w in (("sp_lo", 7), ("sp_hi", 7), ("kc_lo", 7), ("kc_hi", 7),
                    ("rate_par", 4), ("pm_troe", 5), ("pm_sri", 5), ("cheb_tp", 4)):
        if name in out:
            out[name] = out[name].reshape(-1, w)
    return out
