"""Algorithmic cost of one state, counted in the emitted code's own terms.

Used for roofline fractions.  ``state_bytes``: the minimum HBM traffic of
one state at FP64 -- read T, P and N-1 mass fractions, write N production
rates.  ``work``: floating-point operations and transcendental calls that
the reference's emitted C performs for one state (rate_subs.py:283-1391):
eval_conc, eval_rxn_rates, get_rxn_pres_mod, eval_spec_rates.  An FMA
counts 2 flops, a divide 1, a call to exp/log/log10/pow one transcendental.

``fp64_slots``: the FP64-pipe work of one state as a count of FP64
instruction slots, a lower bound for any implementation of the same
arithmetic at the given precision split, so that slots x states/s over
the measured FP64 issue rate cannot exceed 1 unless a kernel skips work.
``contraction_flops``: the tensor-core work of the stoichiometric
contraction of CRS_MODE_GEMM.
"""

from .tables import (FORM_SRI, FORM_TROE, PM_THD, RATE_CONST, RATE_EXP,
                     RATE_NEGEXP, RATE_POW)

__all__ = ["state_bytes", "work", "fp64_slots", "contraction_flops"]


def state_bytes(n_species, elem_bytes=8):
    return elem_bytes * (2 + (n_species - 1)) + elem_bytes * n_species


def _rate(kind, npow):
    """(flops, transcendentals) of one rxn_rate_const expression."""
    if kind == RATE_CONST:
        return 0, 0
    if kind == RATE_EXP:
        return 4, 1          # b*logT, +, Ta/T, -, exp
    if kind == RATE_NEGEXP:
        return 4, 1          # b*logT, Ta/T, -, exp, A*
    if kind == RATE_POW:
        return npow, 0
    # PLOG (two rate rows, two logs, one exp and the interpolation) and
    # Chebyshev (reduced T, P and the dot products, one pow) are counted
    # roughly; no benchmark mechanism uses them
    return 12, 5


def work(tables):
    """dict(flops=..., transcendentals=..., exps=...) for one state."""
    t = tables
    N, R = int(t["dims"][0]), int(t["dims"][1])
    NPM = int(t["dims"][3])
    flops = 5 * N            # eval_conc
    trans = 1                # log(T) in eval_rxn_rates
    for r in range(R):
        f, x = _rate(int(t["rate_kind"][r]), int(t["rate_npow"][r]))
        flops += f
        trans += x
        nr = sum(max(int(v), 1) for v in t["rx_nint"][t["rx_ptr"][r]:t["rx_ptr"][r + 1]])
        flops += nr          # concentration products and the kf factor
        j = int(t["rev_idx"][r])
        if j >= 0:
            ng = int(t["kc_ptr"][j + 1] - t["kc_ptr"][j])
            flops += 13 * ng + (ng - 1) + 1   # Kc polynomial(s), prefactor
            trans += 1                        # exp(Kc)
            npr = sum(max(int(v), 1) for v in t["px_nint"][t["px_ptr"][r]:t["px_ptr"][r + 1]])
            flops += npr + 1                  # products, * kf, / Kc
            flops += 1                        # fwd - rev
        nnz = int(t["nu_ptr"][r + 1] - t["nu_ptr"][r])
        p = int(t["pm_idx"][r])
        for e in range(t["nu_ptr"][r], t["nu_ptr"][r + 1]):
            flops += 1 + (abs(t["nu_val"][e]) != 1.0) + (p >= 0)
        del nnz
    if NPM:
        trans += 1
        flops += 2               # m = P / (RU * T)
    for p in range(NPM):
        ne = int(t["pm_eff_ptr"][p + 1] - t["pm_eff_ptr"][p])
        if int(t["pm_kind"][p]) == PM_THD:
            flops += 2 * ne
            continue
        if int(t["pm_sp"][p]) < 0:
            flops += 2 * ne
        for row in (int(t["pm_k0"][p]), int(t["pm_kinf"][p])):
            f, x = _rate(int(t["rate_kind"][row]), int(t["rate_npow"][row]))
            flops += f
            trans += x
        flops += 2               # Pr
        form = int(t["pm_form"][p])
        if form == FORM_TROE:
            has2 = int(t["pm_troe_t2"][p])
            flops += 5 + 2 * has2 + 3 + 4 + 5
            trans += 2 + has2 + 3 + 1      # exps, 3 log10, pow(10, .)
        elif form == FORM_SRI:
            de = int(t["pm_sri_de"][p])
            flops += 7 + 2 * de
            trans += 2 + 2 + 1 + de        # exps, 2 log10, pow, pow(T, e)
        flops += 3
    return dict(flops=int(flops), transcendentals=int(trans))


def fp64_slots(tables, precision, exp_slots):
    """FP64 instruction slots of one state.

    precision "fp64": every operation of the emitted code in FP64.  The
        algebraic flops count at most two per instruction (as if every
        multiply fused with an add) and each transcendental at
        ``exp_slots``, the measured FP64-pipe cost of the cheapest FP64
        exponential of this library (the table exp: FP64 FMA rate / its
        rate, ~9); logs and powers cost more, so this undercounts.
    precision "mixed": only what the mixed one-state-per-thread kernel
        keeps in FP64: one subtraction (forward - reverse) per reversible
        reaction, one multiply per reaction with a pres_mod term, one FMA
        per nonzero net stoichiometric coefficient (the wdot accumulation).
        Its equilibrium-constant exponents run as float-float on the FP32
        pipe when every reaction has a single T_common group; with several,
        the kernel evaluates the FP64 polynomials, 6 FMAs per group.
    precision "mixed_tile": the mixed split of the large-mechanism state
        tile, which keeps the Kc exponents in FP64 (6 FMAs per T_common
        group) beside the same subtraction, multiplies and accumulation.
    precision "rates": mixed_tile without the accumulation (the rates
        producer of the tensor-core contraction, whose products and sums
        run on the tensor cores).
    Returns dict(slots=..., parts={...}).
    """
    t = tables
    R = int(t["dims"][1])
    NREV = int(t["dims"][2])
    groups = int(t["kc_ptr"][NREV]) if NREV else 0
    nnz = int(t["nu_ptr"][R])
    n_pm = int(sum(1 for r in range(R) if int(t["pm_idx"][r]) >= 0))
    if precision == "fp64":
        w = work(t)
        parts = {"algebraic": w["flops"] / 2.0,
                 "transcendental": w["transcendentals"] * float(exp_slots)}
    elif precision in ("mixed", "mixed_tile", "rates"):
        single = all(int(t["kc_ptr"][j + 1]) - int(t["kc_ptr"][j]) <= 1 for j in range(NREV))
        parts = {"net_rate": float(NREV), "pres_mod_product": float(n_pm)}
        if precision != "mixed" or not single:
            parts["kc_exponent"] = 6.0 * groups
        if precision != "rates":
            parts["accumulation"] = float(nnz)
    else:
        raise ValueError("precision must be fp64, mixed, mixed_tile or rates")
    return {"slots": float(sum(parts.values())), "parts": parts}


def contraction_flops(tables):
    """Tensor-core flops of one state in CRS_MODE_GEMM: the rate row split
    into bf16 hi + lo times the (R x N) stoichiometric matrix,
    2 * 2R * N."""
    N, R = int(tables["dims"][0]), int(tables["dims"][1])
    return 4.0 * R * N
