"""Throughput benchmark: species production rates wdot over many states.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {ours,reference}]

Workload (one step): the fused wdot evaluation (eval_conc -> eval_rxn_rates
-> get_rxn_pres_mod -> eval_spec_rates) of the seeded synthetic
53-species / 325-reaction mechanism over 2^20 independent states per GPU,
FP64 structure-of-arrays inputs resident in HBM (898 MB per step, larger
than the 129 MB L2, so no flush is needed).  ``value`` is the plain FP64
kernel's states/s; the same line carries the mixed-precision kernel at
2^22 states with its measured error against the FP64 kernel, the
end-to-end number through the C ABI from pinned host buffers, roofline
fractions, clocks and the CPU baseline.

``--impl reference`` times the reference's own emitted C for the same
mechanism with OpenMP on every host core (compiled by
oracle/build_ref.py; when it is not available, the CPU oracle port).
Under torchrun every rank evaluates its own 2^20 states (weak scaling,
no collective on the data path).
"""

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_STATES = 1 << 20
N_STATES_MIXED = 1 << 22
MECH = "gri53"
METRIC = "wdot states/s (53sp/325rxn) plain FP64 vs mixed & surrogate at stated rel err"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--states", type=int, default=N_STATES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--large-states", type=int, default=1 << 20)
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--sur-train", type=int, default=1 << 24,
                    help="surrogate training states")
    ap.add_argument("--sur-epochs", type=int, default=8)
    ap.add_argument("--sur-eval", type=int, default=1 << 24,
                    help="fresh states the surrogate is evaluated on")
    ap.add_argument("--sur-bound", type=float, default=0.1,
                    help="error bound the surrogate's gate is calibrated for")
    ap.add_argument("--sur-gate-states", type=int, default=1 << 24,
                    help="held-out states the error network is trained on")
    ap.add_argument("--sur-cal-states", type=int, default=1 << 24,
                    help="held-out states the gate threshold is calibrated on")
    ap.add_argument("--sur-margin", type=float, default=0.5,
                    help="calibrate for margin x bound on the held-out states")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--profile-surrogate", action="store_true",
                    help="one surrogate network forward pass over 2^20 states "
                         "(the case of the network-kernel ncu summary)")
    ap.add_argument("--profile", action="store_true",
                    help="one launch of each wdot kernel on 2^18 states (for ncu)")
    ap.add_argument("--profile-large", action="store_true",
                    help="one evaluation per mode of the 561-species mechanism on 2^16 "
                         "states (for ncu)")
    return ap.parse_args()


def _mechanism(name=MECH):
    """The synthetic mechanism ``name``.  Where the reference's emitted C of
    it is built (oracle/_ref/<name>/), its Chemkin text is the one that build
    was generated from (oracle/_ref/<name>/_mech/), so that the accuracy
    check and the reference arm see the same mechanism as the timed kernels;
    the generator's least-squares thermo fits can differ in a printed digit
    between hosts."""
    from create_rate_subs_gb300 import synth
    from create_rate_subs_gb300.mechanism import Mechanism
    mdir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle",
                        "_ref", name, "_mech")
    mp = os.path.join(mdir, name + ".inp")
    tp = os.path.join(mdir, name + "_therm.dat")
    if not (os.path.exists(mp) and os.path.exists(tp)):
        mp, tp = synth.write_mechanism(name, tempfile.mkdtemp(prefix="crs_bench_"))
    return Mechanism.from_chemkin(mp, tp)


def _config(n):
    return {"workload": "wdot, synthetic %s mechanism (53 species / 325 reactions: "
                        "30 three-body, 25 Troe, 3 Lindemann, 2 SRI, 20 irreversible), "
                        "plain FP64 kernel" % MECH,
            "n_states_per_gpu": n, "layout": "SoA FP64 T,P,Y[52] in, wdot[53] out",
            "l2": "inputs larger than L2 (%d MB per step)" % (n * 856 // 2**20)}


def _cpu_sample(mech, n_target, seconds=12.0, threads=0, name=MECH, sample=1 << 16):
    """CPU baseline on a bounded sample: the reference's emitted C (OpenMP)
    when built, else the oracle port.  Returns dict for cpu_baseline."""
    from create_rate_subs_gb300 import synth
    from oracle.oracle import Oracle, RefLib
    if RefLib.available(name, omp=True):
        lib, kind = RefLib(name, omp=True), "reference"
    else:
        lib, kind = Oracle(mech.blob), "port"
    n = min(n_target, sample)
    T, P, Y = synth.make_states(mech.n_species, n, seed=777)
    lib.wdot_omp(T, P, Y, nthreads=threads)  # warm-up
    done, t0, used = 0, time.perf_counter(), 1
    while True:
        _, used = lib.wdot_omp(T, P, Y, nthreads=threads)
        done += n
        el = time.perf_counter() - t0
        if el > seconds or done >= n_target:
            break
    return {"value": done / el, "unit": "states/s", "cores": int(used), "kind": kind,
            "sample": "%d states of the same workload (%d passes over %d seeded "
                      "states), %.1f s wall" % (done, done // n, n, el)}


class Clocks(object):
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile(prefix="crs_clk_", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.close()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 7:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        try:
            sm = [float(r[0]) for r in rows]
            mx = float(rows[0][1])
        except ValueError:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def _profile_value(key, kernel):
    """A per-state figure (`key[kernel]: value` line) from the committed ncu
    summaries, if any."""
    d = os.path.join(HERE, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".md"):
            continue
        with open(os.path.join(d, fn)) as f:
            txt = f.read()
        m = re.search(r"^%s\[%s\]:\s*([0-9.eE+-]+)" % (re.escape(key), re.escape(kernel)),
                      txt, re.M)
        if m:
            return float(m.group(1))
    return None


def _traffic_from_profiles(kernel):
    """DRAM bytes per state from the committed ncu summary, if any."""
    return _profile_value("dram_bytes_per_state", kernel)


def _fp64_pipe(kernel, states_per_s, peaks):
    """Executed view of a kernel: FP64 instructions per state (DFMA + DADD +
    DMUL, counted by ncu) x states/s against the measured FP64 issue rate."""
    ops = _profile_value("fp64_ops_per_state", kernel)
    if ops is None:
        return None
    achieved = ops * states_per_s
    return {"ops_per_state": ops, "achieved_gops": achieved / 1e9,
            "peak_gops": peaks["fp64_fma_ops"] / 1e9,
            "frac": achieved / peaks["fp64_fma_ops"],
            "source": "FP64 instructions per state from the ncu capture in "
                      "profiles/wdot_kernels_gri53_262144_states.md; peak = FP64 FMA "
                      "issue rate measured in-run (crs_probe_peaks)"}


def _peaks(lib):
    """In-run issue-rate probes (include/crs_probe.h), operations/s."""
    import ctypes
    from create_rate_subs_gb300 import _lib
    pk = (ctypes.c_double * 5)()
    _lib.check(lib.crs_probe_peaks(pk))
    return dict(fp64_fma_ops=pk[0], fp64_exp=pk[1], fp32_fma_ops=pk[2], sfu_ex2=pk[3],
                fp64_table_exp=pk[4])


def _measured_peak(key, fallback):
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            v = json.load(f).get(key)
        if v:
            return float(v), "of measured"
    except (OSError, ValueError):
        pass
    return fallback, "of fallback"


def _roofline(tables, precision, states_per_s, peaks, n_species, gemm=False):
    """Roofline of one mode: the FP64-pipe work of the arithmetic the mode
    keeps in FP64 (work.fp64_slots: a lower bound in FP64 instruction
    slots, each transcendental priced at the measured cost of the table
    exponential), the state bytes at the measured HBM bandwidth and, for
    the tensor-core contraction, its flops at the measured bf16 peak.  The
    bound is the slowest of them; frac = bound time / measured time."""
    from create_rate_subs_gb300.work import contraction_flops, fp64_slots, state_bytes
    exp_price = peaks["fp64_fma_ops"] / peaks["fp64_table_exp"]
    sl = fp64_slots(tables, precision, exp_price)
    t_fp64 = sl["slots"] / peaks["fp64_fma_ops"]
    hbm, hbm_src = _measured_peak("hbm_gbs", 6800.0)
    sb = state_bytes(n_species)
    if gemm:
        sb += 4 * int(tables["dims"][1])   # the bf16 hi+lo rate row, written once
    t_hbm = sb / (hbm * 1e9)
    t_meas = 1.0 / states_per_s
    out = {"bound": "fp64", "unit": "GFLOP/s",
           "achieved": 2 * sl["slots"] * states_per_s / 1e9,
           "peak": 2 * peaks["fp64_fma_ops"] / 1e9,
           "frac": t_fp64 / t_meas,
           "fp64_slots_per_state": sl["slots"], "slots": sl["parts"],
           "exp_price_slots": exp_price,
           "peak_source": "FP64 FMA issue rate and the table exponential's rate, both "
                          "measured in-run (crs_probe_peaks); one slot = one FP64 "
                          "instruction = 2 flops",
           "per_state_ns": {"fp64_bound": t_fp64 * 1e9, "hbm_bound": t_hbm * 1e9,
                            "measured": t_meas * 1e9},
           "hbm": {"achieved_gbs": sb * states_per_s / 1e9, "peak_gbs": hbm,
                   "frac": sb * states_per_s / 1e9 / hbm, "peak_note": hbm_src,
                   "algorithmic_bytes_per_state": sb}}
    if gemm:
        bf16, bsrc = _measured_peak("bf16_tflops_sustained", 1700.0)
        fl = contraction_flops(tables)
        t_tc = fl / (bf16 * 1e12)
        out["tensor"] = {"flops_per_state": fl, "achieved_tflops": fl * states_per_s / 1e12,
                         "peak_tflops": bf16, "peak_note": "bf16 sustained, " + bsrc,
                         "frac": fl * states_per_s / 1e12 / bf16}
        out["per_state_ns"]["tensor_bound"] = t_tc * 1e9
    bound_t = max(v for k, v in out["per_state_ns"].items() if k != "measured") * 1e-9
    out["bound"] = max((k for k in out["per_state_ns"] if k != "measured"),
                       key=lambda k: out["per_state_ns"][k]).replace("_bound", "")
    out["frac"] = bound_t / t_meas
    return out


def _ref_accuracy(name, mech, T, P, Y, results):
    """Errors of GPU results against the reference's own emitted C for the
    same states (oracle/_ref/<name>/libref.so, the parity build), or the
    CPU oracle (bit-exact to it) when that build is absent.  T, P, Y, and
    each result are host arrays; returns {mode: errors}."""
    from oracle.oracle import Oracle, RefLib, gross_scale, wdot_errors
    if RefLib.available(name):
        lib, src = RefLib(name), "the reference's emitted C (oracle/_ref/%s/libref.so)" % name
    else:
        lib, src = Oracle(mech.blob), "the CPU oracle (bit-exact to the reference's C)"
    ref = lib.eval(T, P, Y, want=("fwd", "rev", "pm", "wdot"))
    G = gross_scale(mech.tables, ref["fwd"], ref["rev"], ref["pm"])
    out = {}
    for mode, w in results.items():
        e = wdot_errors(w, ref["wdot"], G)
        out[mode] = {"scaled_max": e["scaled"], "scaled_rms": e["scaled_rms"],
                     "rel_max_1e-8G": e["rel_1e8"], "rel_max_1e-3G": e["rel_wellcond"],
                     "states": int(T.shape[0]), "against": src}
    return out


ERROR_NOTE = ("scaled_max/rms: |w - w_ref| / G with G_k = sum_r |nu_kr| (|fwd_r| + "
              "|rev_r|) pm_r (the survey's normalisation ii); rel_max_1e-8G: max "
              "|w - w_ref| / |w_ref| over entries with |w_ref| >= 1e-8 G (normalisation "
              "i), rel_max_1e-3G the same over |w_ref| >= 1e-3 G")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    mech = _mechanism()
    # each of the K timed steps is one OpenMP pass over a bounded sample
    from create_rate_subs_gb300 import synth
    from oracle.oracle import Oracle, RefLib
    if RefLib.available(MECH, omp=True):
        lib, kind = RefLib(MECH, omp=True), "reference"
    else:
        lib, kind = Oracle(mech.blob), "port"
    n = 1 << 16
    T, P, Y = synth.make_states(mech.n_species, n, seed=778)
    for _ in range(args.warmup):
        lib.wdot_omp(T, P, Y)
    t0 = time.perf_counter()
    used = 1
    for _ in range(args.steps):
        _, used = lib.wdot_omp(T, P, Y)
    el = time.perf_counter() - t0
    v = n * args.steps / el
    line = {"impl": "reference", "metric": METRIC,
            "value": v, "unit": "states/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": _config(N_STATES),
            "cpu_baseline": {"value": v, "unit": "states/s", "cores": int(used),
                             "kind": kind,
                             "sample": "%d states per step (seeded), %d timed steps"
                                       % (n, args.steps)},
            "e2e": {"value": v, "unit": "states/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _time_steps(fn, steps, warmup, stream, dist):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if dist is not None:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    return ms


def run_ours(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from create_rate_subs_gb300 import _lib, synth
    from create_rate_subs_gb300.rates import RateSubs
    from create_rate_subs_gb300.work import state_bytes, work

    mech = _mechanism()
    rs = RateSubs(mech)
    lib = _lib.load()
    N = mech.n_species
    # weak scaling: the job is one seeded batch of world x --states states;
    # each rank evaluates its slab of it (shard.shard_range), drawn from the
    # slab's own seed, with no collective on the data path
    from create_rate_subs_gb300.shard import shard_range
    a, b_ = shard_range(world * args.states, rank, world)
    n = b_ - a
    T, P, Y = synth.make_states(N, n, seed=1000 + a)
    dT, dP, dY = (torch.from_numpy(a).cuda() for a in (T, P, Y[: N - 1].copy()))
    out = torch.empty((N, n), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    import ctypes
    peaks = _peaks(lib)

    modes = {}
    for m in ("fp64", "fp64_strict", "mixed", "fp64_tps", "mixed_tps", "fp64_warp", "mixed_warp"):
        try:
            rs.wdot(dT[:1024], dP[:1024], dY[:, :1024], mode=m)
            modes[m] = True
        except _lib.CRSError as exc:
            if exc.code != 4:
                raise
    plain = "fp64" if "fp64" in modes else "fp64_strict"

    rs.reset_status()
    clk = Clocks(local)
    ms = _time_steps(lambda: rs.wdot(dT, dP, dY, plain, out=out), args.steps,
                     args.warmup, stream, dist)
    clocks = clk.stop()
    value = n * world / (ms * 1e-3)
    per_mode = {}
    for m in modes:
        msm = _time_steps(lambda: rs.wdot(dT, dP, dY, m, out=out), max(3, args.steps // 2), 3,
                          stream, dist)
        per_mode[m] = {"value": n * world / (msm * 1e-3), "ms_per_step": msm}
    strict = None
    if plain != "fp64_strict":
        ms_s = _time_steps(lambda: rs.wdot(dT, dP, dY, "fp64_strict", out=out),
                           max(3, args.steps // 2), 3, stream, dist)
        strict = {"value": n * world / (ms_s * 1e-3), "unit": "states/s",
                  "ms_per_step": ms_s,
                  "note": "FP64 in the reference's own operation order (CUDA exp/log/pow, "
                          "divisions), same workload"}

    # accuracy of each mode against the reference's emitted C on a
    # sub-sample of the timed states
    sub = min(n, 1 << 16)
    accuracy = _ref_accuracy(
        MECH, mech, T[:sub], P[:sub], Y[:, :sub],
        {m: rs.wdot(dT[:sub], dP[:sub], dY[:, :sub], m).cpu().numpy() for m in modes})

    # mixed precision at 2^22 states
    mixed = None
    if "mixed" in modes:
        nm = N_STATES_MIXED
        T2, P2, Y2 = synth.make_states(N, nm, seed=2000 + rank)
        mT, mP, mY = (torch.from_numpy(a).cuda() for a in (T2, P2, Y2[: N - 1].copy()))
        mo = torch.empty((N, nm), dtype=torch.float64, device="cuda")
        msm = _time_steps(lambda: rs.wdot(mT, mP, mY, "mixed", out=mo), args.steps,
                          args.warmup, stream, dist)
        ms_plain22 = _time_steps(lambda: rs.wdot(mT, mP, mY, plain, out=mo),
                                 max(3, args.steps // 2), 3, stream, dist)
        subm = 1 << 16
        err22 = _ref_accuracy(
            MECH, mech, T2[:subm], P2[:subm], Y2[:, :subm],
            {"mixed": rs.wdot(mT[:subm], mP[:subm], mY[:, :subm], "mixed").cpu().numpy(),
             plain: rs.wdot(mT[:subm], mP[:subm], mY[:, :subm], plain).cpu().numpy()})
        mixed = {"states": nm, "value": nm * world / (msm * 1e-3), "unit": "states/s",
                 "ms_per_step": msm, "plain_fp64_same_size": nm * world / (ms_plain22 * 1e-3),
                 "speedup_vs_plain": ms_plain22 / msm,
                 "error_vs_reference": err22["mixed"],
                 "plain_error_vs_reference": err22[plain], "error_note": ERROR_NOTE,
                 "roofline": _roofline(mech.tables, "mixed", nm / (msm * 1e-3), peaks, N),
                 "fp64_pipe": _fp64_pipe("mixed", nm / (msm * 1e-3), peaks)}
        del mT, mP, mY, mo, T2, P2, Y2

    # the ODE right-hand side around wdot (dydt, rate_subs.py:1829-2067)
    ydy = torch.cat([dT[None], dY], dim=0)
    dyo = torch.empty_like(ydy)
    rho = torch.empty_like(dT)
    # the density of each state, for the constant-volume form
    _lib.check(lib.crs_eval_conc_batch(rs.h, n, ctypes.c_void_p(dT.data_ptr()),
                                       ctypes.c_void_p(dP.data_ptr()),
                                       ctypes.c_void_p(dY.data_ptr()), n, None, None,
                                       ctypes.c_void_p(rho.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()),
                                       ctypes.c_void_p(stream.cuda_stream)))
    dydt_res = {}
    for form, arg, conv in (("conp", dP, False), ("conv", rho, True)):
        for m in (plain, "mixed"):
            if m not in modes:
                continue
            msd = _time_steps(lambda: rs.dydt(arg, ydy, conv=conv, mode=m, out=dyo),
                              max(3, args.steps // 2), 3, stream, dist)
            dydt_res["%s_%s" % (form, m)] = {"value": n * world / (msd * 1e-3),
                                             "unit": "states/s", "ms_per_step": msd}
    del ydy, dyo, rho

    # end to end through the C ABI with host buffers: crs_wdot_host on
    # pinned arrays (read and written in place by one launch over the host
    # link; with HOST_STAGED, copied through device buffers in chunks on two
    # streams); host clock around whole calls
    from create_rate_subs_gb300.rates import HOST_STAGED
    hT = torch.from_numpy(T).pin_memory()
    hP = torch.from_numpy(P).pin_memory()
    hY = torch.from_numpy(Y[: N - 1].copy()).pin_memory()
    hW = torch.empty((N, n), dtype=torch.float64).pin_memory()
    hp = lambda t: ctypes.c_void_p(t.data_ptr())
    k_e2e = max(3, args.steps // 2)
    rs.wdot(dT, dP, dY, plain, out=out)
    want = out.cpu().numpy()

    def e2e_time(flag):
        def step():
            _lib.check(lib.crs_wdot_host(rs.h, n, hp(hT), hp(hP), hp(hY), n, hp(hW),
                                         _lib.MODES[plain] | flag))
        hW.fill_(float("nan"))
        for _ in range(3):
            step()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            step()
        torch.cuda.synchronize()
        ms_ = (time.perf_counter() - t0) * 1e3 / k_e2e
        if dist is not None:
            t = torch.tensor([ms_], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms_ = float(t.item())
        return ms_, bool(np.array_equal(hW.numpy(), want))
    ms_e2e, e2e_ok = e2e_time(0)
    ms_staged, staged_ok = e2e_time(HOST_STAGED)
    h2d = (hT.numel() + hP.numel() + hY.numel()) * 8
    d2h = hW.numel() * 8
    del want

    flags, bad = rs.status()
    traffic = _traffic_from_profiles("fp64")
    roof = _roofline(mech.tables, "fp64", value / world, peaks, N)
    roof["traffic"] = traffic * n if traffic is not None else None
    roof["traffic_note"] = ("DRAM bytes per launch: the per-state figure of the ncu capture "
                            "in profiles/ (2^18 states) scaled to this launch's states")
    roof["fp64_pipe"] = _fp64_pipe("fp64", value / world, peaks)
    roof["per_state"] = work(mech.tables)
    line = {
        "metric": METRIC,
        "value": value, "unit": "states/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": _config(n), "plain_mode": plain, "fp64_strict": strict,
        "modes_states_per_s": per_mode,
        "accuracy": accuracy, "accuracy_note": ERROR_NOTE,
        "mixed": mixed,
        "dydt": dydt_res,
        "e2e": {"value": n * world / (ms_e2e * 1e-3), "unit": "states/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": ms_e2e, "matches_device_result": e2e_ok,
                "path": "crs_wdot_host via ctypes on pinned host arrays: one launch reads "
                        "T, P, Y from host memory and writes wdot to it over NVLink-C2C; "
                        "host clock around each call",
                "staged": {"value": n * world / (ms_staged * 1e-3), "unit": "states/s",
                           "ms_per_step": ms_staged, "matches_device_result": staged_ok,
                           "path": "crs_wdot_host with CRS_HOST_STAGED: copies through "
                                   "device buffers, chunks of 2^17 states on two streams"}},
        "gpu_launches": args.steps,
        "roofline": roof,
        "peaks_measured": {k: v / 1e9 for k, v in peaks.items()},
        "status": {"flags": flags, "nonfinite": bad},
        "clocks": clocks,
    }
    del hT, hP, hY, hW
    if not args.no_surrogate:
        del dT, dP, dY, out
        torch.cuda.empty_cache()
        line["surrogate"] = _bench_surrogate(args, rs, stream, dist, world, rank)
        torch.cuda.empty_cache()
    if not args.no_large:
        line["large_mechanism"] = _bench_large(args, stream, dist, world, peaks, rank)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = _cpu_sample(mech, n_target=n, seconds=12.0)
    if rank == 0:
        print(json.dumps(line, default=_jsonable))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def _bench_surrogate(args, rs, stream, dist, world, rank):
    """The learned surrogate on the 53-species mechanism: two networks
    trained by the library's own bf16 kernels on states labelled by the
    exact FP64 kernel, an error network trained on held-out labelled states,
    the gate threshold calibrated for an error bound on further held-out
    states, then evaluation with fallback on fresh states: states/s and the
    error against the exact FP64 kernel on every evaluated state."""
    import torch
    from create_rate_subs_gb300.surrogate import Surrogate
    N = rs.n_species
    B = 16384
    sur = Surrogate(rs, seed=0, batch=B)
    n_tr = (args.sur_train + B - 1) // B * B
    T, P, Y = sur.sample_states(n_tr, seed=5000 + rank)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    losses = sur.fit(states=(T, P, Y), epochs=args.sur_epochs, lr=2e-3, lr_final=2e-5)
    e1.record(stream)
    torch.cuda.synchronize()
    fit_s = e0.elapsed_time(e1) * 1e-3
    del T, P, Y
    torch.cuda.empty_cache()
    e0.record(stream)
    gate_losses = sur.fit_gate(n=args.sur_gate_states, epochs=12, seed=6000 + rank)
    e1.record(stream)
    torch.cuda.synchronize()
    gate_fit_s = e0.elapsed_time(e1) * 1e-3
    # calibration: scores and errors of held-out states, thresholds per bound
    Tc, Pc, Yc = sur.sample_states(args.sur_cal_states, seed=6500 + rank)
    _, g_cal, e_cal = sur.gate_scores(Tc, Pc, Yc)
    del Tc, Pc, Yc
    torch.cuda.empty_cache()
    bound, margin = args.sur_bound, args.sur_margin
    stol = sur.threshold(g_cal, e_cal, margin * bound)
    sur.stol, sur.bound = stol, bound
    net = sur.net
    macs = sum(net.dims[l] * net.dims[l + 1] for l in range(net.L))
    emacs = sum(sur.err_net.dims[l] * sur.err_net.dims[l + 1] for l in range(sur.err_net.L))
    bwd_data = sum(net.dims[l] * net.dims[l + 1] for l in range(1, net.L))
    train_flops_state = 2 * (2 * macs + bwd_data)
    # a timed training pass alone (steps after the fit, same buffers)
    nb = 64
    Xb = torch.randn((B, net.pad[0]), device="cuda").to(torch.bfloat16)
    XTb = Xb.t().contiguous()
    Tgb = torch.randn((B, N), device="cuda")
    Wsave = net.state_dict()
    ms_step = _time_steps(lambda: net.train_step(Xb, XTb, Tgb, 1e-9), nb, 3, stream, dist)
    net.load_state_dict(Wsave)
    # evaluation on fresh states
    ne = args.sur_eval
    Te, Pe, Ye = sur.sample_states(ne, seed=7000 + rank)
    Ye = Ye[: N - 1].contiguous()
    out = torch.empty((N, ne), dtype=torch.float64, device="cuda")
    exact = torch.empty((N, ne), dtype=torch.float64, device="cuda")
    ms_sur = _time_steps(lambda: sur.wdot(Te, Pe, Ye, out=out), 3, 3, stream, dist)
    ms_net = _time_steps(lambda: sur.wdot(Te, Pe, Ye, out=out, with_fallback=False),
                         3, 3, stream, dist)
    ms_plain = _time_steps(lambda: rs.wdot(Te, Pe, Ye, "fp64", out=exact), 3, 3, stream, dist)
    ms_mixed = _time_steps(lambda: rs.wdot(Te, Pe, Ye, "mixed", out=exact), 3, 3, stream, dist)
    # one network's layers alone (features already in X)
    M = (ne + 127) // 128 * 128
    X = torch.zeros((M, net.pad[0]), dtype=torch.bfloat16, device="cuda")
    sur.features(Te, Pe, Ye, ne, ne, X, box=False)
    Yh = torch.empty((ne, net.pad[-1]), dtype=torch.float32, device="cuda")
    ms_fwd = _time_steps(lambda: net.forward(X, ne, Yh), 5, 3, stream, dist)
    ms_inf = _time_steps(lambda: net.infer(X, ne, Yh), 5, 3, stream, dist)
    del X, Yh
    # error of the gated result and of the served network result, every state
    rs.wdot(Te, Pe, Ye, "fp64", out=exact)
    w, nfb = sur.wdot(Te, Pe, Ye, out=out)
    raw, flag, _ = sur._serve(Te, Pe, Ye, tol=0.05)
    e_raw = sur.served_error(raw, exact)
    served = flag == 0

    def q(e):
        if e.numel() == 0:
            return None
        k = torch.sort(e.float()).values
        n_ = k.numel()
        return {"p50": float(k[n_ // 2]), "p90": float(k[int(n_ * 0.9)]),
                "p99": float(k[int(n_ * 0.99)]), "max": float(k[-1])}
    err_gated = q(sur.served_error(w, exact))
    err_raw = q(e_raw)
    err_served = q(e_raw[served])
    # the trade-off: other bounds, each threshold from the same calibration
    sweep = []
    for bd in (0.05, 0.1, 0.2, 0.5):
        st = sur.threshold(g_cal, e_cal, margin * bd)
        mst = _time_steps(lambda: sur.wdot(Te, Pe, Ye, stol=st, out=out), 2, 3, stream, dist)
        wt, nf = sur.wdot(Te, Pe, Ye, stol=st, out=out)
        et = q(sur.served_error(wt, exact))
        sweep.append({"bound": bd, "stol": st, "fallback_fraction": nf / ne,
                      "states_per_s": ne * world / (mst * 1e-3), "error": et,
                      "bound_held": bool(et["max"] <= bd)})
    peak = None
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            peak = json.load(f).get("bf16_tflops")
    except (OSError, ValueError):
        pass
    peak = peak or 1900.0
    fwd_tflops = 2.0 * macs * ne / (ms_fwd * 1e-3) / 1e12
    inf_tflops = 2.0 * macs * ne / (ms_inf * 1e-3) / 1e12
    fused = net.fused_ok()
    res = {
        "network": "2 x MLP %s (served: their mean), SiLU, bf16 weights / fp32 accumulation, "
                   "tcgen05 GEMMs; error network %s"
                   % ("->".join(str(d) for d in net.dims),
                      "->".join(str(d) for d in sur.err_net.dims)),
        "train_states": n_tr, "epochs": args.sur_epochs, "batch": B,
        "train_loss_per_epoch": losses, "fit_seconds": fit_s,
        "gate_fit_states": args.sur_gate_states, "gate_fit_seconds": gate_fit_s,
        "gate_loss_per_epoch": gate_losses,
        "train_step_ms": ms_step,
        "train_states_per_s": B * world / (ms_step * 1e-3),
        "train_tflops": train_flops_state * B / (ms_step * 1e-3) / 1e12,
        "eval_states": ne,
        "bound": bound, "stol": stol,
        "calibration": {"states": int(g_cal.numel()), "margin": margin,
                        "fallback_fraction": 1.0 - float((g_cal <= stol).double().mean()),
                        "rule": "largest score up to which every calibration state has "
                                "error <= margin x bound"},
        "value": ne * world / (ms_sur * 1e-3), "unit": "states/s",
        "ms_per_step": ms_sur,
        "network_only_states_per_s": ne * world / (ms_net * 1e-3),
        "plain_fp64_states_per_s": ne * world / (ms_plain * 1e-3),
        "mixed_states_per_s": ne * world / (ms_mixed * 1e-3),
        "speedup_vs_plain": ms_plain / ms_sur,
        "fallback_fraction": nfb / ne,
        "bound_held": bool(err_gated["max"] <= bound),
        "error_definition": "per state max_k |w_k - w_k,fp64| / (|w_k,fp64| + s_k), "
                            "s_k = std of wdot_k over the training states",
        "error_gated": err_gated, "error_network_all_states": err_raw,
        "error_network_served_states": err_served,
        "bound_sweep": sweep,
        "roofline": {"bound": "tensor",
                     "kernel": ("network inference, all layers in one kernel (crs_mlp_infer)"
                                if fused else "network forward, one tcgen05 GEMM per layer"),
                     "achieved": inf_tflops, "peak": peak, "unit": "TFLOP/s",
                     "frac": inf_tflops / peak, "flops_per_state": 2 * macs,
                     "gated_path_flops_per_state": 2 * (2 * macs + emacs),
                     "peak_note": "bf16 burst, of measured",
                     "layer_by_layer": {"achieved": fwd_tflops, "frac": fwd_tflops / peak,
                                        "ms": ms_fwd},
                     "fused_ms": ms_inf},
    }
    del Te, Pe, Ye, out, exact, w, raw, e_raw, served, wt, g_cal, e_cal
    return res


def _bench_large(args, stream, dist, world, peaks, rank):
    """Large-mechanism configuration: 561 species / 2539 reactions, 2^20
    states; CSR contraction on chip (fp64, mixed) vs the tensor-core
    contraction (gemm); errors against the reference's emitted C on a
    sub-sample; a roofline per mode; the contraction GEMM alone against the
    measured bf16 peak; the reference's C on the host cores beside it."""
    import ctypes
    import torch
    from create_rate_subs_gb300 import _lib, synth
    from create_rate_subs_gb300.mechanism import Mechanism
    from create_rate_subs_gb300.rates import RateSubs
    mech = _mechanism("large561")
    rs = RateSubs(mech)
    N = mech.n_species
    n = args.large_states
    T, P, Y = synth.make_states(N, n, seed=3000)
    dT, dP, dY = (torch.from_numpy(a).cuda() for a in (T, P, Y[: N - 1].copy()))
    out = torch.empty((N, n), dtype=torch.float64, device="cuda")
    res = {"mechanism": "synthetic large561: 561 species / 2539 reactions "
                        "(254 three-body, 127 Troe, 156 irreversible)",
           "n_states": n, "modes": {}}
    sub = 4096
    steps = max(5, args.steps // 2)
    got = {}
    precision = {"fp64": "fp64", "mixed": "mixed_tile", "gemm": "rates"}
    for mode in ("fp64", "mixed", "gemm"):
        ms = _time_steps(lambda: rs.wdot(dT, dP, dY, mode, out=out), steps, 3, stream, dist)
        got[mode] = rs.wdot(dT[:sub], dP[:sub], dY[:, :sub], mode).cpu().numpy()
        sps = n / (ms * 1e-3)
        res["modes"][mode] = {"value": n * world / (ms * 1e-3), "unit": "states/s",
                              "ms_per_step": ms, "timed_steps": steps,
                              "roofline": _roofline(mech.tables, precision[mode], sps, peaks,
                                                    N, gemm=(mode == "gemm"))}
    acc = _ref_accuracy("large561", mech, T[:sub], P[:sub], Y[:, :sub], got)
    for mode in got:
        res["modes"][mode]["error_vs_reference"] = acc[mode]
    res["error_note"] = ERROR_NOTE
    del Y
    # the contraction GEMM alone, at one workspace chunk (2^18 states)
    lib = _lib.load()
    M, Kh = 1 << 18, (mech.n_reactions + 63) // 64 * 64
    K, bn = 2 * Kh, 192
    Np = (N + bn - 1) // bn * bn
    A = torch.randn((M, K), device="cuda").to(torch.bfloat16)
    B = torch.randint(-2, 3, (Np, K), device="cuda").to(torch.bfloat16)
    D = torch.empty((M, Np), device="cuda", dtype=torch.float32)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    st = ctypes.c_void_p(stream.cuda_stream)
    ms = _time_steps(lambda: _lib.check(lib.crs_gemm_bf16(p(A), p(B), p(D), M, Np, K, Np, bn,
                                                          None, st)), 5, 2, stream, dist)
    flops = 2.0 * M * N * (2 * mech.n_reactions)
    peak, psrc = _measured_peak("bf16_tflops", 1900.0)
    res["contraction_gemm"] = {
        "shape": "M=%d states x N=%d species (padded %d) x K=2*%d (bf16 hi+lo, padded %d)"
                 % (M, N, Np, mech.n_reactions, K),
        "ms": ms, "achieved_tflops": flops / (ms * 1e-3) / 1e12, "peak_tflops": peak,
        "frac": flops / (ms * 1e-3) / 1e12 / peak, "peak_note": "bf16 burst, " + psrc,
        "flops_note": "algorithmic 2*M*N*K on the unpadded sizes"}
    del A, B, D, out, dT, dP, dY
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = _cpu_sample(mech, n_target=n, seconds=6.0, name="large561",
                                          sample=1 << 12)
    return res


def _jsonable(o):
    if isinstance(o, (np.integer,)):
        return int(o)
    if isinstance(o, (np.floating,)):
        return float(o)
    raise TypeError(type(o))


def run_profile(args):
    """One launch per mode on 2^18 states: the case the ncu summaries in
    profiles/ were captured on."""
    import torch
    from create_rate_subs_gb300 import synth
    from create_rate_subs_gb300.rates import RateSubs
    torch.cuda.set_device(0)
    mech = _mechanism()
    rs = RateSubs(mech)
    n = 1 << 18
    T, P, Y = synth.make_states(mech.n_species, n, seed=5)
    dT, dP, dY = (torch.from_numpy(a).cuda() for a in (T, P, Y[:-1].copy()))
    out = torch.empty((mech.n_species, n), dtype=torch.float64, device="cuda")
    for mode in ("fp64_strict", "fp64", "mixed", "fp64_tps", "mixed_tps", "fp64_warp", "mixed_warp"):
        rs.wdot(dT, dP, dY, mode, out=out)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "gri53, %d states, one launch per mode" % n,
                      "status": rs.status()}))
    return 0


def run_profile_large(args):
    """One evaluation per large-mechanism mode on 2^16 states: the case of
    the rates-tile ncu summary."""
    import torch
    from create_rate_subs_gb300 import synth
    from create_rate_subs_gb300.mechanism import Mechanism
    from create_rate_subs_gb300.rates import RateSubs
    torch.cuda.set_device(0)
    mech = _mechanism("large561")
    rs = RateSubs(mech)
    n = 1 << 16
    T, P, Y = synth.make_states(mech.n_species, n, seed=5)
    dT, dP, dY = (torch.from_numpy(a).cuda() for a in (T, P, Y[:-1].copy()))
    out = torch.empty((mech.n_species, n), dtype=torch.float64, device="cuda")
    for mode in ("mixed", "gemm"):
        rs.wdot(dT, dP, dY, mode, out=out)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "large561, %d states, one evaluation per mode" % n,
                      "status": rs.status()}))
    return 0


def run_profile_surrogate(args):
    """The surrogate network (random weights) over 2^20 states, once each:
    the gated inference path (k_features, the one-kernel network
    k_mlp_infer, k_output), then the layer-by-layer forward pass that
    training uses (four k_gemm launches with fused bias+SiLU epilogues) on
    the same features."""
    import torch
    from create_rate_subs_gb300.rates import RateSubs
    from create_rate_subs_gb300.surrogate import Surrogate
    torch.cuda.set_device(0)
    rs = RateSubs(_mechanism())
    sur = Surrogate(rs, seed=0)
    n = 1 << 20
    T, P, Y = sur.sample_states(n, seed=5)
    Y = Y[: rs.n_species - 1].contiguous()
    w, nfb = sur.wdot(T, P, Y, tol=float("inf"), with_fallback=False)
    X = torch.zeros((n, sur.net.pad[0]), dtype=torch.bfloat16, device="cuda")
    sur.features(T, P, Y, Y.stride(0), n, X, box=False)
    Yh = torch.empty((n, sur.net.pad[-1]), dtype=torch.float32, device="cuda")
    sur.net.forward(X, n, Yh)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "surrogate network, %d states: gated inference, "
                      "then the layer-by-layer forward" % n}))
    return 0


def main():
    args = _args()
    if args.profile:
        return run_profile(args)
    if args.profile_surrogate:
        return run_profile_surrogate(args)
    if args.profile_large:
        return run_profile_large(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
