"""Benchmark of the tau-leap simulation + observation log-likelihood.

Workload (default ``abc_smc``): one ABC-SMC generation -- 16384 particles, each
with its own parameters drawn from the priors (R0 U(1.5,4), 1/sigma U(2,6),
1/gamma U(3,8)), over 150 areas x 4 age groups, dt 0.5 day, 180 days (360
steps), SEIR-H-D, daily cases per area and age (108,000 observations).  A
step is one full simulation + log-likelihood of every particle.

  value : particle.area.group.steps/s with the inputs already on the device
          (CUDA events on the model's stream around the kernel launches);
  e2e   : the same through the C ABI from host buffers: re-staging the
          parameter tables into pinned memory, host->device copy, kernels,
          device->host copy of the log-likelihoods, every step (the device
          work of a step replayed as one CUDA graph).
The layout of the fast form is the one the library's autotuner picks on a
sample of the batch (``--no-autotune``: its static rules).  After the main
line's figures the bench measures, on the same GPU, the 350-area x 10-age
precision batch, the serving engine (a 350x10 likelihood stream and the mixed
serving stream at 200 and 4 requests/s), the MBP chains of uneven size (one
fused launch per sweep, and as four launches), the particle filter (one, and
sixteen at once), the ABC-SMC weights, the plain FP64 form and the fast form's
log-likelihood error against FP64 per configuration.

``--impl reference`` times the reference's CPU algorithm for the same
workload on this host's cores (the oracle restatement, all threads, a bounded
sample of particles per step).

usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_UNIT = 72          # int32 state in (6x4 B) + out (6x4 B) + transition counts out (6x4 B)
METRIC = "particle.area.group.steps/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def tensor_peak():
    """Dense BF16 tensor throughput (TFLOP/s): the measured sustained figure for a
    kernel timed inside a long run, else the fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        v = d.get("bf16_tflops_sustained") or d.get("bf16_tflops")
        if v:
            return float(v), "measured sustained"
    return 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during a timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int = 0):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


WORKLOADS = {
    # one ABC-SMC generation: every particle has its own parameters
    "abc_smc": dict(name="abc_smc_generation_150x4", particles=16384),
    # PMCMC likelihood batch on the 350-area x 10-age precision model: one parameter set
    "precision": dict(name="pmcmc_precision_350x10", particles=1024),
}


def build_workload(kind: str, P: int, seed: int):
    """Model + parameter tables of a workload.  The observed data are one
    simulation at the true parameters (made with the library itself, fast
    form) plus noise."""
    from beep_gb300 import capi, model_builder as mb, synth
    w = synth.abc_smc_large() if kind == "abc_smc" else synth.precision_large()
    arr0 = mb.model_arrays(w)
    m0 = capi.Model(arr0)
    t_true = capi.Tables(mb.param_tables(w))
    dm0 = capi.DeviceModel(m0)
    truth = dm0.simulate(capi.Batch(m0, [t_true], 1, seed ^ 0x5EED, want_transnum=True, want_pop_traj=True,
                                    want_L=False, form=capi.FORM_FAST))
    dm0.close()
    rng = np.random.default_rng(seed)
    y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], rng)
    arr = dict(arr0)
    arr["obs_value"], arr["obs_sd"] = y, sd
    m = capi.Model(arr)
    if kind == "abc_smc":
        R0, si, gi = synth.abc_smc_priors(rng, P)
        tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
        group_of = np.arange(P)
    else:
        tabs = [t_true]
        group_of = np.zeros(P, np.int32)
    return w, m, tabs, group_of


def cpu_throughput(m, tabs, group_of, seed, target_s: float, nthreads: int, max_particles: int):
    """Oracle restatement on this host: units/s over a bounded particle sample."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from beep_gb300 import capi
    from oracle_lib import oracle_simulate
    units_per_particle = m.narea * m.nage * m.ndivision
    n = max(1, nthreads)
    def sub(k):
        return (tabs[:k] if len(tabs) > 1 else tabs), group_of[:k]
    t0 = time.perf_counter()
    tb, go = sub(n)
    oracle_simulate(m, capi.Batch(m, tb, n, seed, group_of=go), nthreads)
    dt = time.perf_counter() - t0
    n2 = int(min(max_particles, max(n, n * target_s / max(dt, 1e-3))))
    n2 = max(n, (n2 // n) * n)
    tb, go = sub(n2)
    t0 = time.perf_counter()
    oracle_simulate(m, capi.Batch(m, tb, n2, seed, group_of=go), nthreads)
    dt = time.perf_counter() - t0
    return units_per_particle * n2 / dt, n2, dt


def serve_requests(n: int, seed: int):
    """The serving workload's requests: areas U{10..400}, ages U{1..10},
    horizon U(60, 365) days, dt 0.25 or 0.5, particles log-uniform in
    [64, 8192], kinds likelihood / scenario / prediction in equal shares, the
    10-area recipe's populations and mixing at each size, parameters from the
    ABC-SMC priors (16 parameter sets per request)."""
    from beep_gb300 import capi, model_builder as mb, synth
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(n):
        A = int(rng.integers(10, 401))
        G = int(rng.integers(1, 11))
        days = int(rng.uniform(60, 365))
        spd = int(rng.choice([4, 2]))
        P = int(np.exp(rng.uniform(np.log(64), np.log(8192))))
        kind = int(rng.integers(0, 3))
        w = synth.seir_hd_small(seed=seed + 17 * k, narea=A, nage=G, days=days, steps_per_day=spd, name=f"req{k}")
        m = capi.Model(mb.model_arrays(w))
        ng = min(16, P)
        R0, si, gi = synth.abc_smc_priors(rng, ng)
        tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
        go = np.arange(P) % ng
        ti = 0
        if kind == capi.REQ_LIKELIHOOD:
            b = capi.Batch(m, tabs, P, seed + k, group_of=go, form=capi.FORM_FAST)
        elif kind == capi.REQ_SCENARIO:
            b = capi.Batch(m, tabs, P, seed + k, group_of=go, want_pop=True, form=capi.FORM_FAST)
        else:
            ti = m.ndivision // 2
            p0 = np.rint(m.arr["pop_init"]).astype(np.int32).reshape(1, -1)
            b = capi.Batch(m, tabs, P, seed + k, group_of=go, ti=ti, pop_in=np.repeat(p0, P, 0), want_pop=True,
                           form=capi.FORM_FAST)
        reqs.append(dict(kind=kind, model=m, batch=b, particles=P, units=P * A * G * (m.ndivision - ti),
                         size=f"{A}x{G}x{m.ndivision - ti}"))
    return reqs


def run_serving(nreq: int, rate: float, seed: int, budget_bytes: int, inflight: int):
    """Submits the requests at Poisson arrival times and waits for all."""
    from beep_gb300 import capi
    reqs = serve_requests(nreq, seed)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    srv = capi.Server(budget_bytes, inflight)
    t0 = time.perf_counter()
    tickets = []
    for k, r in enumerate(reqs):
        dt = arrivals[k] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append(srv.submit(r["model"], r["batch"], r["kind"]))
    failed = []
    for k, t in enumerate(tickets):
        try:
            srv.wait(t)
        except capi.BeepError as e:
            # a failed request is reported (and run again alone), the stream's figures are over the others
            r = reqs[k]
            failed.append({"request": k, "kind": r["kind"], "size": r["size"], "particles": r["particles"],
                           "error": str(e)})
    ok = [k for k in range(len(tickets)) if all(f["request"] != k for f in failed)]
    st = [srv.stats(tickets[k]) for k in ok]
    srv.close()
    for f in failed:
        r = reqs[f["request"]]
        dmr = capi.DeviceModel(r["model"])
        try:
            out = dmr.simulate(r["batch"])
            f["alone"] = "ok" if out.L is None or np.all(np.isfinite(out.L)) else "non-finite L"
        except capi.BeepError as e:
            f["alone"] = str(e)
        dmr.close()
    reqs_ok = [reqs[k] for k in ok]
    lat = np.array([s["done_s"] - s["submit_s"] for s in st])
    wait = np.array([s["admit_s"] - s["submit_s"] for s in st])
    svc = np.array([s["gpu_end_s"] - s["gpu_start_s"] for s in st])
    span = max(s["done_s"] for s in st) - min(s["submit_s"] for s in st)
    busy = sorted((s["gpu_start_s"], s["gpu_end_s"]) for s in st)
    overlap = sum(1 for a, b in zip(busy, busy[1:]) if b[0] < a[1])
    for r in reqs_ok:
        assert r["batch"].L is None or np.all(np.isfinite(r["batch"].L))
    units = sum(r["units"] for r in reqs_ok)
    errs = []
    for r in [r for r in reqs if r["kind"] == capi.REQ_LIKELIHOOD][:3]:
        dmr = capi.DeviceModel(r["model"])
        e = fast_loglik_error(dmr, r["model"], r["batch"].tables, np.arange(4) % len(r["batch"].tables), 4, seed)
        dmr.close()
        errs.append(e["max_rel_err_vs_fp64_of_own_trajectory"])
    errs = [e for e in errs if e is not None]
    return {
        "loglik_vs_fp64": {"requests": len(errs), "particles_each": 4,
                           "max_rel_err_vs_fp64_of_own_trajectory": float(max(errs)) if errs else None,
                           "tolerance": 1e-6},
        "requests": nreq, "arrival_rate_per_s": rate, "max_inflight": inflight, "hbm_budget_gb": budget_bytes / 2**30,
        "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "queue_wait_p50_ms": float(np.percentile(wait, 50) * 1e3),
        "queue_wait_p99_ms": float(np.percentile(wait, 99) * 1e3),
        "service_p50_ms": float(np.percentile(svc, 50) * 1e3), "service_p99_ms": float(np.percentile(svc, 99) * 1e3),
        "throughput": units / span, "unit": "particle.area.group.steps/s",
        "loglik_evals_per_s": sum(r["particles"] for r in reqs_ok) / span, "makespan_s": span,
        "overlapping_request_pairs": overlap,
        "failed_requests": failed,
        "kinds": {k: sum(1 for r in reqs if r["kind"] == i) for i, k in enumerate(("likelihood", "scenario",
                                                                                   "prediction"))},
        "form": "fast", "data": "synthetic, generated per request",
    }


def profile_file(kind: str, batched: bool) -> str:
    """The committed ncu summary of the workload's dominant kernel: the
    particle-resident fast kernel (one launch = the whole horizon), or the
    step kernel of the step-synchronous layout (one launch = one step)."""
    if batched:
        return os.path.join(ROOT, "profiles", "bx_step_abc_smc.md" if kind == "abc_smc" else "bx_step_precision.md")
    return os.path.join(ROOT, "profiles", "sim_fast_abc_smc.md" if kind == "abc_smc" else "sim_fast_precision.md")


def profile_figure(kind: str, batched: bool, key: str):
    """A per-particle figure of that summary (per particle and launch), or None."""
    import re
    f = profile_file(kind, batched)
    if not os.path.exists(f):
        return None
    m = re.search(key + r":\s*([0-9.eE+]+)", open(f).read())
    return float(m.group(1)) if m else None


def profile_traffic(kind: str, P: int, batched: bool = False):
    """DRAM bytes per launch of the dominant kernel, from the committed ncu
    summary of the workload (captured on a smaller particle count and scaled
    by the particles, the part of the traffic that grows with them)."""
    v = profile_figure(kind, batched, "dram_bytes_per_particle")
    return v * P if v is not None else None


def fp64_loglik_of_trajectory(m, transnum):
    """The observation log-likelihood of one transition-count trajectory
    [S][A][T][DP] in FP64 (ObservationModel::calculate with normal
    observations, src/obsmodel.cc:22-58,245-305): every observation's count is an
    exact integer sum over its steps and cells -- transition counts, or the
    populations at each step's start rebuilt from the start populations and the
    counts (update_pop, src/state.cc:460-485) -- then its normal log-density.
    None for models with other observation models or censored values."""
    a = m.arr
    S = transnum.shape[0]
    if (a["obs_model"] > 1).any() or (a["obs_value_kind"] != 0).any() or m.nstrain != 1:
        return None                                   # Poisson / negative binomial / censored: not handled here
    tn = transnum.reshape(S, -1).astype(np.int64)
    cum = np.vstack([np.zeros((1, tn.shape[1]), np.int64), np.cumsum(tn, 0)])
    ptr, cells = a["obs_cell_ptr"], a["obs_cells"]
    si, sf = a["obs_sett_i"], a["obs_sett_f"]
    obs_of_cell = np.repeat(np.arange(m.nobs), np.diff(ptr))
    v = np.zeros(m.nobs)
    tm = cells >= 0
    if tm.any():
        oc = obs_of_cell[tm]
        np.add.at(v, oc, (cum[sf[oc], cells[tm]] - cum[si[oc], cells[tm]]).astype(np.float64))
    if (~tm).any():
        A, C, T, DP = m.narea, m.ncomp, m.ntrans, m.ndemocatpos
        frm, to = a["trans_from"], a["trans_to"]
        t4 = transnum.astype(np.int64)                            # [S][A][T][DP]
        flow = np.zeros((S, A, C, DP), np.int64)
        for tr in range(T):
            flow[:, :, frm[tr], :] -= t4[:, :, tr, :]
            flow[:, :, to[tr], :] += t4[:, :, tr, :]
        pop0 = np.rint(a["pop_init"]).astype(np.int64).reshape(1, A, C, DP)
        pops = (pop0 + np.vstack([np.zeros((1, A, C, DP), np.int64), np.cumsum(flow, 0)[:-1]])).reshape(S, -1)
        cpp = np.vstack([np.zeros((1, pops.shape[1]), np.int64), np.cumsum(pops, 0)])
        oc = obs_of_cell[~tm]
        pc = -1 - cells[~tm]
        np.add.at(v, oc, (cpp[sf[oc], pc] - cpp[si[oc], pc]).astype(np.float64))
    v = np.maximum(v * a["obs_factor"], 0.0)
    var = a["obs_sd"] ** 2
    return float(np.sum(-0.5 * np.log(2 * np.pi * var) - (a["obs_value"] - v) ** 2 / (2 * var)))


def fast_loglik_error(dm, m, tabs, group_of, n: int, seed: int):
    """The fast form's log-likelihood against FP64 on n particles: each fast
    trajectory scored in FP64 on the host (largest relative error), and, on
    the same particles and streams, the share that kept the FP64 form's
    trajectory and their largest L difference."""
    from beep_gb300 import capi
    go = None if group_of is None else group_of[:n]
    tb = tabs[:n] if len(tabs) > 1 else tabs
    res = {}
    for f in (capi.FORM_FAST, capi.FORM_PLAIN_FP64):
        res[f] = dm.simulate(capi.Batch(m, tb, n, seed, group_of=go, want_transnum=True, form=f))
    fa, pl = res[capi.FORM_FAST], res[capi.FORM_PLAIN_FP64]
    same = np.array([np.array_equal(fa.transnum[k], pl.transnum[k]) for k in range(n)])
    rel = np.abs(fa.L - pl.L) / np.abs(pl.L)
    l64 = [fp64_loglik_of_trajectory(m, fa.transnum[k]) for k in range(n)]
    own = [abs(fa.L[k] - l64[k]) / abs(l64[k]) for k in range(n) if l64[k] is not None]
    return {"particles": n, "identical_trajectories": float(same.mean()),
            "max_rel_err_identical": float(rel[same].max()) if same.any() else None,
            "max_rel_err_vs_fp64_of_own_trajectory": float(max(own)) if own else None, "tolerance": 1e-6}


def run_particle_filter(reps: int, seed: int, N: int = 256, section_steps: int = 28):
    """PMCMC likelihood estimates: the bootstrap particle filter of the
    10-area x 3-age workload (dt 0.25, 100 days, 400 steps), N particles, one
    parameter set, sections of 28 steps with multinomial resampling and the
    ancestor-state gather on the device between sections.  Estimates per
    second in both forms (each call is one full estimate: host in, estimate
    out)."""
    from beep_gb300 import capi, model_builder as mb, synth
    w = synth.seir_hd_small()
    arr0 = mb.model_arrays(w)
    m0 = capi.Model(arr0)
    t = capi.Tables(mb.param_tables(w))
    dm = capi.DeviceModel(m0)
    truth = dm.simulate(capi.Batch(m0, [t], 1, seed ^ 0x5EED, want_transnum=True, want_pop_traj=True, want_L=False,
                                   form=capi.FORM_FAST))
    dm.close()
    rng = np.random.default_rng(seed)
    y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], rng)
    arr = dict(arr0)
    arr["obs_value"], arr["obs_sd"] = y, sd
    m = capi.Model(arr)
    S = m.ndivision
    sections = [(a, min(a + section_steps, S)) for a in range(0, S, section_steps)]
    dm = capi.DeviceModel(m)
    out = {"workload": "pmcmc_pf_10x3", "particles": N, "steps": S, "sections": len(sections),
           "timing": "host wall clock per estimate (beep_pf_loglik)"}
    out["loglik_vs_fp64"] = fast_loglik_error(dm, m, [t], None, 32, seed)
    for form, name in ((capi.FORM_FAST, "fast"), (capi.FORM_PLAIN_FP64, "plain_fp64")):
        for k in range(2):                                   # warm-up
            dm.pf_loglik(t, N, seed + k, 5, 1.0, sections, form=form)
        est = []
        t0 = time.perf_counter()
        for k in range(reps):
            est.append(dm.pf_loglik(t, N, seed + 100 + k, 5, 1.0, sections, form=form)[0])
        dt = (time.perf_counter() - t0) / reps
        out[name] = {"estimates_per_s": 1.0 / dt, "ms_per_estimate": dt * 1e3,
                     "value": N * m.narea * m.nage * S / dt, "unit": "particle.area.group.steps/s",
                     "loglik_mean": float(np.mean(est)), "loglik_sd": float(np.std(est))}
    dm.close()
    # several independent estimates at once (several PMCMC chains, or several proposals): K
    # filters, each on its own device model and stream driven by its own host thread, their
    # section batches prepared once -- one filter leaves most SMs idle (two particles per
    # SM, a latency-bound chain of steps)
    import threading
    K, R = 16, 8
    dms = [capi.DeviceModel(m) for _ in range(K)]
    for i, d in enumerate(dms):
        d.pf_loglik(t, N, seed + 2000 + i, 5, 1.0, sections, form=capi.FORM_FAST)   # warm-up: section batches
    res = [[] for _ in range(K)]

    def chain(i):
        for r in range(R):
            res[i].append(dms[i].pf_loglik(t, N, seed + 3000 + i * R + r, 5, 1.0, sections, form=capi.FORM_FAST)[0])
    ths = [threading.Thread(target=chain, args=(i,)) for i in range(K)]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    dt = time.perf_counter() - t0
    for d in dms:
        d.close()
    est = [x for r in res for x in r]
    out["fast_concurrent"] = {"filters_in_flight": K, "estimates": K * R, "estimates_per_s": K * R / dt,
                              "value": K * R * N * m.narea * m.nage * S / dt, "unit": "particle.area.group.steps/s",
                              "loglik_mean": float(np.mean(est)),
                              "timing": "host wall clock of 16 host threads, each running 8 estimates on its own model"}
    return out


def run_mbp_chains(sweeps: int, seed: int, nchain: int = 128, plain_sweeps: int = 1):
    """MBP chains of uneven size: nchain chains on each of the models 20x2,
    80x4, 200x6 and 350x10 (areas x ages, dt 0.5, 200 days, weekly hospital
    populations).  A sweep is one coupled proposal per chain (parameters
    perturbed by a factor exp(N(0, 0.05)) per parameter), the FP64 acceptance
    ratio exp(L' - L) (uniform priors, invT = 1) and the accept step.  The fast
    form proposes every chain of the four models in one fused persistent launch
    (beep_mbp_propose_fused); it is also timed with the four models' proposals
    as concurrent launches (one host thread and stream each), as the plain FP64
    form runs."""
    import threading
    from beep_gb300 import capi, model_builder as mb, synth
    rng = np.random.default_rng(seed)
    models = []
    for (A, G) in synth.MBP_SIZES:
        w = synth.mbp_chain_model(A, G)
        arr0 = mb.model_arrays(w)
        m0 = capi.Model(arr0)
        dm0 = capi.DeviceModel(m0)
        truth = dm0.simulate(capi.Batch(m0, [capi.Tables(mb.param_tables(w))], 1, seed ^ A, want_transnum=True,
                                        want_pop_traj=True, want_L=False, form=capi.FORM_FAST))
        dm0.close()
        y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], rng)
        arr = dict(arr0)
        arr["obs_value"], arr["obs_sd"] = y, sd
        m = capi.Model(arr)
        th = np.stack([rng.uniform(2.2, 2.8, nchain), rng.uniform(3.6, 4.4, nchain), rng.uniform(4.5, 5.5, nchain)], 1)
        props = []
        for k in range(2 * sweeps + plain_sweeps):
            tp = th * np.exp(rng.normal(0, 0.05, th.shape))
            props.append([capi.Tables(t) for t in mb.param_tables_batch(w, tp[:, 0], tp[:, 1], tp[:, 2])])
        t0 = [capi.Tables(t) for t in mb.param_tables_batch(w, th[:, 0], th[:, 1], th[:, 2])]
        models.append(dict(w=w, m=m, t0=t0, props=props, units=nchain * A * G * m.ndivision))
    units = sum(x["units"] for x in models)
    out = {}
    runs = (("fast", capi.FORM_FAST, sweeps, True), ("fast_separate_launches", capi.FORM_FAST, sweeps, False),
            ("plain_fp64", capi.FORM_PLAIN_FP64, plain_sweeps, False))
    base = 0
    for name, form, nsw, fused in runs:
        if nsw <= 0:
            continue
        for x in models:
            if x.get("form") != form:
                if "ch" in x:
                    x["ch"].close()
                    x["dm"].close()
                x["dm"] = capi.DeviceModel(x["m"])
                x["ch"] = capi.MbpChains(x["dm"], nchain, form=form)
                x["L"] = x["ch"].initialise(x["t0"], seed, stream_of=np.arange(nchain), group_of=np.arange(nchain))
                x["form"] = form
        acc = []
        times = []
        for k in range(nsw):
            reqs = [dict(tables=x["props"][base + k], seed=seed, group_of=np.arange(nchain),
                         stream_of=np.arange(nchain) + (base + k + 1) * nchain, inf_update=capi.INF_DIF_UPDATE)
                    for x in models]
            res = {}

            def work(i, x):
                res[i] = x["ch"].propose(**reqs[i])
            t0 = time.perf_counter()
            if fused:
                for i, L in enumerate(capi.MbpChains.propose_fused([x["ch"] for x in models], reqs)):
                    res[i] = L
            else:
                th_ = [threading.Thread(target=work, args=(i, x)) for i, x in enumerate(models)]
                for t in th_:
                    t.start()
                for t in th_:
                    t.join()
            for i, x in enumerate(models):
                al = np.minimum(1.0, np.exp(np.clip(res[i] - x["L"], -700, 0)))
                ok = rng.random(nchain) < al
                x["ch"].accept(ok.astype(np.uint8))
                x["L"] = np.where(ok, res[i], x["L"])
                acc.append(ok.mean())
            times.append(time.perf_counter() - t0)
        base += nsw
        if fused:
            # the chains' log-likelihoods against FP64 scoring of their own current trajectories
            x = models[-1]
            errs = []
            for c in range(min(8, nchain)):
                tn_c, _ = x["ch"].read_state(c)
                l64 = fp64_loglik_of_trajectory(x["m"], tn_c)
                if l64 is not None:
                    errs.append(abs(x["L"][c] - l64) / abs(l64))
            out["loglik_vs_fp64"] = {"model": f"{x['m'].narea}x{x['m'].nage}", "chains": len(errs),
                                     "max_rel_err_vs_fp64_of_own_trajectory": float(max(errs)) if errs else None,
                                     "tolerance": 1e-6}
        t = statistics.mean(times)
        out[name] = {"value": units / t, "unit": "chain.area.group.steps/s", "ms_per_sweep": t * 1e3, "sweeps": nsw,
                     "acceptance": float(np.mean(acc)),
                     "launches_per_sweep": 1 if fused else len(models)}
    for x in models:
        if "ch" in x:
            x["ch"].close()
            x["dm"].close()
    out.update({"workload": "mbp_chains_uneven", "chains": 4 * nchain,
                "models": [f"{A}x{G}" for (A, G) in synth.MBP_SIZES], "steps": models[0]["m"].ndivision,
                "units_per_sweep": units, "data": "synthetic, weekly hospital populations",
                "timing": "host wall clock per sweep (proposals of every chain + FP64 acceptance); fast: one "
                          "fused persistent launch per sweep; separate launches / plain: 4 concurrent model streams"})
    return out


def run_precision(seed: int, P: int = 1024, steps: int = 3, warmup: int = 1, plain_particles: int = 304):
    """The 350-area x 10-age PMCMC batch (1460 steps, 1024 particles of one
    parameter set): the fast form in its automatic layout (tensor cores batched
    over the particles), the plain FP64 form on a subset, the fast form's
    log-likelihood error against FP64, and the tensor roofline of the per-step
    force-of-infection products."""
    from beep_gb300 import capi
    w, m, tabs, group_of = build_workload("precision", P, seed)
    dm = capi.DeviceModel(m)
    db = capi.DeviceBatch(dm, capi.Batch(m, tabs, P, seed, group_of=group_of, form=capi.FORM_FAST))
    db.upload()
    db.time(warmup)
    ms = db.time(steps)
    _, k3 = db.time_kernels(1)         # the three kernels' shares, from a separate run with events
    ms_prod = k3[0]
    units = P * m.narea * m.nage * m.ndivision
    out = {"workload": WORKLOADS["precision"]["name"], "particles": P, "areas": m.narea, "ages": m.nage,
           "steps": m.ndivision, "observations": m.nobs,
           "fast": {"value": units / (ms / 1e3), "unit": METRIC, "ms_per_step": ms,
                    "loglik_evals_per_s": P / (ms / 1e3), "launches": db.launches(),
                    "foi": {1: "fp32-simt", 2: "tensor-core per particle", 3: "tensor-core batched"}[db.foi_path()]}}
    if db.foi_path() == 3 and ms_prod > 0:
        # useful work of the area contraction: 2 flops per (source, target) pair per (particle, strain, age) row
        useful = 2.0 * P * m.nstrain * m.nage * m.narea * m.narea * m.ndivision
        tp, tkind = tensor_peak()
        ach = useful / (ms_prod / 1e3) / 1e12
        out["foi_products"] = {"ms_per_step": ms_prod, "share_of_step": ms_prod / ms, "useful_flops_per_launch": useful,
                               "roofline": {"bound": "tensor", "achieved": ach, "peak": tp, "unit": "TFLOP/s",
                                            "frac": ach / tp, "peak_kind": tkind,
                                            "note": "useful flops of the contraction over the product kernels' "
                                                    "time; the kernels issue five split-BF16 products on padded "
                                                    "tiles"}}
    if db.foi_path() == 3:
        out["kernel_split"] = {"product_ms": k3[0], "step_ms": k3[1], "observation_ms": k3[2],
                               "note": "device time per batch run in each of the step's three kernels (CUDA events)"}
        out["step_kernel_issue_roofline"] = issue_roofline("precision", P, k3[1] / 1e3 / m.ndivision, None, True)
    db.close()
    Pp = min(P, plain_particles)
    pb = capi.DeviceBatch(dm, capi.Batch(m, tabs, Pp, seed, group_of=group_of[:Pp], form=capi.FORM_PLAIN_FP64))
    pb.upload()
    pb.time(1)
    pms = pb.time(2)                                     # mean of two launches (4.8 s each)
    pb.close()
    out["plain_fp64"] = {"value": Pp * m.narea * m.nage * m.ndivision / (pms / 1e3), "unit": METRIC,
                         "ms_per_step": pms, "particles": Pp, "loglik_evals_per_s": Pp / (pms / 1e3),
                         "launches_timed": 2}
    out["fast_over_plain_loglik_evals"] = out["fast"]["loglik_evals_per_s"] / out["plain_fp64"]["loglik_evals_per_s"]
    out["loglik_vs_fp64"] = fast_loglik_error(dm, m, tabs, group_of, 12, seed)
    dm.close()
    return out, (w, m, tabs)


def run_serving_precision(nreq: int, seed: int, model, tables, plain_evals_per_s: float, rate: float = 200.0):
    """The serving form on the 350-area x 10-age model: likelihood requests of
    uneven particle counts (log-uniform in [64, 1024]) arriving at `rate` per
    second, admitted as memory and slots free up and run side by side.  Reports
    log-likelihood evaluations per second over the makespan and their ratio to
    the plain FP64 form's."""
    from beep_gb300 import capi
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(nreq):
        P = int(np.exp(rng.uniform(np.log(64), np.log(1024))))
        reqs.append(capi.Batch(model, tables, P, seed + k, group_of=np.zeros(P, np.int32), form=capi.FORM_FAST))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    srv = capi.Server(200 << 30, 8)
    t0 = time.perf_counter()
    tickets = []
    for k, b in enumerate(reqs):
        dt = arrivals[k] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append(srv.submit(model, b, capi.REQ_LIKELIHOOD))
    failed = []
    for k, t in enumerate(tickets):
        try:
            srv.wait(t)
        except capi.BeepError as e:
            # a failed request is reported (and run again alone), the stream's figures are over the others
            r = reqs[k]
            failed.append({"request": k, "kind": r["kind"], "size": r["size"], "particles": r["particles"],
                           "error": str(e)})
    ok = [k for k in range(len(tickets)) if all(f["request"] != k for f in failed)]
    st = [srv.stats(tickets[k]) for k in ok]
    srv.close()
    for f in failed:
        r = reqs[f["request"]]
        dmr = capi.DeviceModel(r["model"])
        try:
            out = dmr.simulate(r["batch"])
            f["alone"] = "ok" if out.L is None or np.all(np.isfinite(out.L)) else "non-finite L"
        except capi.BeepError as e:
            f["alone"] = str(e)
        dmr.close()
    reqs_ok = [reqs[k] for k in ok]
    span = max(x["done_s"] for x in st) - min(x["submit_s"] for x in st)
    lat = np.array([x["done_s"] - x["submit_s"] for x in st])
    svc = np.array([x["gpu_end_s"] - x["gpu_start_s"] for x in st])
    evals = sum(len(b.L) for b in reqs)
    assert all(np.all(np.isfinite(b.L)) for b in reqs)
    return {"requests": nreq, "arrival_rate_per_s": rate, "particles_total": int(evals),
            "loglik_evals_per_s": evals / span, "makespan_s": span,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "service_p50_ms": float(np.percentile(svc, 50) * 1e3),
            "serving_over_plain_loglik_evals": evals / span / plain_evals_per_s,
            "note": "serving-form log-likelihood evaluations/s over the plain FP64 form's on the same model"}


def issue_roofline(kind: str, P: int, t_dev: float, clocks: dict, batched: bool = False):
    """The dominant kernel's instruction-issue roofline: warp instructions per
    launch (per-particle count of the committed ncu capture of the workload,
    times the particles) over the SMs' issue capacity during the launch -- 4
    schedulers per SM, one warp instruction per cycle each, at the median SM
    clock sampled during the timing.  t_dev is the launch's duration.  The
    kernels are bound by their sampler arithmetic, so this, not HBM, is the
    bound that applies."""
    per = profile_figure(kind, batched, "warp_instructions_per_particle")
    if per is None:
        return None
    f = profile_file(kind, batched)
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        sms = 152
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    inst = per * P
    achieved = inst / t_dev
    peak = sms * 4 * mhz * 1e6
    return {"bound": "issue", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "T warp-instructions/s",
            "frac": achieved / peak, "sms": sms, "sm_mhz": mhz,
            "warp_instructions_per_launch": inst, "source": os.path.relpath(f, ROOT)}


def run_abc_weights(seed: int, n: int = 16384, reps: int = 3):
    """beep_abcsmc_weights at the ABC-SMC generation's size: n new against n
    previous particles, three parameters (host wall clock per call, host
    arrays in and out)."""
    from beep_gb300 import capi
    rng = np.random.default_rng(seed)
    lo, hi = np.array([1.5, 2.0, 3.0]), np.array([4.0, 6.0, 8.0])
    tl = rng.uniform(lo, hi, (n, 3))
    wl = rng.uniform(0.2, 2.0, n)
    tn = np.clip(tl[rng.integers(0, n, n)] + rng.normal(0, 0.2, (n, 3)), lo, hi)
    ic = np.linalg.inv(np.cov(tl.T, aweights=wl))
    lp = np.full(n, -np.log(np.prod(hi - lo)))
    capi.abcsmc_weights(tn, lp, tl, wl, ic, 1.3)
    t0 = time.perf_counter()
    for _ in range(reps):
        w = capi.abcsmc_weights(tn, lp, tl, wl, ic, 1.3)
    dt = (time.perf_counter() - t0) / reps
    assert np.all(np.isfinite(w))
    return {"new": n, "previous": n, "parameters": 3, "ms_per_call": dt * 1e3, "pairs_per_s": n * n / dt,
            "timing": "host wall clock per call (host arrays in and out)"}


def max_over_ranks(dist, *times):
    """The slowest rank's times (every rank gets them); identity on one rank."""
    if dist is None:
        return times
    import torch
    tt = torch.tensor(list(times), dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return tuple(float(x) for x in tt)


def units_total(units_per_rank: int, ws: int) -> int:
    """Whole-job units of a weak-scaling run: every rank processes its own batch."""
    return units_per_rank * ws


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, ws, dist
    return 0, 1, None


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    from beep_gb300 import capi  # noqa: F401
    nthreads = os.cpu_count() or 1
    P = args.particles or WORKLOADS[args.workload]["particles"]
    w, m, tabs, group_of = build_workload_cpu(args.workload, P, args.seed)
    upp = m.narea * m.nage * m.ndivision
    # per step a bounded sample sized for a few seconds of work
    _, n2, dt = cpu_throughput(m, tabs, group_of, args.seed, 3.0, nthreads, P)
    times = []
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import oracle_simulate
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle_simulate(m, capi.Batch(m, tabs[:n2] if len(tabs) > 1 else tabs, n2, args.seed + k,
                                      group_of=group_of[:n2]), nthreads)
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    t = statistics.mean(times)
    value = upp * n2 / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "particle.area.group.steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.workload, m, P, note=f"sample of {n2} particles per step"),
        "loglik_evals_per_s": n2 / t,
        "cpu_baseline": {"value": value, "unit": "particle.area.group.steps/s", "cores": nthreads, "kind": "port",
                         "sample": f"{n2} of {P} particles per step, full 360-step horizon + log-likelihood"},
        "e2e": {"value": value, "unit": "particle.area.group.steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def build_workload_cpu(kind, P, seed):
    """The same workload without a GPU: the observed data come from the oracle
    (only used by the reference arm, which runs the oracle anyway)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from beep_gb300 import capi, model_builder as mb, synth
    from oracle_lib import oracle_simulate
    w = synth.abc_smc_large() if kind == "abc_smc" else synth.precision_large()
    arr0 = mb.model_arrays(w)
    m0 = capi.Model(arr0)
    t_true = capi.Tables(mb.param_tables(w))
    truth = oracle_simulate(m0, capi.Batch(m0, [t_true], 1, seed ^ 0x5EED, want_transnum=True, want_pop_traj=True,
                                           want_L=False))
    rng = np.random.default_rng(seed)
    y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], rng)
    arr = dict(arr0)
    arr["obs_value"], arr["obs_sd"] = y, sd
    m = capi.Model(arr)
    if kind == "abc_smc":
        R0, si, gi = synth.abc_smc_priors(rng, P)
        tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
        return w, m, tabs, np.arange(P)
    return w, m, [t_true], np.zeros(P, np.int32)


def workload_config(kind, m, P, note=None):
    c = {"workload": WORKLOADS[kind]["name"], "particles": P, "areas": m.narea, "ages": m.nage,
         "steps": m.ndivision, "dt_days": m.dt, "observations": m.nobs, "model": "SEIR-H-D",
         "l2": "working set larger than L2 (per-particle state and observation sums, GB scale)"}
    if note:
        c["note"] = note
    return c


def run_ours(args, rank, ws, dist):
    from beep_gb300 import build as bbuild, capi
    bbuild.build()
    capi.set_option("fast_foi", {"auto": capi.FOI_AUTO, "simt": capi.FOI_SIMT, "tensor": capi.FOI_TENSOR,
                                 "batched": capi.FOI_BATCHED}[args.foi])
    capi.set_option("fast_ctas_per_sm", args.ctas)
    P = args.particles or WORKLOADS[args.workload]["particles"]
    seed = args.seed + 7919 * rank
    w, m, tabs, group_of = build_workload(args.workload, P, seed)
    dm = capi.DeviceModel(m, device=int(os.environ.get("LOCAL_RANK", "0")) if ws > 1 else 0)
    form = capi.FORM_FAST if args.form == "fast" else capi.FORM_PLAIN_FP64
    batch = capi.Batch(m, tabs, P, seed, group_of=group_of, stream_of=np.arange(P) + rank * P, form=form)
    # the layout (force-of-infection path, particles per SM) chosen by the library's autotuner on
    # a sample of this batch, unless forced by the options
    tuned = None
    if form == capi.FORM_FAST and args.foi == "auto" and args.ctas == 0 and not args.no_autotune:
        t0 = time.perf_counter()
        path = dm.autotune(batch)
        tuned = {"foi_path": path, "seconds": time.perf_counter() - t0,
                 "sample": "up to 64 particles per SM over 90 steps mid-horizon, each fast-form layout timed"}
    db = capi.DeviceBatch(dm, batch)
    h2d, d2h = db.bytes()
    db.upload()
    units = P * m.narea * m.nage * m.ndivision
    # warm-up
    db.time(args.warmup)

    def barrier():
        if dist is not None:
            dist.barrier()

    # device-resident timing
    barrier()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as cs:
        ms = db.time(args.steps)
    clocks = cs.summary()
    t_dev = ms / 1e3
    # end-to-end timing through host buffers
    barrier()
    e2e_times = []
    db.run_graph()                                   # captures the step's device work once
    for k in range(args.steps):
        t0 = time.perf_counter()
        db.run_graph()                               # re-stage tables, replay copies + kernel, unpack L
        e2e_times.append(time.perf_counter() - t0)
    t_e2e = statistics.mean(e2e_times)
    t_dev, t_e2e = max_over_ranks(dist, t_dev, t_e2e)
    assert np.all(np.isfinite(batch.L))
    # the plain FP64 form on a subset of the particles (same workload, units/s)
    plain = None
    if form == capi.FORM_FAST and args.plain_particles > 0:
        Pp = min(P, args.plain_particles)
        tfp = args.plain_steps or m.ndivision
        pb = capi.DeviceBatch(dm, capi.Batch(m, tabs[:Pp] if len(tabs) > 1 else tabs, Pp, seed, group_of=group_of[:Pp],
                                             tf=tfp, form=capi.FORM_PLAIN_FP64))
        pb.upload()
        pb.time(1)
        pms = pb.time(3)                                 # mean of three launches (1.5 s each)
        plain = {"value": Pp * m.narea * m.nage * tfp / (pms / 1e3), "unit": "particle.area.group.steps/s",
                 "ms_per_step": pms, "particles": Pp, "steps": tfp, "launches_timed": 3,
                 "loglik_evals_per_s": Pp / (pms / 1e3) * tfp / m.ndivision}
        pb.close()
    # the fast form's log-likelihood against the FP64 form on the same particles and streams:
    # where the trajectories are identical, the error of the FP32 evaluation itself
    acc = None
    if form == capi.FORM_FAST and args.plain_particles > 0 and rank == 0:
        traj_bytes = 4 * m.ndivision * m.narea * m.ntrans * m.ndemocatpos
        na = int(max(8, min(32, 2e9 // traj_bytes, P)))
        acc = fast_loglik_error(dm, m, tabs, group_of, na, seed)
        acc["note"] = ("particles whose FP32 draws crossed a near tie follow another trajectory; each fast "
                       "trajectory is also scored in FP64 on the host")
    if rank != 0:
        return
    hbm, hbm_kind = peaks()
    batched = db.foi_path() == 3
    if batched:
        # the dominant kernel of the step-synchronous layout is the step kernel: one launch =
        # one step of every particle, timed by CUDA events around each launch
        _, k3 = db.time_kernels(1)
        t_kernel = k3[1] / 1e3 / m.ndivision
        units_launch = P * m.narea * m.nage
        kernels = {"product_ms": k3[0], "step_ms": k3[1], "observation_ms": k3[2],
                   "note": "device time per batch run in each of the step's three kernels (CUDA events)"}
    else:
        t_kernel, units_launch, kernels = t_dev, units, None
    achieved = BYTES_PER_UNIT * units_launch / t_kernel / 1e9
    traffic = profile_traffic(args.workload, P, batched) if args.form == "fast" else None
    mbp = None
    if args.mbp_sweeps > 0 and ws == 1:
        mbp = run_mbp_chains(args.mbp_sweeps, args.seed + 99)
    pf = None
    if args.pf_estimates > 0 and ws == 1:
        pf = run_particle_filter(args.pf_estimates, args.seed + 777)
    serving = None
    if args.serve_requests > 0 and ws == 1:
        serving = run_serving(args.serve_requests, 200.0, args.seed + 4242, 200 << 30, 8)
        if args.serve_sustained > 0:
            serving["sustainable_rate"] = run_serving(args.serve_sustained, args.sustained_rate, args.seed + 4343,
                                                      200 << 30, 8)
    precision = serving_precision = None
    if args.precision_particles > 0 and ws == 1 and args.workload == "abc_smc":
        precision, (_, pm, ptabs) = run_precision(args.seed + 2, args.precision_particles,
                                                  plain_particles=args.precision_plain_particles)
        if args.serve_precision > 0:
            serving_precision = run_serving_precision(args.serve_precision, args.seed + 5151, pm, ptabs,
                                                      precision["plain_fp64"]["loglik_evals_per_s"])
    weights = run_abc_weights(args.seed + 31) if ws == 1 else None
    cpu = None
    if not args.no_cpu:
        nthreads = os.cpu_count() or 1
        v, n2, dt = cpu_throughput(m, tabs, group_of, seed, args.cpu_seconds, nthreads, P)
        cpu = {"value": v, "unit": "particle.area.group.steps/s", "cores": nthreads, "kind": "port",
               "sample": f"{n2} of {P} particles (full 360-step horizon + log-likelihood), {dt:.1f} s"}
    line = {
        "metric": METRIC, "value": units_total(units, ws) / t_dev, "unit": "particle.area.group.steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.form == "fast" else "f64",
        "data": "synthetic", "config": workload_config(args.workload, m, P),
        "form": args.form,
        "foi": {0: None, 1: "fp32-simt", 2: "tensor-core split-bf16 (per particle)",
                3: "tensor-core split-bf16 batched over particles (step-synchronous)"}[db.foi_path()],
        "particles_per_sm": db.ctas_per_sm(),
        "autotuner": tuned,
        "plain_fp64": plain,
        "loglik_vs_fp64": acc,
        "loglik_evals_per_s": P * ws / t_dev,
        "clocks": clocks,
        "e2e": {"value": units_total(units, ws) / t_e2e, "unit": "particle.area.group.steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e * 1e3},
        "gpu_launches": args.steps * db.launches(),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": hbm_kind, "traffic": traffic,
                     "kernel": "bx_step (one step of every particle)" if batched else "sim_fast_kernel (whole horizon)",
                     "algorithmic_bytes": f"{BYTES_PER_UNIT} B x {units_launch} units per launch"},
        "issue_roofline": (issue_roofline(args.workload, P, t_kernel, clocks, batched) if args.form == "fast"
                           else None),
        "kernel_split": kernels,
        "cpu_baseline": cpu,
        "precision_350x10": precision,
        "serving_350x10": serving_precision,
        "serving": serving,
        "mbp_chains": mbp,
        "particle_filter": pf,
        "abc_smc_weights": weights,
        "loglik_vs_fp64_by_config": {
            "C0_pf_10x3": pf.get("loglik_vs_fp64") if pf else None,
            "C1_abc_smc_150x4": acc,
            "C2_precision_350x10": precision.get("loglik_vs_fp64") if precision else None,
            "C3_mbp_350x10": mbp.get("loglik_vs_fp64") if mbp else None,
            "C4_serving": serving.get("loglik_vs_fp64") if serving else None},
    }
    print(json.dumps(line))
    db.close()
    dm.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="abc_smc", choices=sorted(WORKLOADS))
    ap.add_argument("--particles", type=int, default=0, help="default: the workload's particle count")
    ap.add_argument("--seed", type=int, default=20260001)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--form", default="fast", choices=["fast", "plain"])
    ap.add_argument("--ctas", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="particles (CTAs) per SM of the fast form: 0 = automatic, 1 = one, 2..4 = at most that many "
                         "(library option fast_ctas_per_sm)")
    ap.add_argument("--foi", default="auto", choices=["auto", "simt", "tensor", "batched"],
                    help="force of infection of the fast form (library option fast_foi)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the autotuner: the fast form's layout follows the library's static rules")
    ap.add_argument("--plain-particles", type=int, default=1024)
    ap.add_argument("--plain-steps", type=int, default=0, help="time the plain form over this many steps (0: all)")
    ap.add_argument("--mbp-sweeps", type=int, default=6,
                    help="sweeps of the MBP-chain workload (4 x 128 chains of uneven size) after the main measurement")
    ap.add_argument("--pf-estimates", type=int, default=10,
                    help="particle-filter likelihood estimates (256 particles, 10 x 3 model) per form after the main measurement")
    ap.add_argument("--serve-requests", type=int, default=512,
                    help="requests of the serving stream (Poisson arrivals at 200/s) after the main measurement")
    ap.add_argument("--serve-sustained", type=int, default=64,
                    help="requests of the same stream at a rate the GPU sustains (latency without queueing)")
    ap.add_argument("--sustained-rate", type=float, default=4.0,
                    help="arrivals per second of that phase (about 2/3 of the rate the server completes)")
    ap.add_argument("--precision-particles", type=int, default=1024,
                    help="particles of the 350x10 precision batch run after the main measurement (0: skip)")
    ap.add_argument("--precision-plain-particles", type=int, default=152)
    ap.add_argument("--serve-precision", type=int, default=24,
                    help="350x10 likelihood requests through the server (serving form vs plain form)")
    args = ap.parse_args()
    rank, ws, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, ws, dist)
    else:
        run_ours(args, rank, ws, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
