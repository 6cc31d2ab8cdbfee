"""Generates the golden fixtures in this folder from the reference itself.

Needs the reference source tree (--ref; default BEEP_REF_DIR, else a checkout
named ``reference`` beside the repository) and builds the
reference oracle with oracle/Makefile.ref.  For each fixture:
  1. a seeded synthetic workload is written in the reference's TOML/CSV format
     with placeholder observations;
  2. the reference (driven by the keyed variate stream) simulates once at the
     true parameters; the observed values are that trajectory's sums plus
     normal noise of variance max(count, 5), written back with an SD column;
  3. the reference runs again and its model, set_param tables, per-particle
     log-likelihoods, checksums and (for a few particles) full transition and
     population trajectories are saved as a bundle ``<name>.bnd``.

usage: python tests/golden/make_golden.py [--ref REFERENCE_TREE] [--only NAMES]
                                         [--harness BINARY --outdir DIR]

--harness runs another build of the harness (for instance the reference
compiled with its own CMake flags, -mfma and the compiler's default FP
contraction) and --outdir writes its bundles elsewhere, so that they can be
compared with the committed ones.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from beep_gb300 import bundle, synth  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def run_harness(workdir, toml, out, npart, ntraj, seed, mode, pf=False, theta=None, pfn=0, mbp=0, sampledir=None,
                abcw=None):
    cmd = [HARNESS, f"out={out}", f"npart={npart}", f"ntraj={ntraj}", f"seed={seed}", f"pf={1 if pf else 0}"]
    if abcw:
        cmd += [f"abcw={abcw[0]}", f"abck={abcw[1]}"]
    if sampledir:
        cmd.append(f"sampledir={sampledir}")
    if theta is not None:
        cmd.append(f"theta={theta}")
    if pfn:
        cmd.append(f"pfn={pfn}")
    if mbp:
        cmd.append(f"mbp={mbp}")
    cmd += ["--", f"inputfile={os.path.basename(toml)}", f"mode={mode}"]
    if pfn:
        cmd += [f"nparticle={pfn}", "nsample=400", "nburnin=200", "invT=1"]
    if abcw:
        cmd += ["nsample=100", "ngeneration=2"]
    r = subprocess.run(cmd, cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness failed:\n{r.stdout}\n{r.stderr}")
    return bundle.read_bundle(out)


def obs_values_from(b, w: synth.Workload):
    """Per data file and column: (values, sd) from trajectory 0 of bundle b plus noise."""
    tn = b["g0.transnum"][0].astype(np.int64)     # [S][A][T][DP]
    pop = b["g0.pop"][0].astype(np.int64)         # [S][A][C][DP]
    T = tn.shape[2]
    C = pop.shape[2]
    DP = tn.shape[3]
    cells = b["obs_cells"]
    ptr = b["obs_cell_ptr"]
    si, sf = b["obs_sett_i"], b["obs_sett_f"]
    rng = np.random.default_rng(w.seed + 7)
    vals = []
    for o in range(len(si)):
        v = 0
        for s in range(si[o], sf[o]):
            for q in range(ptr[o], ptr[o + 1]):
                cell = int(cells[q])
                if cell >= 0:
                    c, rem = divmod(cell, T * DP)
                    tr, dp = divmod(rem, DP)
                    v += tn[s, c, tr, dp]
                else:
                    k = -1 - cell
                    c, rem = divmod(k, C * DP)
                    co, dp = divmod(rem, DP)
                    v += pop[s, c, co, dp]
        vals.append(v)
    vals = np.array(vals, np.float64)
    sd = np.sqrt(np.maximum(vals, 5.0))
    noisy = np.maximum(0, np.round(vals + rng.normal(0.0, 1.0, len(vals)) * sd))
    # observation order = data table -> column -> row (src/data.cc:1119-1320)
    out = {}
    k = 0
    for tab in synth.data_tables(w):
        out[tab["file"]] = {}
        nrow = len(tab["times"])
        for col in tab["columns"]:
            out[tab["file"]][col] = (noisy[k:k + nrow], np.sqrt(np.maximum(noisy[k:k + nrow], 5.0)))
            k += nrow
    assert k == len(vals), (k, len(vals))
    return out


def mbp_theta_rows(base, nchain, seed):
    """2*nchain parameter rows around the workload's own values: row 2k starts
    chain k, row 2k+1 is its proposal.  Perturbed are the E, I and H mean
    durations (positions 1, 2, 4), the I->H branch probability with its
    complement (5, 6) and the R-spline knots (9..13) -- the reference's
    parameter order for these workloads; the infectivity (3) is kept."""
    rng = np.random.default_rng(seed + 11)
    rows = []
    for _ in range(2 * nchain):
        t = np.array(base, np.float64)
        for i, lo, hi in ((1, 2.0, 6.0), (2, 3.0, 8.0), (4, 4.0, 12.0)):
            t[i] = min(hi - 1e-3, max(lo + 1e-3, t[i] * rng.uniform(0.85, 1.15)))
        t[5] = t[5] * rng.uniform(0.7, 1.3)
        t[6] = 1.0 - t[5]
        for i in range(9, 14):
            t[i] = min(3.99, max(0.51, t[i] * rng.uniform(0.85, 1.15)))
        rows.append(t)
    return rows


def prior_theta_rows(w: synth.Workload):
    """Parameter rows for the prior fixture, made from the reference's own
    values: the E, I and H durations and the R(t) knots scaled by U(0.8, 1.2)
    (the reference's parameter order: E 1, I 2, H 4, R knots from 9)."""
    def rows_of(base):
        rng = np.random.default_rng(w.seed + 3)
        rows = []
        for _ in range(4):
            t = np.array(base, np.float64)
            for i in (1, 2, 4):
                t[i] *= rng.uniform(0.8, 1.2)
            for i in range(9, 9 + len(w.R_val)):
                t[i] = min(3.9, max(0.6, t[i] * rng.uniform(0.8, 1.2)))
            rows.append(t)
        return rows
    return rows_of


ONLY = None   # fixture names to (re)generate (--only); None: all
OUTDIR = HERE  # where the bundles go (--outdir)


def make_fixture(name, w: synth.Workload, npart, ntraj, seed, pf=False, theta_rows=None, keep_dir=None, pfn=0,
                 mbp=0, samples=False, abcw=None, outdir=None):
    if ONLY is not None and name not in ONLY:
        return
    outdir = outdir or OUTDIR
    work = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        toml = synth.write_beep_inputs(w, work)
        mode = "pmcmc" if pf else "abcsmc"
        b0 = run_harness(work, toml, os.path.join(work, "b0.bnd"), 1, 1, seed + 1, mode, pf=False)
        vals = obs_values_from(b0, w)
        synth.write_beep_inputs(w, work, obs_values=vals)
        theta = None
        if callable(theta_rows):
            theta_rows = theta_rows(b0["g0.theta"])
        if theta_rows is not None:
            theta = os.path.join(work, "theta.csv")
            with open(theta, "w") as f:
                for row in theta_rows:
                    f.write(",".join(repr(float(x)) for x in row) + "\n")
        if (mbp or abcw) and theta_rows is None:
            # MBP: a start and a proposal row per chain; ABC-SMC weights: the previous
            # generation's rows, then the new samples' (all inside the prior bounds)
            theta = os.path.join(work, "theta.csv")
            base = b0["g0.theta"]
            nrow_pairs = mbp if mbp else (abcw[0] + abcw[1] + 1) // 2
            with open(theta, "w") as f:
                for row in mbp_theta_rows(base, nrow_pairs, w.seed):
                    f.write(",".join(repr(float(x)) for x in row) + "\n")
        out = os.path.join(outdir, f"{name}.bnd")
        sdir = os.path.join(work, "samples") if samples else None
        if sdir:
            os.makedirs(sdir)
        run_harness(work, toml, out, npart, ntraj, seed, mode, pf=pf, theta=theta, pfn=pfn, mbp=mbp, sampledir=sdir,
                    abcw=abcw)
        if abcw:
            # only the weights' inputs and outputs are kept (the bundle holds every row's tables)
            full = bundle.read_bundle(out)
            bundle.write_bundle(out, {k: v for k, v in full.items() if k.startswith("abc.")})
        if sdir:
            # the reference's own sample files of the sampled lineage
            for f in sorted(os.listdir(sdir)):
                shutil.copy(os.path.join(sdir, f), os.path.join(outdir, f"{name}_{f}"))
        if keep_dir:
            shutil.copytree(work, os.path.join(keep_dir, name), dirs_exist_ok=True)
        print(f"{name}: {os.path.getsize(out) / 1e3:.0f} kB")
    finally:
        shutil.rmtree(work, ignore_errors=True)


def make_prediction_fixture(name, w: synth.Workload, ngroup, npart, seed):
    """Prediction with model modifications (the reference's mode=prediction,
    src/simulate.cc:142-165, src/model.cc:1446-1585): posterior samples are the
    reference's own trajectories of ngroup parameter rows x npart particles
    (run without modifications), written as BEEP sample files by
    beep_gb300.samples; the reference then loads each sample and simulates it
    from the modifications' start to the end.  The bundle also holds a full
    simulation of the workload's own parameter values under the modifications
    (g0.*) with the multiplier tables."""
    from beep_gb300 import samples
    if ONLY is not None and name not in ONLY:
        return
    work = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        toml = synth.write_beep_inputs(w, work)
        b0 = run_harness(work, toml, os.path.join(work, "b0.bnd"), 1, 1, seed + 1, "abcsmc")
        synth.write_beep_inputs(w, work, obs_values=obs_values_from(b0, w))
        # posterior samples: ngroup parameter rows around the workload's values, npart trajectories each
        base = b0["g0.theta"]
        rows = mbp_theta_rows(base, (ngroup + 1) // 2, w.seed)[:ngroup]
        theta = os.path.join(work, "theta.csv")
        with open(theta, "w") as f:
            for row in rows:
                f.write(",".join(repr(float(x)) for x in row) + "\n")
        bs = run_harness(work, toml, os.path.join(work, "bs.bnd"), npart, npart, seed + 2, "abcsmc", theta=theta)
        names = bytes(bs["param_names"].astype(np.uint8)).decode().split("\n")[:-1]
        sdir = os.path.join(work, "samples")
        os.makedirs(sdir)
        dims = [int(x) for x in bs["dims"]]
        period, S = dims[7], dims[6]
        times = samples.division_times(period, S, start=0.0)
        k = 0
        for g in range(ngroup):
            for p in range(npart):
                # EF is written as 0: State::save prints doubles %g-style and State::load's number
                # parser rejects the exponent form an EF above 1e6 takes (the prediction does not use it)
                samples.write_sample(sdir, k, 0.0, names, bs[f"g{g}.theta"], bs[f"g{g}.transnum"][p], times)
                k += 1
        out = os.path.join(OUTDIR, f"{name}.bnd")
        cmd = [HARNESS, f"out={out}", "npart=4", "ntraj=2", f"seed={seed}", "pf=0", f"pred={sdir}",
               f"predn={ngroup * npart}", "--", f"inputfile={os.path.basename(toml)}", "mode=prediction",
               f"prediction_end={w.days}"]   # the inference horizon: the splines keep their knots
        r = subprocess.run(cmd, cwd=work, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"harness failed:\n{r.stdout}\n{r.stderr}")
        print(f"{name}: {os.path.getsize(out) / 1e3:.0f} kB")
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("BEEP_REF_DIR") or os.path.join(os.path.dirname(ROOT), "reference"))
    ap.add_argument("--keep", default=None, help="keep the generated TOML/CSV inputs here")
    ap.add_argument("--only", default=None, help="comma-separated fixture names to (re)generate; default all")
    ap.add_argument("--harness", default=None, help="a harness binary to run instead of oracle/_ref/ref_harness")
    ap.add_argument("--outdir", default=None, help="write the bundles here instead of tests/golden")
    a = ap.parse_args()
    global ONLY, HARNESS, OUTDIR
    ONLY = set(a.only.split(",")) if a.only else None
    if a.outdir:
        OUTDIR = os.path.abspath(a.outdir)
        os.makedirs(OUTDIR, exist_ok=True)
    if a.harness:
        HARNESS = os.path.abspath(a.harness)
    else:
        subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref", f"REF={a.ref}", "-j8"], cwd=ROOT, check=True)

    # tiny: 4 areas x 3 ages, 40 days at dt 0.25
    tiny = synth.seir_hd_small(seed=20260100, narea=4, nage=3, days=40, name="tiny")
    make_fixture("tiny_sim", tiny, npart=8, ntraj=3, seed=0x1234567890ABCDEF)
    # particle-filter sections need period >= 10 x the largest observation step (src/details.cc:115)
    tiny70 = synth.seir_hd_small(seed=20260102, narea=3, nage=2, days=70, name="tiny70")
    make_fixture("tiny_pf", tiny70, npart=6, ntraj=2, seed=0x0F1E2D3C4B5A6978, pf=True, pfn=32, samples=True)
    # one age group (the reference's nage == 1 branch of get_NMI, src/state.cc:555-560)
    one = synth.seir_hd_small(seed=20260101, narea=5, nage=1, days=30, name="oneage")
    make_fixture("oneage_sim", one, npart=6, ntraj=2, seed=77)
    # two strains: the susceptible shift to the first strain, per-strain infectious maps and
    # R factors (src/state.cc:392-401, 223-290; src/model.cc:1318-1362)
    strains = synth.seir_hd_strains()
    make_fixture("strain_sim", strains, npart=8, ntraj=2, seed=0x5712A1)
    # a two-strain model large enough for the several-particles-per-SM layout (280 columns;
    # model and tables only)
    make_fixture("strain70_model", synth.seir_hd_strains(narea=70, nage=2, days=20, name="strains70"), npart=2, ntraj=0,
                 seed=0x5712A2)
    # every observation model: normal X%, Poisson with censoring, fixed-SD normal, loaded
    # SDs with a threshold; missing entries (src/obsmodel.cc:245-305, src/data.cc:1589-1623)
    make_fixture("obsmodel_sim", synth.seir_hd_obs_models(), npart=8, ntraj=2, seed=0x0B5E)
    # tables that vary with time and area: covariates (areafactor), stepped age-mixing
    # factors (Ntime), external force of infection (src/model.cc:1144-1362, src/state.cc:403-423)
    make_fixture("features_sim", synth.seir_hd_features(), npart=8, ntraj=2, seed=0xFEA7)
    # the particle filter on those tables (sections start part-way through the horizon;
    # 84 days: the reference's sections need 10 times the weekly observation step)
    make_fixture("features_pf", synth.seir_hd_features(days=84, name="features84"), npart=8, ntraj=1, seed=0xFEA8,
                 pf=True, pfn=64)
    # the 10-area x 3-age plain PMCMC workload at full horizon
    c0 = synth.seir_hd_small(seed=20260000, narea=10, nage=3, days=100, name="c0")
    make_fixture("c0_sim", c0, npart=16, ntraj=1, seed=20260000)
    make_fixture("c0_pf", c0, npart=8, ntraj=1, seed=20260001, pf=True, pfn=64)
    # MBP chains: 4 chains, three proposal variants each (coupled draws, SIMU cells)
    tmbp = synth.seir_hd_small(seed=20260103, narea=4, nage=2, days=40, name="tinymbp")
    make_fixture("tiny_mbp", tmbp, npart=1, ntraj=1, seed=0x5EED0F00D, mbp=4)
    make_fixture("c0_mbp", c0, npart=1, ntraj=0, seed=20260003, mbp=4)
    # ABC-SMC importance weights: 40 previous-generation samples, 24 new ones
    make_fixture("c0_abcw", c0, npart=1, ntraj=0, seed=20260004, abcw=(24, 40))
    # prediction with model modifications: a transition-rate factor on some areas, a beta
    # factor over a window, an external-FOI factor (src/model.cc:1495-1580); the time-varying
    # tables of the features workload (covariates, stepped age mixing, external FOI)
    pw = synth.seir_hd_features(seed=20260107, days=60, name="pred")
    pw.modifications = [
        {"type": "trans_rate_fac", "trans": "E->I", "start": "30", "factor": "0.6", "geo_filt": "area:A1|A3"},
        {"type": "beta_fac", "start": "36", "end": "50", "factor": "0.5"},
        {"type": "efoi_fac", "start": "30", "factor": "2.5", "geo_filt": "area:A0|A2|A4"},
    ]
    make_prediction_fixture("pred_sim", pw, ngroup=2, npart=2, seed=0x9E7D)
    # priors and bounds: the reference's Model::prior and inbounds on parameter rows around the
    # workload's values and on probe rows outside the bounds; log-normal smoothing of R(t)
    pw2 = synth.seir_hd_features(seed=20260109, days=40, name="priors")
    pw2.R_smooth, pw2.R_smooth_type = 0.3, "log_smooth"
    make_fixture("prior_spec", pw2, npart=1, ntraj=0, seed=0x7A10, theta_rows=prior_theta_rows(pw2))
    # beyond the fast form's usual instantiations: 18 age groups and Erlang-staged latent
    # and infectious periods (3 stages each: 10 compartments, 10 transitions)
    ww = synth.seir_hd_small(seed=20260108, narea=5, nage=18, days=30, name="wide")
    ww.stages = 3
    ww.seed_E[:, :] = 20                       # exposed in every area and age: a visible epidemic in 30 days
    make_fixture("wide_sim", ww, npart=8, ntraj=2, seed=0x31DE)
    # demographic changes (State::democat_change_pop_adjust, src/state.cc:339-376): FP64
    # populations; the particle filter carries them between sections, MBP chains adjust
    # their proposals (src/mbp.cc:265)
    dw = synth.seir_hd_democat()
    make_fixture("democat_sim", dw, npart=8, ntraj=2, seed=0xDC0C)
    make_fixture("democat_pf", dw, npart=4, ntraj=1, seed=0xDC0E, pf=True, pfn=32)
    make_fixture("democat_mbp", dw, npart=1, ntraj=0, seed=0xDC0D, mbp=4)


if __name__ == "__main__":
    main()
