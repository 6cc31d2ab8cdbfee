"""Seeded synthetic workloads for the SEIR-H-D model family.

Every workload is generated from a seed by one recipe:

* compartments S, E, I, H, R, D with exponential residence times
  (E mean 1/sigma, I mean 1/gamma, H mean ``h_mean``) and transitions
  S->E (infection), E->I, I->H (p_H), I->R (1-p_H), H->D (p_D), H->R (1-p_D);
* ``narea`` areas with integer populations split over ``nage`` age groups by
  a Dirichlet(2,...,2) draw;
* an age-mixing matrix, symmetric, entries U(lo, hi), diagonal multiplied;
* a gravity area-mixing kernel exp(-d/scale) on U(0,1)^2 coordinates with
  rows normalised (optionally with random long-range entries);
* R(t) as a piecewise-linear spline, optional area covariates and stepped
  age-mixing factors;
* E individuals seeded in area 0 (Poisson(10));
* observations: daily E->I counts and weekly H->D counts per area (or per
  area and age, or weekly H populations), the observed values coming from one
  simulation at the true parameters plus normal noise of variance
  max(count, 5), with the standard deviation column loaded from the file
  ("normal load").

``write_beep_inputs`` writes the workload in the reference's own input format
(TOML + CSV, the format documented for examples/*.toml of the reference) so
that the reference itself can run it; ``beep_gb300.model_builder`` builds the
device tables from the same spec without the reference.
"""
from __future__ import annotations

import dataclasses
import os
from typing import List, Optional

import numpy as np


@dataclasses.dataclass
class Workload:
    name: str
    seed: int
    narea: int
    nage: int
    days: int
    steps_per_day: int
    pop: np.ndarray                 # [A][G] int64
    age_mix: np.ndarray             # [G][G] raw matrix as written to CSV
    geo: np.ndarray                 # [A][A] raw matrix as written to CSV
    seed_E: np.ndarray              # [A][G] initial exposed
    sigma_inv: float = 4.0
    gamma_inv: float = 5.0
    h_mean: float = 8.0
    p_H: float = 0.05
    p_D: float = 0.2
    R_bp: List[int] = dataclasses.field(default_factory=list)   # knot days, first 0 last days
    R_val: List[float] = dataclasses.field(default_factory=list)
    R_smooth: Optional[float] = None          # smoothing sd of the R(t) knots (the reference's `smooth`)
    R_smooth_type: str = ""                   # "log_smooth" or "smooth"
    efoi: float = 0.0
    covar: Optional[np.ndarray] = None        # [ncovar][A]
    covar_effect: List[float] = dataclasses.field(default_factory=list)
    matmod: List[dict] = dataclasses.field(default_factory=list)  # {"ages": [..], "bp": [...], "val": [...]}
    obs_kind: str = "cases_deaths"            # cases_deaths | cases_age | hosp_pop
    # discrete strains (the reference's `strains` command): names, susceptibility and
    # R factor values/priors as TOML strings, and the exposed seeds of each strain
    # [NS][A][G] (the susceptibles start in the first strain)
    strains: Optional[dict] = None
    # model modifications of the reference's prediction mode (TOML `modification`): dicts
    # of its keys, e.g. {"type": "beta_fac", "start": "36", "end": "50", "factor": "0.5"}
    modifications: List[dict] = dataclasses.field(default_factory=list)
    # demographic changes of the age distribution (TOML `democat_change`): dicts with
    # "times" (days), "frac" [len(times)][nage] (each row sums to one) and optionally
    # "geo_filt" (e.g. "area:A1|A4"); populations then stop being integers
    democat_change: List[dict] = dataclasses.field(default_factory=list)
    # Erlang stages of the latent and infectious periods: E1..Ek and I1..Ik, each with
    # an exponential residence of mean sigma_inv / k (gamma_inv / k) -- 4k + 2 transitions
    stages: int = 1
    # prior ranges (inference modes)
    R_prior: tuple = (0.5, 4.0)
    sigma_inv_prior: tuple = (2.0, 6.0)
    gamma_inv_prior: tuple = (3.0, 8.0)
    h_mean_prior: tuple = (4.0, 12.0)

    @property
    def ndivision(self) -> int:
        return self.days * self.steps_per_day

    def e_names(self) -> List[str]:
        return ["E"] if self.stages == 1 else [f"E{i + 1}" for i in range(self.stages)]

    def i_names(self) -> List[str]:
        return ["I"] if self.stages == 1 else [f"I{i + 1}" for i in range(self.stages)]

    def comp_names(self) -> List[str]:
        return ["S"] + self.e_names() + self.i_names() + ["H", "R", "D"]

    def cases_transition(self) -> str:
        """The observed E->I transition (the last latent stage into the first infectious one)."""
        return f"{self.e_names()[-1]}->{self.i_names()[0]}"

    def age_names(self) -> List[str]:
        return [f"age{a}" for a in range(self.nage)]

    def area_names(self) -> List[str]:
        return [f"A{c}" for c in range(self.narea)]


def _gravity(rng, n, scale, long_range_frac=0.0, long_range_max=0.01):
    xy = rng.random((n, 2))
    d = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    k = np.exp(-d / scale)
    if long_range_frac > 0:
        mask = rng.random((n, n)) < long_range_frac
        k = k + mask * rng.uniform(0.0, long_range_max, (n, n))
    k = k / k.sum(1, keepdims=True)
    return k


def _split_pop(rng, total, nage):
    w = rng.dirichlet([2.0] * nage)
    parts = np.floor(w * total).astype(np.int64)
    parts[0] += total - parts.sum()
    return parts


def seir_hd_small(seed: int = 20260000, narea: int = 10, nage: int = 3, days: int = 100,
                  steps_per_day: int = 4, nknot: int = 5, name: str = "c0") -> Workload:
    """Plain PMCMC likelihood workload (10 areas x 3 ages, dt 0.25, 100 days)."""
    rng = np.random.default_rng(seed)
    totals = rng.integers(50000, 500001, narea)
    pop = np.stack([_split_pop(rng, int(t), nage) for t in totals])
    am = rng.uniform(0.5, 2.0, (nage, nage))
    am = np.triu(am) + np.triu(am, 1).T
    am[np.diag_indices(nage)] *= 3.0
    geo = _gravity(rng, narea, 0.2)
    seedE = np.zeros((narea, nage), np.int64)
    seedE[0, nage // 2] = max(1, rng.poisson(10))
    bp = [int(round(k * days / (nknot - 1))) for k in range(nknot)]
    val = [2.5] + list(rng.uniform(0.6, 2.5, nknot - 1))
    return Workload(name=name, seed=seed, narea=narea, nage=nage, days=days, steps_per_day=steps_per_day,
                    pop=pop, age_mix=am, geo=geo, seed_E=seedE, R_bp=bp, R_val=[float(v) for v in val])


def _fmt(x) -> str:
    return repr(float(x))


def write_beep_inputs(w: Workload, outdir: str, obs_values: Optional[dict] = None) -> str:
    """Writes the workload as a reference TOML + CSV directory; returns the TOML path.

    ``obs_values`` maps data-file name -> {column -> (values, sds)}; without it
    placeholder observations (0, sd 1) of the right shape are written."""
    os.makedirs(outdir, exist_ok=True)
    data = os.path.join(outdir, "data")
    os.makedirs(data, exist_ok=True)
    A, G = w.narea, w.nage
    ages, areas = w.age_names(), w.area_names()

    with open(os.path.join(data, "population.csv"), "w") as f:
        cols = ["area"] + (ages if G > 1 else ["population"])
        if w.covar is not None:
            cols += [f"cov{j}" for j in range(w.covar.shape[0])]
        f.write(",".join(cols) + "\n")
        for c in range(A):
            row = [areas[c]] + [str(int(v)) for v in w.pop[c]]
            if w.covar is not None:
                row += [_fmt(w.covar[j, c]) for j in range(w.covar.shape[0])]
            f.write(",".join(row) + "\n")
    if G > 1:
        with open(os.path.join(data, "age_mixing_matrix.csv"), "w") as f:
            for a in range(G):
                f.write(",".join(_fmt(v) for v in w.age_mix[a]) + "\n")
    if A > 1:
        with open(os.path.join(data, "geo_mixing_matrix.csv"), "w") as f:
            for c in range(A):
                f.write(",".join(_fmt(v) for v in w.geo[c]) + "\n")
    comps = w.comp_names()
    e_first = w.e_names()[0]
    with open(os.path.join(data, "init_pop.csv"), "w") as f:
        if w.strains is None:
            f.write("area," + ("age," if G > 1 else "") + "compartment,population\n")
            for c in range(A):
                for a in range(G):
                    for co in comps:
                        if co == "S":
                            v = int(w.pop[c, a] - w.seed_E[c, a])
                        elif co == e_first:
                            v = int(w.seed_E[c, a])
                        else:
                            v = 0
                        f.write(f"{areas[c]}," + (f"{ages[a]}," if G > 1 else "") + f"{co},{v}\n")
        else:
            seeds = np.asarray(w.strains["seed_E"])
            f.write("area," + ("age," if G > 1 else "") + "strain,compartment,population\n")
            for c in range(A):
                for a in range(G):
                    for st, sn in enumerate(w.strains["names"]):
                        for co in comps:
                            if co == "S":
                                v = int(w.pop[c, a] - seeds[:, c, a].sum()) if st == 0 else 0
                            elif co == e_first:
                                v = int(seeds[st, c, a])
                            else:
                                v = 0
                            f.write(f"{areas[c]}," + (f"{ages[a]}," if G > 1 else "") + f"{sn},{co},{v}\n")

    tables = data_tables(w)
    for tab in tables:
        rows = tab["times"]
        cols = tab["columns"]
        vals = (obs_values or {}).get(tab["file"])
        sd_col = tab.get("sd_col", True)
        with open(os.path.join(data, tab["file"]), "w") as f:
            f.write("time," + ",".join(f"{c},{c} SD" if sd_col else c for c in cols) + "\n")
            for r, t in enumerate(rows):
                cells = []
                for j, c in enumerate(cols):
                    if vals is None:
                        cells += ["0", "1"] if sd_col else ["1"]
                        continue
                    v, sd = vals[c]
                    nd = tab.get("nodata_every")
                    if nd and (r + j) % nd == 0:
                        x = "."                                   # no data
                    elif tab.get("censor_below") is not None and v[r] < tab["censor_below"]:
                        x = "*"                                   # below the table's threshold
                    else:
                        x = str(int(v[r]))
                    cells += [x, _fmt(sd[r])] if sd_col else [x]
                f.write(f"{t}," + ",".join(cells) + "\n")

    nk = len(w.R_bp)
    bp = "|".join(["start"] + [str(b) for b in w.R_bp[1:-1]] + ["end"])
    rval = "|".join(_fmt(v) for v in w.R_val)
    rprior = "|".join([f"Uniform({w.R_prior[0]},{w.R_prior[1]})"] * nk)
    lines = [
        'time_format = "number"',
        'start = "0"',
        f'end = "{w.days}"',
        f'steps_per_unit_time = {w.steps_per_day}',
        'datadir = "data"',
        'outputdir = "output"',
        'areas = "population.csv"',
        'init_pop = "init_pop.csv"',
    ]
    if w.strains is not None:
        sd = w.strains
        lines.append('strains = {cats="' + " | ".join(sd["names"]) + f'", sus_value="{sd["sus_value"]}", '
                     f'sus_prior="{sd["sus_prior"]}", Rfactor_value="{sd["Rfactor_value"]}", '
                     f'Rfactor_prior="{sd["Rfactor_prior"]}"' + "}")
    if G > 1:
        lines.append('ages = {cats="' + " | ".join(ages) + '"}')
        lines.append('age_mixing_matrix = "age_mixing_matrix.csv"')
    if A > 1:
        lines.append('geo_mixing_matrix = "geo_mixing_matrix.csv"')
    lines += [
        "comps = [",
        '{name="S"},',
    ]
    k = w.stages
    en, iname = w.e_names(), w.i_names()
    for e in en:
        lines.append(f'{{name="{e}", dist="Exp", mean_value="{_fmt(w.sigma_inv / k)}", '
                     f'mean_prior="Uniform({_fmt(w.sigma_inv_prior[0] / k)},{_fmt(w.sigma_inv_prior[1] / k)})"}},'
                     if k > 1 else
                     f'{{name="E", dist="Exp", mean_value="{_fmt(w.sigma_inv)}", mean_prior="Uniform({w.sigma_inv_prior[0]},{w.sigma_inv_prior[1]})"}},')
    for i in iname:
        lines.append(f'{{name="{i}", dist="Exp", mean_value="{_fmt(w.gamma_inv / k)}", inf_value="1", '
                     f'mean_prior="Uniform({_fmt(w.gamma_inv_prior[0] / k)},{_fmt(w.gamma_inv_prior[1] / k)})"}},'
                     if k > 1 else
                     f'{{name="I", dist="Exp", mean_value="{_fmt(w.gamma_inv)}", inf_value="1", mean_prior="Uniform({w.gamma_inv_prior[0]},{w.gamma_inv_prior[1]})"}},')
    lines += [
        f'{{name="H", dist="Exp", mean_value="{_fmt(w.h_mean)}", mean_prior="Uniform({w.h_mean_prior[0]},{w.h_mean_prior[1]})"}},',
        '{name="R"},',
        '{name="D"}',
        "]",
        "trans = [",
        f'{{from="S", to="{en[0]}", infection="yes"}},',
    ]
    chain = en + iname
    for a_, b_ in zip(chain, chain[1:]):
        lines.append(f'{{from="{a_}", to="{b_}"}},')
    lines += [
        f'{{from="{iname[-1]}", to="H", prob_value="{_fmt(w.p_H)}", prob_prior="Dir(1)"}},',
        f'{{from="{iname[-1]}", to="R", prob_value="*", prob_prior="Dir(1)"}},',
        f'{{from="H", to="D", prob_value="{_fmt(w.p_D)}", prob_prior="Dir(1)"}},',
        '{from="H", to="R", prob_value="*", prob_prior="Dir(1)"}',
        "]",
        f'R_spline = [{{ value="{rval}", prior="{rprior}", bp="{bp}"' +
        (f', smooth="{_fmt(w.R_smooth)}", smooth_type="{w.R_smooth_type}"' if w.R_smooth is not None else "") + "}]",
        f'efoi_spline = [{{ value="{_fmt(w.efoi)}"}}]',
    ]
    if w.covar is not None:
        lines.append("area_covars = [")
        for j, eff in enumerate(w.covar_effect):
            lines.append(f'{{name="cov{j}", value="{_fmt(eff)}", prior="Uniform(-1,1)", func="linear"}},')
        lines.append("]")
    if w.matmod:
        lines.append("age_mixing_modify = [")
        for i, mm in enumerate(w.matmod):
            mbp = "|".join(["start"] + [str(b) for b in mm["bp"][1:-1]] + ["end"])
            names = "|".join(f"mm{i}_{k}" for k in range(len(mm["val"])))   # repeated break times need names
            lines.append(f'{{type="row_column", agecat="{"|".join(ages[a] for a in mm["ages"])}", bp="{mbp}", '
                         f'param="{names}", '
                         f'value="{"|".join(_fmt(v) for v in mm["val"])}", '
                         f'prior="{"|".join(f"Fixed({_fmt(v)})" for v in mm["val"])}"}},')
        lines.append("]")
    if w.democat_change:
        lines.append("democat_change = [")
        for k, dc in enumerate(w.democat_change):
            fname = f"democat_change{k}.csv"
            with open(os.path.join(data, fname), "w") as f:
                f.write("time," + ",".join(ages) + "\n")
                for t, row in zip(dc["times"], dc["frac"]):
                    f.write(f"{int(t)}," + ",".join(_fmt(v) for v in row) + "\n")
            geo = f', geo_filt="{dc["geo_filt"]}"' if dc.get("geo_filt") else ""
            lines.append(f'{{name="age", file="{fname}"{geo}}},')
        lines.append("]")
    if w.modifications:
        lines.append("modification = [")
        for mod in w.modifications:
            lines.append("{" + ", ".join(f'{k}="{v}"' for k, v in mod.items()) + "},")
        lines.append("]")
    lines.append("data_tables = [")
    for tab in tables:
        lines.append("{" + ", ".join(f'{k}="{v}"' for k, v in tab["toml"].items()) + "},")
    lines += ["]"]
    toml = os.path.join(outdir, f"{w.name}.toml")
    with open(toml, "w") as f:
        f.write("\n".join(lines) + "\n")
    return toml


def data_tables(w: Workload) -> List[dict]:
    """The observation tables of the workload, in the order they are declared."""
    areas = w.area_names()
    tabs = []
    if w.obs_kind == "cases_deaths":
        tabs.append(dict(file="cases.csv", times=list(range(0, w.days)), columns=areas,
                         toml=dict(type="transition", observation=w.cases_transition(), timestep="1", obsmodel="normal load",
                                   geo_dep="area", file="cases.csv")))
        tabs.append(dict(file="deaths.csv", times=list(range(0, w.days - 6, 7)), columns=areas,
                         toml=dict(type="transition", observation="H->D", timestep="7", obsmodel="normal load",
                                   geo_dep="area", file="deaths.csv")))
    elif w.obs_kind == "cases_age":
        for a, an in enumerate(w.age_names()):
            tabs.append(dict(file=f"cases_{an}.csv", times=list(range(0, w.days)), columns=areas,
                             toml=dict(type="transition", observation=w.cases_transition(), timestep="1", obsmodel="normal load",
                                       geo_dep="area", democats_filt=f"age:{an}", file=f"cases_{an}.csv")))
    elif w.obs_kind == "hosp_pop":
        tabs.append(dict(file="hosp.csv", times=list(range(0, w.days, 7)), columns=areas,
                         toml=dict(type="population", observation="H", obsmodel="normal load",
                                   geo_dep="area", file="hosp.csv")))
    elif w.obs_kind == "obs_models":
        # every observation model the reference parses (src/inputs.cc:413-473) with
        # censored ('*' below the table's threshold) and missing ('.') entries
        tabs.append(dict(file="cases.csv", times=list(range(0, w.days)), columns=areas, sd_col=False,
                         toml=dict(type="transition", observation=w.cases_transition(), timestep="1", obsmodel="normal 10%",
                                   geo_dep="area", file="cases.csv")))
        tabs.append(dict(file="deaths.csv", times=list(range(0, w.days - 6, 7)), columns=areas, sd_col=False,
                         censor_below=5, nodata_every=5,
                         toml=dict(type="transition", observation="H->D", timestep="7", obsmodel="poisson",
                                   threshold="5", geo_dep="area", file="deaths.csv")))
        tabs.append(dict(file="hosp.csv", times=list(range(0, w.days, 7)), columns=areas, sd_col=False,
                         nodata_every=7,
                         toml=dict(type="population", observation="H", obsmodel="normal 30",
                                   geo_dep="area", file="hosp.csv")))
        tabs.append(dict(file="cases_w.csv", times=list(range(0, w.days - 6, 7)), columns=areas, censor_below=20,
                         toml=dict(type="transition", observation=w.cases_transition(), timestep="7", obsmodel="normal load",
                                   threshold="20", geo_dep="area", file="cases_w.csv")))
    else:
        raise ValueError(w.obs_kind)
    return tabs


def seir_hd_strains(seed: int = 20260104, narea: int = 5, nage: int = 2, days: int = 60, name: str = "strains") -> Workload:
    """The small SEIR-H-D workload with two strains (the reference's `strains`
    command, as in its two-strain example): the second strain with
    susceptibility factor 0.7 relative to the first and R factor 1.4; exposed
    seeds of both strains in different areas; daily cases and weekly deaths per
    area summed over ages and strains."""
    w = seir_hd_small(seed=seed, narea=narea, nage=nage, days=days, name=name)
    seeds = np.zeros((2, narea, nage), np.int64)
    seeds[0] = w.seed_E
    seeds[1, narea - 1, 0] = 8
    w.strains = {"names": ["s1", "s2"], "sus_value": "0.7 | *", "sus_prior": "MDir(0.5)",
                 "Rfactor_value": "1.0 | 1.4", "Rfactor_prior": "Fixed(1) | Uniform(0.5,2)", "seed_E": seeds}
    return w


def seir_hd_obs_models(seed: int = 20260105, narea: int = 4, nage: int = 2, days: int = 70,
                       name: str = "obsmodels") -> Workload:
    """The small SEIR-H-D workload observed through every observation model
    the reference reads: normal with a percentage SD, Poisson with a threshold
    (censored entries), normal with a fixed SD on populations, normal with
    loaded SDs and a threshold; some entries missing."""
    w = seir_hd_small(seed=seed, narea=narea, nage=nage, days=days, name=name)
    w.obs_kind = "obs_models"
    return w


def seir_hd_democat(seed: int = 20260110, narea: int = 6, nage: int = 3, days: int = 70,
                    name: str = "democat") -> Workload:
    """The small SEIR-H-D workload with demographic changes of the age
    distribution (the reference's `democat_change`, src/data.cc:958-1040):
    one over every area (age shares interpolated between three dates) and one
    over two areas (two dates), observed through every observation model
    (population observations read the fractional populations).  Exposed
    individuals are seeded in every area so that the epidemic is visible."""
    w = seir_hd_small(seed=seed, narea=narea, nage=nage, days=days, name=name)
    w.obs_kind = "obs_models"
    w.seed_E[:, :] = 5
    rng = np.random.default_rng(seed + 1)
    times = [0, days // 3, days - 5]
    w.democat_change = [
        dict(times=times, frac=[list(rng.dirichlet([4.0] * nage)) for _ in times]),
        dict(times=[days // 5, days // 2], frac=[list(rng.dirichlet([4.0] * nage)) for _ in range(2)],
             geo_filt="area:A1|A4"),
    ]
    return w


def seir_hd_features(seed: int = 20260106, narea: int = 6, nage: int = 3, days: int = 60,
                     name: str = "features") -> Workload:
    """The small SEIR-H-D workload with the per-step tables that vary in time
    and area: two area covariates (effects 0.3 and -0.2), stepped age-mixing
    factors on two age groups from day 25, an external force of infection
    (5 per day) and an R(t) spline of 7 knots."""
    w = seir_hd_small(seed=seed, narea=narea, nage=nage, days=days, nknot=7, name=name)
    rng = np.random.default_rng(seed + 1)
    w.covar = rng.normal(0.0, 1.0, (2, narea))
    w.covar_effect = [0.3, -0.2]
    w.matmod = [{"ages": [0, 2], "bp": [0, 25, 25, days], "val": [1.0, 1.0, 0.6, 0.6]}]
    w.efoi = 5.0
    return w


def abc_smc_large(seed: int = 20260001, narea: int = 150, nage: int = 4, days: int = 180,
                  steps_per_day: int = 2, name: str = "c1") -> Workload:
    """Batched ABC-SMC workload: 150 areas x 4 ages, dt 0.5, 180 days; area
    populations log-normal(12, 0.8) rounded; constant R0 (a per-particle
    parameter); daily E->I observations per area and age."""
    rng = np.random.default_rng(seed)
    totals = np.maximum(np.rint(rng.lognormal(12.0, 0.8, narea)).astype(np.int64), 100)
    pop = np.stack([_split_pop(rng, int(t), nage) for t in totals])
    am = rng.uniform(0.5, 2.0, (nage, nage))
    am = np.triu(am) + np.triu(am, 1).T
    am[np.diag_indices(nage)] *= 3.0
    geo = _gravity(rng, narea, 0.2)
    seedE = np.zeros((narea, nage), np.int64)
    seedE[0, nage // 2] = max(1, rng.poisson(10))
    return Workload(name=name, seed=seed, narea=narea, nage=nage, days=days, steps_per_day=steps_per_day,
                    pop=pop, age_mix=am, geo=geo, seed_E=seedE, R_bp=[0, days], R_val=[2.5, 2.5],
                    obs_kind="cases_age", R_prior=(1.5, 4.0))


MBP_SIZES = ((20, 2), (80, 4), (200, 6), (350, 10))


def mbp_chain_model(narea: int, nage: int, seed: int = 20260003) -> Workload:
    """One model of the MBP-chain workload: the 10-area recipe at narea x nage,
    dt 0.5 over 200 days, weekly hospital-population observations per area."""
    w = seir_hd_small(seed=seed + 1000 * narea + nage, narea=narea, nage=nage, days=200, steps_per_day=2,
                      name=f"mbp_{narea}x{nage}")
    w.obs_kind = "hosp_pop"
    return w


def abc_smc_priors(rng, n: int):
    """Per-particle parameters from the ABC-SMC priors: R0 U(1.5,4), 1/sigma U(2,6), 1/gamma U(3,8)."""
    return rng.uniform(1.5, 4.0, n), rng.uniform(2.0, 6.0, n), rng.uniform(3.0, 8.0, n)


def precision_large(seed: int = 20260002, narea: int = 350, nage: int = 10, days: int = 365,
                    steps_per_day: int = 4, name: str = "c2") -> Workload:
    """Precision workload: 350 areas x 10 ages, dt 0.25, 365 days.  Gravity
    mixing exp(-d/0.1) plus 5% long-range entries U(0, 0.01); age mixing
    U(0.2, 3) symmetric with 3 stepped modification factors; R(t) with 20
    knots U(0.5, 2); two area covariates N(0,1) with effects 0.1 and 0.05;
    daily cases and weekly deaths per area."""
    rng = np.random.default_rng(seed)
    totals = rng.integers(50000, 500001, narea)
    pop = np.stack([_split_pop(rng, int(t), nage) for t in totals])
    am = rng.uniform(0.2, 3.0, (nage, nage))
    am = np.triu(am) + np.triu(am, 1).T
    geo = _gravity(rng, narea, 0.1, long_range_frac=0.05, long_range_max=0.01)
    seedE = np.zeros((narea, nage), np.int64)
    seedE[0, nage // 2] = max(1, rng.poisson(10))
    nknot = 20
    bp = [int(round(k * days / (nknot - 1))) for k in range(nknot)]
    val = [float(v) for v in rng.uniform(0.5, 2.0, nknot)]
    val[0] = 2.5
    matmod = []
    groups = np.array_split(rng.permutation(nage), 3)
    for g in groups:
        t = int(rng.integers(30, days - 30))
        f = float(rng.uniform(0.4, 1.0))
        matmod.append({"ages": sorted(int(a) for a in g), "bp": [0, t, t, days], "val": [1.0, 1.0, f, f]})
    covar = rng.normal(0.0, 1.0, (2, narea))
    return Workload(name=name, seed=seed, narea=narea, nage=nage, days=days, steps_per_day=steps_per_day,
                    pop=pop, age_mix=am, geo=geo, seed_E=seedE, R_bp=bp, R_val=val, covar=covar,
                    covar_effect=[0.1, 0.05], matmod=matmod)
