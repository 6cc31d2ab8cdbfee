"""Builds the hot path's tables for a synthetic SEIR-H-D workload without the
reference: the parameter-independent model (Data / Model members) and, per
parameter set, what ``State::set_param`` derives (src/state.cc:66-91).

Each step restates the reference's arithmetic:
  * area mixing: dense matrix rows -> diagonal + off-diagonal lists, then the
    per-capita normalisation and genQ.factor of Data::geo_normalise
    (src/data_matrix.cc:55-80, 205-223);
  * age mixing: Data::age_mixing_matrix (scaling by age shares, symmetrising)
    and Data::agematrix_normalise (src/data_matrix.cc:100-189);
  * transition rates: Model::create_transrate (src/model.cc:1116-1140);
  * splines: Model::create_disc_spline, piecewise linear at step midpoints
    (src/model.cc:1018-1041);
  * area factors from linear covariates, normalised by the population-weighted
    mean: Model::create_areafactor / calculate_area_av (src/model.cc:1182-1250);
  * age-mixing modifications: Model::create_Ntime (src/model.cc:1254-1301);
  * beta = R(t) / lambda_max(NGM) with NGM = F V^-1 over the infectious states
    (src/model.cc:1318-1362, 2485-2621).  The reference finds lambda_max by a
    warm-started power iteration converged to ~1e-13; here it is taken from a
    dense eigen-solve, so beta agrees with the reference to ~1e-13 relative.
Everything else is bit-identical to the reference's tables (tested against
the golden bundles made by the reference itself).
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import synth

COMPS = ["S", "E", "I", "H", "R", "D"]
# (from, to) in declaration order; S->E is the infection transition
TRANS = [(0, 1), (1, 2), (2, 3), (2, 4), (3, 5), (3, 4)]
OBS_NORMAL, OBS_NORMAL_PERCENT, OBS_POISSON = 0, 1, 2   # beep_obs_model
OBSVAL_VALUE, OBSVAL_UNKNOWN, OBSVAL_THRESH = 0, 1, 2   # beep_obs_value_kind
THRESH, UNKNOWN = 999999998.0, 999999997.0             # the reference's markers of censored / missing values
EPSILON_FACTOR = 0.01                                   # the reference's default epsilon_factor
UNSET = 999999999.0


def _seq_sum(vals) -> float:
    s = 0.0
    for v in vals:
        s += float(v)
    return s


def model_arrays(w: synth.Workload, obs_values: Optional[dict] = None) -> Dict[str, np.ndarray]:
    """The parameter-independent model (beep_model_desc fields) of a workload.

    ``obs_values``: data file -> column -> (values, sds) as written to the
    workload's data tables; placeholders (0, sd 1) when None."""
    A, G = w.narea, w.nage
    NS = nstrain(w)
    DP, C, T = G * NS, len(COMPS), len(TRANS)
    S = w.ndivision
    pop = np.asarray(w.pop, np.int64)
    total_pop = pop.sum(1)                       # Area::total_pop (unsigned)
    popsize = float(total_pop.sum())

    # area mixing (dense load, then per-capita normalisation)
    diag = np.zeros(A)
    rowptr = [0]
    to: List[int] = []
    val: List[float] = []
    geo = np.asarray(w.geo, np.float64) if A > 1 else np.ones((1, 1))
    tp = total_pop.astype(np.float64)
    for c in range(A):
        d = float(geo[c, c])
        row = geo[c]
        tos = np.flatnonzero((row != 0) & (np.arange(A) != c))
        vs = row[tos]
        # d*pop_c + sum_i v_i*pop_i, added left to right (cumsum is sequential)
        s = float(np.cumsum(np.concatenate(([d * tp[c]], vs * tp[tos])))[-1])
        diag[c] = d / s
        to += tos.tolist()
        val += (vs / s).tolist()
        rowptr.append(len(to))
    factor = np.array([(1.0 / float(total_pop[c])) / diag[c] for c in range(A)])

    # dp = strain * G + age (the strain democat last, src/data.cc); susceptibles start
    # in the first strain, the exposed seeds in their own strains
    pop_init = np.zeros((A, C, DP))
    if NS == 1:
        pop_init[:, 0, :] = pop - w.seed_E
        pop_init[:, 1, :] = w.seed_E
    else:
        seeds = np.asarray(w.strains["seed_E"])
        pop_init[:, 0, :G] = pop - seeds.sum(0)
        for st in range(NS):
            pop_init[:, 1, st * G:(st + 1) * G] = seeds[st]

    arr: Dict[str, np.ndarray] = {
        "dims": np.array([A, G, DP, NS, C, T, S, w.days, w.steps_per_day], np.int32),
        "dt": np.array([float(w.days) / S]),
        "popsize": np.array([popsize]),
        "trans_from": np.array([f for f, _ in TRANS], np.int32),
        "trans_to": np.array([t for _, t in TRANS], np.int32),
        "infection_trans": np.array([0], np.int32),
        "democatpos_age": np.arange(G, dtype=np.int32),
        "M_diag": diag, "M_rowptr": np.array(rowptr, np.int32), "M_to": np.array(to, np.int32),
        "M_val": np.array(val, np.float64), "M_factor": factor, "pop_init": pop_init,
    }
    arr.update(_observations(w, obs_values))
    arr.update(_democat_change(w))
    return arr


def _democat_change(w: synth.Workload) -> Dict[str, np.ndarray]:
    """Demographic changes of the age distribution as Data::load_democat_change
    (src/data.cc:958-1040) loads them: each change's areas (its geo filter,
    Data::create_area_sel, src/data.cc:1783-1823), one group of the first
    strain's dp (value f = age f), and per step the shares interpolated
    linearly in time between the file's rows around the step's day, each row
    normalised by its sum (Data::get_demo_frac, src/data.cc:821-870)."""
    if not w.democat_change:
        return {}
    A, G, S, spd = w.narea, w.nage, w.ndivision, w.steps_per_day
    names = w.area_names()
    nval, aptr, areas, dptr, dps, frac = [], [0], [], [0], [], []
    for dc in w.democat_change:
        if dc.get("geo_filt"):
            sel = set(dc["geo_filt"].split(":", 1)[1].split("|"))
            areas += [c for c in range(A) if names[c] in sel]
        else:
            areas += list(range(A))
        aptr.append(len(areas))
        nval.append(G)
        dps += list(range(G))
        dptr.append(len(dps))
        times = [int(t) for t in dc["times"]]
        rows = []
        for r in dc["frac"]:
            vals = [float(synth._fmt(v)) for v in r]          # the values as the file carries them
            rows.append([v / _seq_sum(vals) for v in vals])
        row = 0
        for sett in range(S):
            t = sett // spd
            while row < len(times) - 2 and times[row + 1] <= t:
                row += 1
            if t < times[row]:
                fr = 0.0
            elif t > times[row + 1]:
                fr = 1.0
            else:
                fr = (t - times[row]) / (times[row + 1] - times[row])
            frac += [rows[row][i] * (1 - fr) + rows[row + 1][i] * fr for i in range(G)]
    return {"dcc_nval": np.array(nval, np.int32), "dcc_area_ptr": np.array(aptr, np.int32),
            "dcc_area": np.array(areas, np.int32), "dcc_dp_ptr": np.array(dptr, np.int32),
            "dcc_dp": np.array(dps, np.int32), "dcc_frac": np.array(frac, np.float64)}


def nstrain(w: synth.Workload) -> int:
    return 1 if w.strains is None else len(w.strains["names"])


def _obsmodel(spec: str):
    """(model, fixed sd, percent) of a data table's `obsmodel` string (src/inputs.cc:413-473)."""
    parts = spec.split()
    if parts[0].lower() == "poisson":
        return OBS_POISSON, None, None
    if len(parts) == 1 or parts[1].lower() == "load":
        return OBS_NORMAL, None, None
    if parts[1].endswith("%"):
        return OBS_NORMAL_PERCENT, None, float(parts[1][:-1])
    return OBS_NORMAL, float(parts[1]), None


def _observations(w: synth.Workload, obs_values: Optional[dict]) -> Dict[str, np.ndarray]:
    """Observation list in the reference's order: data table -> column -> row
    (Data::load_timeseries_datatable, src/data.cc:1119-1320), with the values
    the data files carry: missing ('.') and censored ('*', below the table's
    threshold) entries as the reference marks them, and the standard deviation
    of each observation model (Data::set_obs_sd, src/data.cc:1589-1623: a
    percentage of the value blended with the column's largest value)."""
    G, T, C = w.nage, len(TRANS), len(COMPS)
    DP = G * nstrain(w)
    spd = w.steps_per_day
    # per data column (all its rows at once): windows, cells, values, kinds, SDs
    si, sf, vals, sds, kinds, models, thr, cells = [], [], [], [], [], [], [], []
    ncell = []                                      # cells of each observation
    tr_of = {"E->I": 1, "H->D": 4}
    for tab in synth.data_tables(w):
        tt = tab["toml"]
        times = np.asarray(tab["times"], np.int64)
        nrow = len(times)
        model, fixed_sd, percent = _obsmodel(tt["obsmodel"])
        threshold = float(tt["threshold"]) if "threshold" in tt else UNSET
        for ci, col in enumerate(tab["columns"]):
            c = ci
            if "democats_filt" in tt:                 # one age group, every strain
                age = int(tt["democats_filt"].split("age")[-1])
                dps = [dp for dp in range(DP) if dp % G == age]
            else:
                dps = list(range(DP))
            if tt["type"] == "transition":
                step = int(tt["timestep"])
                si.append(times * spd)
                sf.append((times + step) * spd)
                tr = tr_of[tt["observation"]]
                row_cells = [(c * T + tr) * DP + dp for dp in dps]
            else:
                si.append(times * spd)
                sf.append(times * spd + 1)
                co = COMPS.index(tt["observation"])
                row_cells = [-1 - ((c * C + co) * DP + dp) for dp in dps]
            cells.append(np.tile(np.asarray(row_cells, np.int64), nrow))
            ncell.append(np.full(nrow, len(dps), np.int64))
            ov = obs_values.get(tab["file"], {}).get(col) if obs_values else None
            kind = np.full(nrow, OBSVAL_VALUE, np.int64)
            if ov is None:
                v = np.full(nrow, 1.0 if not tab.get("sd_col", True) else 0.0)
                sd = np.ones(nrow)
            else:
                v = np.asarray(ov[0], np.float64)[:nrow].copy()
                sd = np.asarray(ov[1], np.float64)[:nrow].copy() if ov[1] is not None else np.ones(nrow)
                r = np.arange(nrow)
                nd = tab.get("nodata_every")
                unknown = (r + ci) % nd == 0 if nd else np.zeros(nrow, bool)
                cens = (~unknown & (v < tab["censor_below"]) if tab.get("censor_below") is not None
                        else np.zeros(nrow, bool))
                kind[unknown], kind[cens] = OBSVAL_UNKNOWN, OBSVAL_THRESH
                v = np.where(unknown, UNKNOWN, np.where(cens, THRESH, np.trunc(v)))
            # standard deviations by observation model
            valued = v[kind == OBSVAL_VALUE]
            vmax = float(valued.max()) if valued.size else 0.0
            if model == OBS_POISSON:
                sd = np.full(nrow, UNSET)
            elif percent is not None:
                sd = (v * (1 - EPSILON_FACTOR) + vmax * EPSILON_FACTOR) * 0.01 * percent
            elif fixed_sd is not None:
                sd = np.full(nrow, fixed_sd)
            vals.append(v)
            kinds.append(kind)
            sds.append(sd)
            models.append(np.full(nrow, model, np.int64))
            thr.append(np.full(nrow, threshold))
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
    si, sf, vals, sds, kinds, models, thr = (cat(si, np.int32), cat(sf, np.int32), cat(vals, np.float64),
                                              cat(sds, np.float64), cat(kinds, np.int32), cat(models, np.int32),
                                              cat(thr, np.float64))
    cptr = np.concatenate([[0], np.cumsum(cat(ncell, np.int64))]).astype(np.int32)
    cells = cat(cells, np.int32)
    n = len(si)
    return {
        "obs_sett_i": np.array(si, np.int32), "obs_sett_f": np.array(sf, np.int32),
        "obs_value_kind": np.array(kinds, np.int32), "obs_value": np.array(vals, np.float64),
        "obs_model": np.array(models, np.int32), "obs_sd": np.array(sds, np.float64),
        "obs_shape": np.zeros(n), "obs_threshold": np.array(thr, np.float64), "obs_factor": np.ones(n),
        "obs_factor_spline": np.full(n, -1, np.int32), "obs_cell_ptr": np.array(cptr, np.int32),
        "obs_cells": np.array(cells, np.int32),
    }


def _star_values(spec: str) -> np.ndarray:
    """A '|'-separated value list where '*' stands for what completes the others to 1."""
    parts = [p.strip() for p in spec.split("|")]
    vals = [float(p) for p in parts if p != "*"]
    return np.array([1.0 - sum(vals) if p == "*" else float(p) for p in parts])


def _disc_spline(days: int, S: int, bp: Sequence[float], vals: Sequence[float]) -> np.ndarray:
    """Model::create_disc_spline (src/model.cc:1018-1041), factor 1, multfac 1."""
    out = np.zeros(S)
    p = 0
    for s in range(S):
        t = float((s + 0.5) * days) / S
        while p + 1 < len(bp) and t > bp[p + 1]:
            p += 1
        if p + 1 == len(bp):
            out[s] = out[s - 1]
        else:
            fac = (t - bp[p]) / (bp[p + 1] - bp[p])
            out[s] = 1.0 * (vals[p] * 1.0 * (1 - fac) + vals[p + 1] * 1.0 * fac)
    return out


def age_matrix(w: synth.Workload) -> np.ndarray:
    """genQ.N[0] after Data::age_mixing_matrix + agematrix_normalise."""
    G = w.nage
    if G == 1:
        return np.ones((1, 1))
    pop = np.asarray(w.pop, np.int64)
    popa = pop.sum(0)                     # unsigned accumulation per age
    poptot = float(pop.sum())
    m = np.array(w.age_mix, np.float64)
    for j in range(G):
        for i in range(G):
            m[j, i] = m[j, i] / (float(popa[j]) / poptot)
    sym = np.empty_like(m)
    for j in range(G):
        for i in range(G):
            sym[j, i] = 0.5 * (m[j, i] + m[i, j])
    s = 0.0
    s2 = 0.0
    for a in range(G):
        for aa in range(G):
            s += float(popa[aa]) * sym[aa, a]
            s2 += float(popa[aa])
    s /= s2
    return sym / s


def param_tables(w: synth.Workload, sigma_inv: Optional[float] = None, gamma_inv: Optional[float] = None,
                 R_scale: float = 1.0, h_mean: Optional[float] = None) -> Dict[str, np.ndarray]:
    """set_param tables for one parameter set (defaults: the workload's true values).

    ``R_scale`` multiplies every knot of R(t) (an R0 proposal)."""
    A, G = w.narea, w.nage
    NS = nstrain(w)
    DP, C, T, S = G * NS, len(COMPS), len(TRANS), w.ndivision
    si = w.sigma_inv if sigma_inv is None else sigma_inv
    gi = w.gamma_inv if gamma_inv is None else gamma_inv
    hm = w.h_mean if h_mean is None else h_mean
    transrate = np.zeros((T, DP))
    transrate[1, :] = 1.0 / si
    transrate[2, :] = (1.0 / gi) * w.p_H
    transrate[3, :] = (1.0 / gi) * (1 - w.p_H)
    transrate[4, :] = (1.0 / hm) * w.p_D
    transrate[5, :] = (1.0 / hm) * (1 - w.p_D)
    # Model::create_susceptibility: the product over democats (ages have none, strains
    # their values, '*' completing them to 1); R factors per strain
    strain_sus, rfactor = np.ones(NS), np.ones(NS)
    if NS > 1:
        strain_sus = _star_values(w.strains["sus_value"])
        rfactor = _star_values(w.strains["Rfactor_value"])
    sus = np.repeat(strain_sus, G)
    inf = np.zeros(C)
    inf[2] = 1.0
    N0 = age_matrix(w)
    Ntime = np.repeat(N0[None], S, axis=0)
    for mm in w.matmod:
        f = _disc_spline(w.days, S, mm["bp"], mm["val"])
        for s in range(S):
            for a in mm["ages"]:
                Ntime[s, a, :] *= f[s]
                Ntime[s, :, a] *= f[s]
    Rv = [v * R_scale for v in w.R_val]
    Rspl = _disc_spline(w.days, S, w.R_bp, Rv)
    pop = np.asarray(w.pop, np.float64)
    dist = pop.sum(0) / pop.sum()
    # per strain st: NGM over the infectious states E, I of that strain's age groups
    # (Model::calculate_beta_from_R, calculate_Vinv, calculate_F, src/model.cc:1318-1362)
    Q = G
    beta = np.zeros((NS, S))
    for st in range(NS):
        V = np.zeros((2 * Q, 2 * Q))
        for q in range(Q):
            dp = st * Q + q
            V[q, q] += transrate[1, dp]
            V[Q + q, q] -= transrate[1, dp]
            V[Q + q, Q + q] += transrate[2, dp]
            V[Q + q, Q + q] += transrate[3, dp]
        Vinv = np.linalg.inv(V)
        ratio = None
        for s in range(S):
            if s == 0 or not np.array_equal(Ntime[s - 1], Ntime[s]):
                F = np.zeros((Q, 2 * Q))
                for a in range(Q):
                    for q in range(Q):
                        F[q, Q + a] += dist[q] * sus[st * Q + q] * 1.0 * Ntime[s][q, a]
                NGM = F @ Vinv[:, :Q]
                ratio = float(np.max(np.linalg.eigvals(NGM).real))
            beta[st, s] = rfactor[st] * Rspl[s] / ratio
    # area factors: covariates (linear) normalised by the population-weighted mean
    af = np.ones((w.days, A))
    if w.covar is not None:
        for j in range(w.covar.shape[0]):
            for c in range(A):
                af[:, c] *= np.exp(w.covar_effect[j] * w.covar[j, c])
        tp = np.asarray(w.pop, np.int64).sum(1)
        area_av = 0.0
        for c in range(A):
            av = _seq_sum(af[:, c]) / w.days
            area_av += av * float(tp[c])
        area_av /= float(tp.sum())
        af = af / area_av
    return {
        "transrate": transrate, "susceptibility": sus, "infectivity": inf,
        "beta_rows": beta, "beta_row_of": np.repeat(np.arange(NS, dtype=np.int32)[:, None], A, 1),
        "areafactor": af, "Ntime": Ntime, "geo_spline": np.ones(S),
        "efoi_spline": np.full((1, S), float(w.efoi)), "efoi_agedist": np.ones((1, G)),
        "efoi_ref": np.zeros((NS, A), np.int32), "obs_spline": np.zeros((0, S)),
    }


def param_tables_batch(w: synth.Workload, R0, sigma_inv, gamma_inv) -> List[Dict[str, np.ndarray]]:
    """set_param tables for many parameter sets that differ only in R0 (a
    constant R(t)), 1/sigma and 1/gamma.  Tables that do not depend on these
    are the same numpy arrays in every set (so the C ABI shares them)."""
    base = param_tables(w)
    n = len(R0)
    S, DP = w.ndivision, w.nage
    out = []
    N0 = base["Ntime"][0]
    pop = np.asarray(w.pop, np.float64)
    dist = pop.sum(0) / pop.sum()
    # NGM = diag(dist) N0 * v with v = Vinv[I,E] = 1/(gamma p_H + gamma (1-p_H)) for every age
    lam0 = float(np.max(np.linalg.eigvals(dist[:, None] * N0).real))
    for k in range(n):
        g = 1.0 / gamma_inv[k]
        tr = base["transrate"].copy()
        tr[1, :] = 1.0 / sigma_inv[k]
        tr[2, :] = g * w.p_H
        tr[3, :] = g * (1 - w.p_H)
        v = 1.0 / (tr[2, 0] + tr[3, 0])
        beta = np.full((1, S), float(R0[k]) / (v * lam0))
        t = dict(base)
        t["transrate"] = tr
        t["beta_rows"] = beta
        out.append(t)
    return out


def observed_from_trajectory(arr: Dict[str, np.ndarray], transnum: np.ndarray, pop_traj: np.ndarray,
                             rng) -> Tuple[np.ndarray, np.ndarray]:
    """Observed values = the trajectory's sums over each observation's cells and
    steps plus normal noise of variance max(count, 5); SD column sqrt(max(y, 5))."""
    S = transnum.shape[0]
    tn = transnum.reshape(S, -1).astype(np.int64)
    pp = pop_traj.reshape(S, -1).astype(np.int64)
    ctn = np.vstack([np.zeros((1, tn.shape[1]), np.int64), np.cumsum(tn, 0)])
    cpp = np.vstack([np.zeros((1, pp.shape[1]), np.int64), np.cumsum(pp, 0)])
    ptr = arr["obs_cell_ptr"]
    cells = arr["obs_cells"]
    si, sf = arr["obs_sett_i"], arr["obs_sett_f"]
    nobs = len(si)
    oid = np.repeat(np.arange(nobs), np.diff(ptr))
    vals = np.zeros(nobs, np.int64)
    tmask = cells >= 0
    tc = cells[tmask]
    to = oid[tmask]
    np.add.at(vals, to, ctn[sf[to], tc] - ctn[si[to], tc])
    pc = -1 - cells[~tmask]
    po = oid[~tmask]
    np.add.at(vals, po, cpp[sf[po], pc] - cpp[si[po], pc])
    v = vals.astype(np.float64)
    noisy = np.maximum(0, np.round(v + rng.normal(0.0, 1.0, nobs) * np.sqrt(np.maximum(v, 5.0))))
    return noisy, np.sqrt(np.maximum(noisy, 5.0))
