"""Helpers for loading the golden fixtures."""
from __future__ import annotations

import os

import numpy as np

from beep_gb300 import bundle, capi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["tiny_sim", "oneage_sim", "c0_sim", "strain_sim", "obsmodel_sim", "features_sim", "pred_sim", "wide_sim",
            "democat_sim"]
# the fast form's fixtures: all but the demographic-change model (FP64 populations,
# plain form only)
FAST_FIXTURES = [f for f in FIXTURES if f != "democat_sim"]
PF_FIXTURES = ["tiny_pf", "c0_pf", "features_pf", "democat_pf"]
MBP_FIXTURES = ["tiny_mbp", "c0_mbp", "democat_mbp"]
MBP_VARIANTS = 3   # 0 INF_DIF_UPDATE, 1 INF_UPDATE, 2 INF_DIF_UPDATE with SIMU cells


def load(name):
    b = bundle.read_bundle(os.path.join(GOLDEN, f"{name}.bnd"))
    m, tabs = capi.load_model_bundle(b)
    seed = int(np.uint32(b["seed_words"][0])) | (int(np.uint32(b["seed_words"][1])) << 32)
    return b, m, tabs, seed


def prediction_runs(b):
    """The loaded-sample prediction runs of a prediction fixture: per sample k its
    tables (with the modifications' multipliers), start step, start populations
    [A][C][DP], stream, and the reference's counts [S-ti][A][T][DP] and final
    populations."""
    ti = int(b["pred.ti"][0])
    out = []
    for k in range(int(b["pred.n"][0])):
        p = f"pred{k}."
        out.append(dict(tables=capi.Tables(b, p), ti=ti, pop_ti=b[p + "pop_ti"], stream=int(b[p + "stream"][0]),
                        transnum=b[p + "transnum"], pop_end=b[p + "pop_end"]))
    return out


def checksums(transnum, pop):
    """The reference harness's four trajectory checksums for [S][A][T][DP] and [S][A][C][DP]."""
    S, A, T, DP = transnum.shape
    C = pop.shape[2]
    s, c, t, d = np.meshgrid(np.arange(S), np.arange(A), np.arange(T), np.arange(DP), indexing="ij")
    wt = 1 + ((s * 131 + c * 31 + t * 7 + d) % 1009)
    s2, c2, k2, d2 = np.meshgrid(np.arange(S), np.arange(A), np.arange(C), np.arange(DP), indexing="ij")
    wp = 1 + ((s2 * 131 + c2 * 31 + k2 * 7 + d2) % 1009)
    tn = transnum.astype(np.float64)
    pp = pop.astype(np.float64)
    # summed left to right in the harness's loop order (step, area, then transition or
    # compartment, then dp): exact for fractional populations too
    seq = lambda x: np.cumsum(x.ravel())[-1]
    return np.array([seq(tn), seq(tn * wt), seq(pp), seq(pp * wp)])


def mbp_case(b, v):
    """Inputs of MBP variant v of a fixture: (ginit, gprop, sinit, sprop, inf_update, simu)."""
    nc = int(b["mbp.nchain"][0])
    p = f"mbp{v}."
    simu = b[p + "simu"].astype(np.uint8)
    return (np.arange(nc) * 2, np.arange(nc) * 2 + 1, b[p + "stream_init"].astype(np.uint32),
            b[p + "stream_prop"].astype(np.uint32), int(b[p + "inf_update"][0]), simu if simu.any() else None)


def tn_checksums(transnum):
    """The reference harness's two transition-count checksums of [S][A][T][DP]."""
    S, A, T, DP = transnum.shape
    s, c, t, d = np.meshgrid(np.arange(S), np.arange(A), np.arange(T), np.arange(DP), indexing="ij")
    wt = 1 + ((s * 131 + c * 31 + t * 7 + d) % 1009)
    tn = transnum.astype(np.float64)
    return np.array([tn.sum(), (tn * wt).sum()])
