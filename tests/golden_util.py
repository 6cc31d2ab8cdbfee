"""Helpers for loading the golden fixtures."""
from __future__ import annotations

import os

import numpy as np

from beep_gb300 import bundle, capi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["tiny_sim", "oneage_sim", "c0_sim"]
PF_FIXTURES = ["tiny_pf", "c0_pf"]


def load(name):
    b = bundle.read_bundle(os.path.join(GOLDEN, f"{name}.bnd"))
    m, tabs = capi.load_model_bundle(b)
    seed = int(np.uint32(b["seed_words"][0])) | (int(np.uint32(b["seed_words"][1])) << 32)
    return b, m, tabs, seed


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
    return np.array([tn.sum(), (tn * wt).sum(), pp.sum(), (pp * wp).sum()])
