"""Loads the oracle restatement (oracle/_build/libbeep_oracle.so) for tests and
the CPU baseline.  The oracle is the parity checker, never the product."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

from beep_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_LIB = None


def oracle_lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(ORACLE_DIR, "_build", "libbeep_oracle.so")
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
        L = C.CDLL(path)
        L.beep_oracle_simulate.argtypes = [C.POINTER(capi.ModelDesc), C.POINTER(capi.SimBatch), C.c_int]
        L.beep_oracle_simulate.restype = C.c_int
        L.beep_oracle_poisson.argtypes = [C.c_double, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.beep_oracle_poisson.restype = C.c_int32
        L.beep_oracle_binomial.argtypes = [C.c_double, C.c_int32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                           C.c_uint32]
        L.beep_oracle_binomial.restype = C.c_int32
        for f in ("beep_oracle_exp", "beep_oracle_log", "beep_oracle_log_factorial"):
            getattr(L, f).argtypes = [C.c_double]
            getattr(L, f).restype = C.c_double
        L.beep_oracle_obs_prob.argtypes = [C.c_double, C.c_int32, C.c_double, C.c_int32, C.c_double, C.c_double,
                                           C.c_double]
        L.beep_oracle_obs_prob.restype = C.c_double
        L.beep_oracle_pf.argtypes = [C.POINTER(capi.ModelDesc), C.POINTER(capi.ParamTables), C.c_int32, C.c_uint64,
                                     C.c_uint32, C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.beep_oracle_pf.restype = C.c_int
        L.beep_oracle_abcsmc_weights.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                                 C.c_void_p, C.c_void_p, C.c_double, C.c_int32, C.c_void_p]
        L.beep_oracle_abcsmc_weights.restype = None
        L.beep_oracle_mbp.argtypes = [C.POINTER(capi.ModelDesc), C.c_int32, C.POINTER(capi.ParamTables),
                                      C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int32,
                                      C.c_void_p] + [C.c_void_p] * 6 + [C.c_int]
        L.beep_oracle_mbp.restype = C.c_int
        _LIB = L
    return _LIB


def oracle_simulate(model: capi.Model, batch: capi.Batch, nthreads: int = 0) -> capi.Batch:
    st = oracle_lib().beep_oracle_simulate(C.byref(model.desc), C.byref(batch.st), nthreads)
    if st != 0:
        raise RuntimeError(f"oracle failed: {capi.STATUS.get(st, st)}")
    return batch


def oracle_pf(model: capi.Model, tables: capi.Tables, N: int, seed: int, resample_stream: int, invT: float,
              sections, nthreads: int = 0, lineage: bool = False):
    """Bootstrap particle filter of the oracle: (estimate, per-section terms, L [nsec][N], ancestors [nsec][N])
    and, with lineage, the sampled lineage's counts [S][A][T][DP] as a fifth element."""
    import numpy as np
    ti = np.array([a for a, _ in sections], np.int32)
    tf = np.array([b for _, b in sections], np.int32)
    ns = len(sections)
    ll = np.zeros(1)
    lls = np.zeros(ns)
    L = np.zeros((ns, N))
    anc = np.zeros((ns, N), np.int32)
    lin = np.zeros((model.ndivision, model.narea, model.ntrans, model.ndemocatpos), np.int32) if lineage else None
    st = oracle_lib().beep_oracle_pf(C.byref(model.desc), C.byref(tables.st), N, seed, resample_stream, invT, 0, ns,
                                     ti.ctypes.data, tf.ctypes.data, ll.ctypes.data, lls.ctypes.data, L.ctypes.data,
                                     anc.ctypes.data, None if lin is None else lin.ctypes.data, nthreads)
    if st != 0:
        raise RuntimeError(f"oracle particle filter failed: {capi.STATUS.get(st, st)}")
    if lineage:
        return float(ll[0]), lls, L, anc, lin
    return float(ll[0]), lls, L, anc


def oracle_abcsmc_weights(theta_new, logprior_new, theta_last, w_last, inv_cov, size, normalise=True):
    import numpy as np
    tn = np.ascontiguousarray(theta_new, np.float64)
    lp = np.ascontiguousarray(logprior_new, np.float64)
    tl = np.ascontiguousarray(theta_last, np.float64)
    wl = np.ascontiguousarray(w_last, np.float64)
    ic = np.ascontiguousarray(inv_cov, np.float64)
    out = np.zeros(tn.shape[0])
    oracle_lib().beep_oracle_abcsmc_weights(tn.shape[1], tn.shape[0], tn.ctypes.data, lp.ctypes.data, tl.shape[0],
                                            tl.ctypes.data, wl.ctypes.data, ic.ctypes.data, float(size),
                                            1 if normalise else 0, out.ctypes.data)
    return out


def oracle_mbp(model: capi.Model, tables, ginit, gprop, seed: int, sinit, sprop, inf_update: int, simu=None,
               want_tn: bool = False, nthreads: int = 0):
    """MBP chains of the oracle: dict of L_init, L_prop, Li_init, Li_fixed (and tn_init / tn_prop)."""
    import numpy as np
    nc = len(ginit)
    groups = (capi.ParamTables * len(tables))(*[t.st for t in tables])
    gi = np.ascontiguousarray(ginit, np.int32)
    gp = np.ascontiguousarray(gprop, np.int32)
    si = np.ascontiguousarray(sinit, np.uint32)
    sp = np.ascontiguousarray(sprop, np.uint32)
    sm = None if simu is None else np.ascontiguousarray(simu, np.uint8)
    out = {k: np.zeros(nc) for k in ("L_init", "L_prop", "Li_init", "Li_fixed")}
    shape = (nc, model.ndivision, model.narea, model.ntrans, model.ndemocatpos)
    if want_tn:
        out["tn_init"] = np.zeros(shape, np.int32)
        out["tn_prop"] = np.zeros(shape, np.int32)
    p = lambda a: None if a is None else a.ctypes.data
    st = oracle_lib().beep_oracle_mbp(C.byref(model.desc), nc, groups, p(gi), p(gp), seed, p(si), p(sp), inf_update,
                                      p(sm), p(out["L_init"]), p(out["L_prop"]), p(out["Li_init"]),
                                      p(out["Li_fixed"]), p(out.get("tn_init")), p(out.get("tn_prop")), nthreads)
    if st != 0:
        raise RuntimeError(f"oracle failed: {capi.STATUS.get(st, st)}")
    return out
