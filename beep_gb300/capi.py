"""ctypes binding of the C ABI declared in include/beep_gpu.h.

This is the binding a Python caller (or a test) uses; the structures mirror
the header field for field.  ``Model`` and ``Tables`` keep the numpy arrays
that back the structures alive for as long as the structures are in use.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import weakref
from typing import Dict, List, Optional, Sequence

import numpy as np

_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_f64p = C.POINTER(C.c_double)

STATUS = {0: "OK", 1: "BAD_INPUT", 2: "NAN_RATE", 3: "OOM", 4: "TIMEOUT", 5: "DEVICE_ERROR",
          6: "NO_DEVICE", 7: "COUNT_OVERFLOW"}

FORM_PLAIN_FP64 = 0
FORM_FAST = 1


class ModelDesc(C.Structure):
    _fields_ = [
        ("narea", C.c_int32), ("nage", C.c_int32), ("ndemocatpos", C.c_int32), ("nstrain", C.c_int32),
        ("ncomp", C.c_int32), ("ntrans", C.c_int32),
        ("ndivision", C.c_int32), ("period", C.c_int32), ("division_per_time", C.c_int32),
        ("dt", C.c_double), ("popsize", C.c_double),
        ("trans_from", _i32p), ("trans_to", _i32p), ("infection_trans", C.c_int32), ("democatpos_age", _i32p),
        ("M_diag", _f64p), ("M_rowptr", _i32p), ("M_to", _i32p), ("M_val", _f64p), ("M_factor", _f64p),
        ("pop_init", _f64p),
        ("nobs", C.c_int32),
        ("obs_sett_i", _i32p), ("obs_sett_f", _i32p), ("obs_value_kind", _i32p), ("obs_value", _f64p),
        ("obs_model", _i32p), ("obs_sd", _f64p), ("obs_shape", _f64p), ("obs_threshold", _f64p),
        ("obs_factor", _f64p), ("obs_factor_spline", _i32p), ("obs_cell_ptr", _i32p), ("obs_cells", _i32p),
        ("ndemocat_change", C.c_int32), ("dcc_nval", _i32p), ("dcc_area_ptr", _i32p), ("dcc_area", _i32p),
        ("dcc_dp_ptr", _i32p), ("dcc_dp", _i32p), ("dcc_frac", _f64p),
    ]


DCC_INT_ARRAYS = ("dcc_nval", "dcc_area_ptr", "dcc_area", "dcc_dp_ptr", "dcc_dp")


class PriorSpec(C.Structure):
    _fields_ = [
        ("nparam", C.c_int32), ("type", _i32p), ("val1", _f64p), ("val2", _f64p), ("val1_param", _i32p),
        ("val2_param", _i32p), ("gt_ptr", _i32p), ("gt_param", _i32p), ("lt_ptr", _i32p), ("lt_param", _i32p),
        ("ndirichlet", C.c_int32), ("dir_ptr", _i32p), ("dir_param", _i32p), ("dir_frac", _f64p),
        ("nsmooth", C.c_int32), ("smooth_kind", _i32p), ("smooth_par1", _i32p), ("smooth_par2", _i32p),
        ("smooth_mult1", _f64p), ("smooth_mult2", _f64p), ("smooth_value", _f64p), ("ml_mode", C.c_int32),
    ]


PRIOR_INT_ARRAYS = ("type", "val1_param", "val2_param", "gt_ptr", "gt_param", "lt_ptr", "lt_param", "dir_ptr",
                    "dir_param", "smooth_kind", "smooth_par1", "smooth_par2")
PRIOR_F64_ARRAYS = ("val1", "val2", "dir_frac", "smooth_mult1", "smooth_mult2", "smooth_value")


class Priors:
    """A ``beep_prior_spec`` over arrays named as its fields (e.g. a bundle's ``prior.*``)."""

    def __init__(self, arrays, prefix: str = "prior."):
        self.arr = {}
        self.st = PriorSpec()
        for k in PRIOR_INT_ARRAYS:
            self.arr[k] = np.ascontiguousarray(np.asarray(arrays.get(prefix + k, []), np.int32).reshape(-1))
            setattr(self.st, k, self.arr[k].ctypes.data_as(_i32p))
        for k in PRIOR_F64_ARRAYS:
            self.arr[k] = np.ascontiguousarray(np.asarray(arrays.get(prefix + k, []), np.float64).reshape(-1))
            setattr(self.st, k, self.arr[k].ctypes.data_as(_f64p))
        self.st.nparam = int(self.arr["type"].size)
        self.st.ndirichlet = int(self.arr["dir_ptr"].size) - 1 if self.arr["dir_ptr"].size else 0
        self.st.nsmooth = int(self.arr["smooth_kind"].size)
        self.st.ml_mode = int(np.asarray(arrays.get(prefix + "ml_mode", [0])).reshape(-1)[0])

    def evaluate(self, theta):
        """(log-prior [n], in bounds [n]) of parameter rows theta [n][nparam] (beep_log_prior)."""
        th = np.ascontiguousarray(np.asarray(theta, np.float64).reshape(-1, self.st.nparam))
        lp = np.zeros(th.shape[0])
        ib = np.zeros(th.shape[0], np.int32)
        check(lib().beep_log_prior(C.byref(self.st), th.shape[0], th.ctypes.data_as(_f64p), lp.ctypes.data_as(_f64p),
                                   ib.ctypes.data_as(_i32p)))
        return lp, ib.astype(bool)


class ParamTables(C.Structure):
    _fields_ = [
        ("transrate", _f64p), ("susceptibility", _f64p), ("infectivity", _f64p),
        ("nbeta_row", C.c_int32), ("beta_rows", _f64p), ("beta_row_of", _i32p),
        ("areafactor", _f64p), ("Ntime", _f64p), ("geo_spline", _f64p),
        ("nefoi", C.c_int32), ("efoi_spline", _f64p), ("efoi_agedist", _f64p), ("efoi_ref", _i32p),
        ("nobs_spline", C.c_int32), ("obs_spline", _f64p),
        ("efoi_mult", _f64p), ("transmean_mult", _f64p),
    ]


class SimBatch(C.Structure):
    _fields_ = [
        ("nparticle", C.c_int32), ("ngroup", C.c_int32), ("groups", C.POINTER(ParamTables)),
        ("group_of", _i32p), ("seed", C.c_uint64), ("stream_of", _u32p),
        ("ti", C.c_int32), ("tf", C.c_int32), ("pop_in", _i32p),
        ("L_out", _f64p), ("pop_out", _i32p), ("transnum_out", _i32p), ("pop_traj_out", _i32p),
        ("form", C.c_int32),
        ("pop_in_f64", _f64p), ("pop_out_f64", _f64p), ("pop_traj_out_f64", _f64p),
    ]


class PFRequest(C.Structure):
    _fields_ = [
        ("nparticle", C.c_int32), ("tables", C.POINTER(ParamTables)), ("seed", C.c_uint64),
        ("resample_stream", C.c_uint32), ("invT", C.c_double), ("nsection", C.c_int32),
        ("section_ti", _i32p), ("section_tf", _i32p), ("form", C.c_int32),
        ("loglik_out", _f64p), ("loglik_section_out", _f64p), ("L_out", _f64p), ("ancestors_out", _i32p),
        ("lineage_transnum_out", _i32p),
    ]


class MbpRequest(C.Structure):
    _fields_ = [
        ("groups", C.POINTER(ParamTables)), ("ngroup", C.c_int32), ("group_of", _i32p), ("seed", C.c_uint64),
        ("stream_of", _u32p), ("inf_update", C.c_int32), ("simu", C.POINTER(C.c_uint8)), ("L_out", _f64p),
    ]


INF_UPDATE = 0
INF_DIF_UPDATE = 1

ABI_VERSION = 4   # BEEP_GPU_ABI_VERSION of include/beep_gpu.h these structures mirror

REQ_LIKELIHOOD, REQ_SCENARIO, REQ_PREDICTION, REQ_PF_LIKELIHOOD = 0, 1, 2, 3


class Request(C.Structure):
    _fields_ = [("kind", C.c_int32), ("model", C.POINTER(ModelDesc)), ("batch", C.POINTER(SimBatch)),
                ("pf", C.POINTER(PFRequest))]


class RequestStats(C.Structure):
    _fields_ = [("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("gpu_start_s", C.c_double), ("gpu_end_s", C.c_double), ("device_bytes", C.c_int64),
                ("state", C.c_int32), ("status", C.c_int32)]


def _ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(ctype))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


MODEL_INT_ARRAYS = ("trans_from", "trans_to", "democatpos_age", "M_rowptr", "M_to", "obs_sett_i", "obs_sett_f",
                    "obs_value_kind", "obs_model", "obs_factor_spline", "obs_cell_ptr", "obs_cells")
MODEL_F64_ARRAYS = ("M_diag", "M_val", "M_factor", "pop_init", "obs_value", "obs_sd", "obs_shape", "obs_threshold",
                    "obs_factor")
TABLE_INT_ARRAYS = ("beta_row_of", "efoi_ref")
TABLE_F64_ARRAYS = ("transrate", "susceptibility", "infectivity", "beta_rows", "areafactor", "Ntime", "geo_spline",
                    "efoi_spline", "efoi_agedist", "obs_spline")


class Model:
    """Parameter-independent model arrays + the ``beep_model_desc`` over them."""

    def __init__(self, arrays: Dict[str, np.ndarray]):
        d = arrays
        dims = [int(x) for x in d["dims"]]
        (self.narea, self.nage, self.ndemocatpos, self.nstrain, self.ncomp, self.ntrans,
         self.ndivision, self.period, self.division_per_time) = dims
        self.dt = float(np.asarray(d["dt"]).reshape(-1)[0])
        self.popsize = float(np.asarray(d["popsize"]).reshape(-1)[0])
        self.infection_trans = int(np.asarray(d["infection_trans"]).reshape(-1)[0])
        self.arr: Dict[str, np.ndarray] = {}
        for k in MODEL_INT_ARRAYS:
            self.arr[k] = _i32(d[k]).reshape(-1)
        for k in MODEL_F64_ARRAYS:
            self.arr[k] = _f64(d[k]).reshape(-1)
        self.nobs = int(self.arr["obs_sett_i"].size)
        self.desc = ModelDesc()
        for k in ("narea", "nage", "ndemocatpos", "nstrain", "ncomp", "ntrans", "ndivision", "period",
                  "division_per_time", "infection_trans", "nobs"):
            setattr(self.desc, k, getattr(self, k))
        self.desc.dt = self.dt
        self.desc.popsize = self.popsize
        for k in MODEL_INT_ARRAYS:
            setattr(self.desc, k, _ptr(self.arr[k], C.c_int32))
        for k in MODEL_F64_ARRAYS:
            setattr(self.desc, k, _ptr(self.arr[k], C.c_double))
        # demographic changes (optional): populations become FP64
        self.ndemocat_change = int(np.asarray(d["dcc_nval"]).size) if "dcc_nval" in d else 0
        self.pop64 = self.ndemocat_change > 0
        if self.pop64:
            for k in DCC_INT_ARRAYS:
                self.arr[k] = _i32(d[k]).reshape(-1)
                setattr(self.desc, k, _ptr(self.arr[k], C.c_int32))
            self.arr["dcc_frac"] = _f64(d["dcc_frac"]).reshape(-1)
            self.desc.dcc_frac = _ptr(self.arr["dcc_frac"], C.c_double)
            self.desc.ndemocat_change = self.ndemocat_change
        self.sections = None
        if "section_ti" in d:
            self.sections = list(zip(_i32(d["section_ti"]).tolist(), _i32(d["section_tf"]).tolist()))

    @property
    def pop_size(self) -> int:
        return self.narea * self.ncomp * self.ndemocatpos

    @property
    def trans_size(self) -> int:
        return self.narea * self.ntrans * self.ndemocatpos


class Tables:
    """One parameter set's tables (``beep_param_tables``)."""

    def __init__(self, arrays: Dict[str, np.ndarray], prefix: str = ""):
        self.arr: Dict[str, np.ndarray] = {}
        for k in TABLE_INT_ARRAYS:
            self.arr[k] = _i32(arrays[prefix + k]).reshape(-1)
        for k in TABLE_F64_ARRAYS:
            self.arr[k] = _f64(arrays[prefix + k]).reshape(-1)
        self.shapes = {k: np.asarray(arrays[prefix + k]).shape for k in TABLE_INT_ARRAYS + TABLE_F64_ARRAYS}
        self.st = ParamTables()
        for k in TABLE_INT_ARRAYS:
            setattr(self.st, k, _ptr(self.arr[k], C.c_int32))
        for k in TABLE_F64_ARRAYS:
            setattr(self.st, k, _ptr(self.arr[k], C.c_double))
        for k in ("efoi_mult", "transmean_mult"):        # prediction modifications (optional)
            if arrays.get(prefix + k) is not None:
                self.arr[k] = _f64(arrays[prefix + k]).reshape(-1)
                setattr(self.st, k, _ptr(self.arr[k], C.c_double))
        self.st.nbeta_row = int(self.shapes["beta_rows"][0])
        self.st.nefoi = int(self.shapes["efoi_spline"][0])
        self.st.nobs_spline = int(self.shapes["obs_spline"][0]) if len(self.shapes["obs_spline"]) == 2 else 0


class Batch:
    """A ``beep_sim_batch`` plus the output arrays it writes into."""

    def __init__(self, model: Model, tables: Sequence[Tables], nparticle: int, seed: int, ti: int = 0,
                 tf: Optional[int] = None, group_of=None, stream_of=None, pop_in=None,
                 want_L: bool = True, want_pop: bool = False, want_transnum: bool = False,
                 want_pop_traj: bool = False, form: int = FORM_PLAIN_FP64):
        tf = model.ndivision if tf is None else tf
        self.tables = list(tables)
        self.groups = (ParamTables * max(1, len(self.tables)))(*[t.st for t in self.tables])
        self.group_of = None if group_of is None else _i32(group_of)
        self.stream_of = None if stream_of is None else np.ascontiguousarray(np.asarray(stream_of, np.uint32))
        # populations: int32, or FP64 for a model with demographic changes
        pdt = np.float64 if model.pop64 else np.int32
        self.pop_in = None if pop_in is None else np.ascontiguousarray(np.asarray(pop_in, pdt))
        ns = tf - ti
        self.L = np.zeros(nparticle, np.float64) if want_L else None
        self.pop = np.zeros((nparticle, model.narea, model.ncomp, model.ndemocatpos), pdt) if want_pop else None
        self.transnum = (np.zeros((nparticle, ns, model.narea, model.ntrans, model.ndemocatpos), np.int32)
                         if want_transnum else None)
        self.pop_traj = (np.zeros((nparticle, ns, model.narea, model.ncomp, model.ndemocatpos), pdt)
                         if want_pop_traj else None)
        b = SimBatch()
        b.nparticle = nparticle
        b.ngroup = len(self.tables)
        b.groups = self.groups
        b.group_of = _ptr(self.group_of, C.c_int32)
        b.seed = seed
        b.stream_of = _ptr(self.stream_of, C.c_uint32)
        b.ti, b.tf = ti, tf
        b.L_out = _ptr(self.L, C.c_double)
        b.transnum_out = _ptr(self.transnum, C.c_int32)
        if model.pop64:
            b.pop_in_f64 = _ptr(self.pop_in, C.c_double)
            b.pop_out_f64 = _ptr(self.pop, C.c_double)
            b.pop_traj_out_f64 = _ptr(self.pop_traj, C.c_double)
        else:
            b.pop_in = _ptr(self.pop_in, C.c_int32)
            b.pop_out = _ptr(self.pop, C.c_int32)
            b.pop_traj_out = _ptr(self.pop_traj, C.c_int32)
        b.form = form
        self.st = b


def load_model_bundle(arrays: Dict[str, np.ndarray]):
    """(Model, [Tables per parameter set]) from a bundle's arrays."""
    m = Model(arrays)
    ng = int(np.asarray(arrays.get("ngroup", [1])).reshape(-1)[0])
    return m, [Tables(arrays, f"g{k}.") for k in range(ng)]


# ---------------------------------------------------------------------------
# the CUDA library

_LIB = None


def library_path() -> str:
    """In-tree libbeep_gpu.so; BEEP_GPU_LIB overrides the path (for instrumented builds)."""
    return os.environ.get("BEEP_GPU_LIB") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "libbeep_gpu.so")


def lib():
    """Loads libbeep_gpu.so (built by ``beep_gb300.build``); raises if it is missing."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build the CUDA library first (beep_gb300.build.build())")
        L = C.CDLL(path)
        L.beep_abi_version.restype = C.c_int32
        L.beep_last_error.restype = C.c_char_p
        L.beep_device_init.argtypes = [C.c_int32]
        L.beep_model_create.argtypes = [C.POINTER(ModelDesc), C.POINTER(C.c_void_p)]
        L.beep_model_destroy.argtypes = [C.c_void_p]
        L.beep_simulate.argtypes = [C.c_void_p, C.POINTER(SimBatch)]
        L.beep_batch_create.argtypes = [C.c_void_p, C.POINTER(SimBatch), C.POINTER(C.c_void_p)]
        for f in ("beep_batch_stage", "beep_batch_upload", "beep_batch_launch", "beep_batch_download",
                  "beep_batch_destroy"):
            getattr(L, f).argtypes = [C.c_void_p]
        L.beep_batch_time.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]
        L.beep_batch_time_split.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.beep_batch_time_split.restype = C.c_int32
        L.beep_batch_time_kernels.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double), _f64p]
        L.beep_batch_time_kernels.restype = C.c_int32
        L.beep_batch_run_graph.argtypes = [C.c_void_p]
        L.beep_batch_run_graph.restype = C.c_int32
        L.beep_autotune.argtypes = [C.c_void_p, C.POINTER(SimBatch), C.POINTER(C.c_int32)]
        L.beep_autotune.restype = C.c_int32
        L.beep_batch_foi_path.argtypes = [C.c_void_p]
        L.beep_batch_foi_path.restype = C.c_int32
        L.beep_batch_ctas_per_sm.argtypes = [C.c_void_p]
        L.beep_batch_ctas_per_sm.restype = C.c_int32
        L.beep_batch_launches.argtypes = [C.c_void_p]
        L.beep_batch_launches.restype = C.c_int32
        L.beep_batch_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.beep_batch_bytes.restype = C.c_int32
        L.beep_simulate_plain_noalloc.argtypes = [C.c_void_p, C.POINTER(ParamTables), C.c_int32, C.c_uint64,
                                                  C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p]
        L.beep_simulate_plain_noalloc.restype = C.c_int32
        L.beep_abcsmc_weights.argtypes = [C.c_int32, C.c_int32, _f64p, _f64p, C.c_int32, _f64p, _f64p, _f64p,
                                          C.c_double, C.c_int32, _f64p]
        L.beep_abcsmc_weights.restype = C.c_int32
        L.beep_log_prior.argtypes = [C.POINTER(PriorSpec), C.c_int32, _f64p, _f64p, _i32p]
        L.beep_log_prior.restype = C.c_int32
        L.beep_pf_loglik.argtypes = [C.c_void_p, C.POINTER(PFRequest)]
        L.beep_pf_loglik.restype = C.c_int32
        L.beep_set_option.argtypes = [C.c_char_p, C.c_int64]
        L.beep_set_option.restype = C.c_int32
        L.beep_mbp_create.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]
        L.beep_mbp_destroy.argtypes = [C.c_void_p]
        for f in ("beep_mbp_initialise", "beep_mbp_propose"):
            getattr(L, f).argtypes = [C.c_void_p, C.POINTER(MbpRequest)]
        L.beep_mbp_set_state.argtypes = [C.c_void_p, C.POINTER(MbpRequest), _i32p]
        L.beep_mbp_propose_fused.argtypes = [C.c_int32, C.POINTER(C.c_void_p), C.POINTER(MbpRequest)]
        L.beep_mbp_set_state.restype = C.c_int32
        L.beep_mbp_accept.argtypes = [C.c_void_p, C.POINTER(C.c_uint8)]
        L.beep_mbp_state_likelihood.argtypes = [C.c_void_p, C.POINTER(MbpRequest), _f64p]
        L.beep_mbp_acceptance.argtypes = [C.c_int32] + [C.c_double] * 6
        L.beep_mbp_acceptance.restype = C.c_double
        L.beep_mbp_read_state.argtypes = [C.c_void_p, C.c_int32, _i32p, _f64p]
        L.beep_mbp_ctas_per_sm.argtypes = [C.c_void_p]
        L.beep_mbp_ctas_per_sm.restype = C.c_int32
        for f in ("beep_mbp_create", "beep_mbp_destroy", "beep_mbp_initialise", "beep_mbp_propose", "beep_mbp_accept",
                  "beep_mbp_state_likelihood", "beep_mbp_read_state"):
            getattr(L, f).restype = C.c_int32
        L.beep_server_create.argtypes = [C.c_int32, C.c_int64, C.c_int32, C.POINTER(C.c_void_p)]
        L.beep_server_destroy.argtypes = [C.c_void_p]
        L.beep_serve_submit.argtypes = [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_uint64)]
        L.beep_serve_poll.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_int32)]
        L.beep_serve_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_double]
        L.beep_serve_stats.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(RequestStats)]
        L.beep_serve_release.argtypes = [C.c_void_p, C.c_uint64]
        for f in ("beep_server_create", "beep_server_destroy", "beep_serve_submit", "beep_serve_poll",
                  "beep_serve_wait", "beep_serve_stats", "beep_serve_release"):
            getattr(L, f).restype = C.c_int32
        for f in ("beep_device_init", "beep_model_create", "beep_model_destroy", "beep_simulate", "beep_batch_create",
                  "beep_batch_stage", "beep_batch_upload", "beep_batch_launch", "beep_batch_download",
                  "beep_batch_time", "beep_batch_destroy"):
            getattr(L, f).restype = C.c_int32
        _LIB = L
    return _LIB


FOI_AUTO, FOI_SIMT, FOI_TENSOR, FOI_BATCHED = 0, 1, 2, 3


def set_option(name: str, value: int) -> None:
    """Process-wide library option (beep_set_option), e.g. ``set_option("fast_foi", FOI_TENSOR)``."""
    check(lib().beep_set_option(name.encode(), int(value)))


class BeepError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def check(status: int) -> None:
    if status != 0:
        raise BeepError(status, (lib().beep_last_error() or b"").decode())


# Handles still open at interpreter exit are closed here, dependents first
# (servers and MBP chain sets, then batches, then models), while the library
# and the CUDA runtime are still loaded; finalisers at shutdown run in no
# defined order.
_OPEN: Dict[int, "weakref.WeakSet"] = {0: weakref.WeakSet(), 1: weakref.WeakSet(), 2: weakref.WeakSet()}


def _track(obj, rank: int):
    _OPEN[rank].add(obj)


@atexit.register
def _close_open_handles():
    for rank in (0, 1, 2):
        for obj in list(_OPEN[rank]):
            try:
                obj.close()
            except Exception:
                pass


class DeviceModel:
    """A ``beep_model`` handle on the GPU."""

    def __init__(self, model: Model, device: int = 0):
        L = lib()
        check(L.beep_device_init(device))
        self.model = model
        h = C.c_void_p()
        check(L.beep_model_create(C.byref(model.desc), C.byref(h)))
        self.h = h
        # handles made on this model (batches, chain sets) that are still open: the
        # model is destroyed only after the last of them, whatever order the garbage
        # collector finalises them in
        self._deps = 0
        self._closing = False
        _track(self, 2)

    def simulate(self, batch: Batch) -> Batch:
        check(lib().beep_simulate(self.h, C.byref(batch.st)))
        return batch

    def autotune(self, batch: Batch) -> int:
        """Chooses the fast form's FOI path for this model by timing a sample of the batch."""
        c = C.c_int32()
        check(lib().beep_autotune(self.h, C.byref(batch.st), C.byref(c)))
        return c.value

    def pf_loglik(self, tables: "Tables", N: int, seed: int, resample_stream: int, invT: float, sections,
                  form: int = FORM_PLAIN_FP64, lineage: bool = False):
        """Bootstrap particle filter on the device: (estimate, per-section terms, L, ancestors) and, with
        lineage, the sampled particle's transition counts [S][A][T][DP] as a fifth element."""
        ti = np.array([a for a, _ in sections], np.int32)
        tf = np.array([b for _, b in sections], np.int32)
        ns = len(sections)
        ll = np.zeros(1)
        lls = np.zeros(ns)
        Lo = np.zeros((ns, N))
        anc = np.zeros((ns, N), np.int32)
        r = PFRequest()
        r.nparticle, r.tables, r.seed, r.resample_stream, r.invT = N, C.pointer(tables.st), seed, resample_stream, invT
        r.nsection, r.section_ti, r.section_tf, r.form = ns, _ptr(ti, C.c_int32), _ptr(tf, C.c_int32), form
        r.loglik_out, r.loglik_section_out = _ptr(ll, C.c_double), _ptr(lls, C.c_double)
        r.L_out, r.ancestors_out = _ptr(Lo, C.c_double), _ptr(anc, C.c_int32)
        m = self.model
        lin = np.zeros((m.ndivision, m.narea, m.ntrans, m.ndemocatpos), np.int32) if lineage else None
        r.lineage_transnum_out = _ptr(lin, C.c_int32)
        check(lib().beep_pf_loglik(self.h, C.byref(r)))
        if lineage:
            return float(ll[0]), lls, Lo, anc, lin
        return float(ll[0]), lls, Lo, anc

    def close(self):
        if self.h:
            if self._deps > 0:
                self._closing = True            # the last dependent handle destroys the model
                return
            lib().beep_model_destroy(self.h)
            self.h = None

    def _release_dep(self):
        self._deps -= 1
        if self._closing and self._deps == 0:
            self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceBatch:
    """A ``beep_batch``: a batch kept on the device and run repeatedly."""

    def __init__(self, dm: DeviceModel, batch: Batch):
        self.batch = batch
        self.dm = dm
        h = C.c_void_p()
        check(lib().beep_batch_create(dm.h, C.byref(batch.st), C.byref(h)))
        self.h = h
        dm._deps += 1
        _track(self, 1)

    def stage(self):
        check(lib().beep_batch_stage(self.h))

    def upload(self):
        check(lib().beep_batch_upload(self.h))

    def launch(self):
        check(lib().beep_batch_launch(self.h))

    def download(self) -> Batch:
        check(lib().beep_batch_download(self.h))
        return self.batch

    def run(self) -> Batch:
        self.upload()
        self.launch()
        return self.download()

    def run_graph(self) -> Batch:
        """stage + upload + launch + download with the device work replayed as a CUDA graph."""
        check(lib().beep_batch_run_graph(self.h))
        return self.batch

    def time(self, iters: int) -> float:
        ms = C.c_double()
        check(lib().beep_batch_time(self.h, iters, C.byref(ms)))
        return ms.value

    def time_split(self, iters: int):
        """(ms per launch, of which ms in the per-step tensor-core products) -- step-synchronous layout."""
        ms, prod = C.c_double(), C.c_double()
        check(lib().beep_batch_time_split(self.h, iters, C.byref(ms), C.byref(prod)))
        return ms.value, prod.value

    def time_kernels(self, iters: int):
        """(ms per launch, [ms in the products, the step kernels, the observation kernels]) --
        step-synchronous layout (zeros otherwise)."""
        ms, k3 = C.c_double(), np.zeros(3)
        check(lib().beep_batch_time_kernels(self.h, iters, C.byref(ms), k3.ctypes.data_as(_f64p)))
        return ms.value, k3

    def bytes(self):
        a, b = C.c_int64(), C.c_int64()
        check(lib().beep_batch_bytes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def launches(self) -> int:
        return lib().beep_batch_launches(self.h)

    def foi_path(self) -> int:
        """1 = FP32 SIMT force of infection, 2 = tensor cores (one particle per CTA), 3 = tensor cores
        batched over the particles (step-synchronous layout), 0 = plain form."""
        return lib().beep_batch_foi_path(self.h)

    def ctas_per_sm(self) -> int:
        """Particles (CTAs) per SM the fast-form kernel is laid out for; 0 = plain form or the
        step-synchronous layout (particles not pinned to SMs)."""
        return lib().beep_batch_ctas_per_sm(self.h)

    def close(self):
        if self.h:
            lib().beep_batch_destroy(self.h)
            self.h = None
            self.dm._release_dep()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def abcsmc_weights(theta_new, logprior_new, theta_last, w_last, inv_cov, size: float, normalise: bool = True):
    """ABC-SMC importance weights on the GPU (beep_abcsmc_weights)."""
    tn = _f64(theta_new)
    lp = _f64(logprior_new)
    tl = _f64(theta_last)
    wl = _f64(w_last)
    ic = _f64(inv_cov)
    out = np.zeros(tn.shape[0])
    check(lib().beep_abcsmc_weights(tn.shape[1], tn.shape[0], _ptr(tn, C.c_double), _ptr(lp, C.c_double),
                                    tl.shape[0], _ptr(tl, C.c_double), _ptr(wl, C.c_double), _ptr(ic, C.c_double),
                                    size, 1 if normalise else 0, _ptr(out, C.c_double)))
    return out


class MbpChains:
    """A ``beep_mbp_chains`` set: nchain MBP chains with two trajectory states each."""

    def __init__(self, dm: DeviceModel, nchain: int, form: int = FORM_PLAIN_FP64):
        self.dm = dm
        self.model = dm.model
        self.nchain = nchain
        h = C.c_void_p()
        check(lib().beep_mbp_create(dm.h, nchain, form, C.byref(h)))
        self.h = h
        dm._deps += 1
        _track(self, 0)

    def _request(self, tables: Sequence[Tables], seed: int, group_of=None, stream_of=None,
                 inf_update: int = INF_DIF_UPDATE, simu=None, want_L: bool = True):
        keep = {}
        r = MbpRequest()
        keep["groups"] = (ParamTables * len(tables))(*[t.st for t in tables])
        r.groups, r.ngroup = keep["groups"], len(tables)
        keep["go"] = None if group_of is None else _i32(group_of)
        r.group_of = _ptr(keep["go"], C.c_int32)
        r.seed = seed
        keep["so"] = None if stream_of is None else np.ascontiguousarray(np.asarray(stream_of, np.uint32))
        r.stream_of = _ptr(keep["so"], C.c_uint32)
        r.inf_update = inf_update
        keep["simu"] = None if simu is None else np.ascontiguousarray(np.asarray(simu, np.uint8))
        r.simu = _ptr(keep["simu"], C.c_uint8)
        keep["L"] = np.zeros(self.nchain) if want_L else None
        r.L_out = _ptr(keep["L"], C.c_double)
        return r, keep

    def initialise(self, tables: Sequence[Tables], seed: int, group_of=None, stream_of=None) -> np.ndarray:
        """State::simulate of every chain; returns the log-likelihoods."""
        r, keep = self._request(tables, seed, group_of, stream_of)
        check(lib().beep_mbp_initialise(self.h, C.byref(r)))
        return keep["L"]

    def set_state(self, tables: Sequence[Tables], transnum, group_of=None) -> np.ndarray:
        """State::initialise_from_particle of every chain from given counts; returns the log-likelihoods."""
        tn = np.ascontiguousarray(transnum, np.int32)
        r, keep = self._request(tables, 0, group_of)
        check(lib().beep_mbp_set_state(self.h, C.byref(r), _ptr(tn, C.c_int32)))
        return keep["L"]

    def propose(self, tables: Sequence[Tables], seed: int, group_of=None, stream_of=None,
                inf_update: int = INF_DIF_UPDATE, simu=None) -> np.ndarray:
        """Mbp::mbp of every chain; returns the proposals' log-likelihoods."""
        r, keep = self._request(tables, seed, group_of, stream_of, inf_update, simu)
        check(lib().beep_mbp_propose(self.h, C.byref(r)))
        return keep["L"]

    @staticmethod
    def propose_fused(sets: Sequence["MbpChains"], requests: Sequence[dict]) -> list:
        """Mbp::mbp of the chains of several chain sets (different models) in one
        persistent launch (beep_mbp_propose_fused).  requests[k] holds set k's
        propose() arguments (tables, seed, group_of, stream_of, inf_update, simu);
        returns each set's proposal log-likelihoods."""
        built = [c._request(q["tables"], q["seed"], q.get("group_of"), q.get("stream_of"),
                            q.get("inf_update", INF_DIF_UPDATE), q.get("simu")) for c, q in zip(sets, requests)]
        hs = (C.c_void_p * len(sets))(*[c.h for c in sets])
        rs = (MbpRequest * len(sets))(*[r for r, _ in built])
        check(lib().beep_mbp_propose_fused(len(sets), hs, rs))
        return [keep["L"] for _, keep in built]

    def accept(self, accept) -> None:
        a = np.ascontiguousarray(np.asarray(accept, np.uint8))
        check(lib().beep_mbp_accept(self.h, _ptr(a, C.c_uint8)))

    def state_likelihood(self, tables: Sequence[Tables], group_of=None) -> np.ndarray:
        """State::likelihood of every chain's current state under the given tables."""
        r, keep = self._request(tables, 0, group_of, want_L=False)
        out = np.zeros(self.nchain)
        check(lib().beep_mbp_state_likelihood(self.h, C.byref(r), _ptr(out, C.c_double)))
        return out

    def read_state(self, chain: int):
        m = self.model
        tn = np.zeros((m.ndivision, m.narea, m.ntrans, m.ndemocatpos), np.int32)
        mean = np.zeros(tn.shape, np.float64)
        check(lib().beep_mbp_read_state(self.h, chain, _ptr(tn, C.c_int32), _ptr(mean, C.c_double)))
        return tn, mean

    def ctas_per_sm(self) -> int:
        """Chains per SM of the fast form's last prepared batch (0: plain form or none yet)."""
        return lib().beep_mbp_ctas_per_sm(self.h)

    def close(self):
        if self.h:
            lib().beep_mbp_destroy(self.h)
            self.h = None
            self.dm._release_dep()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mbp_acceptance(cutoff: bool, invT: float, EFcut: float, EF_prop: float, EF_init: float, Pr_prop: float,
                   Pr_init: float) -> float:
    """Mbp::get_al (beep_mbp_acceptance)."""
    return lib().beep_mbp_acceptance(1 if cutoff else 0, invT, EFcut, EF_prop, EF_init, Pr_prop, Pr_init)


class Server:
    """A ``beep_server``: continuous batching of requests on one GPU."""

    def __init__(self, hbm_budget_bytes: int, max_inflight: int = 8, device: int = 0):
        h = C.c_void_p()
        check(lib().beep_server_create(device, int(hbm_budget_bytes), max_inflight, C.byref(h)))
        self.h = h
        self._live = {}
        _track(self, 0)

    def submit(self, model: Model, batch: Batch, kind: int = REQ_LIKELIHOOD) -> int:
        """Queues a request; the model and batch (and their arrays) are kept until it is released."""
        r = Request()
        r.kind = kind
        r.model = C.pointer(model.desc)
        r.batch = C.pointer(batch.st)
        t = C.c_uint64()
        check(lib().beep_serve_submit(self.h, C.byref(r), C.byref(t)))
        self._live[t.value] = (model, batch, r)
        return t.value

    def submit_pf(self, model: Model, tables: Tables, N: int, seed: int, resample_stream: int, invT: float,
                  sections, form: int = FORM_PLAIN_FP64, lineage: bool = False) -> int:
        """Queues a particle-filter likelihood request; wait() returns a dict with loglik,
        loglik_section, L [nsec][N], ancestors [nsec][N] (and lineage)."""
        ti = np.array([a for a, _ in sections], np.int32)
        tf = np.array([b for _, b in sections], np.int32)
        ns = len(sections)
        out = {"loglik": np.zeros(1), "loglik_section": np.zeros(ns), "L": np.zeros((ns, N)),
               "ancestors": np.zeros((ns, N), np.int32)}
        if lineage:
            out["lineage"] = np.zeros((model.ndivision, model.narea, model.ntrans, model.ndemocatpos), np.int32)
        r = PFRequest()
        r.nparticle, r.tables, r.seed, r.resample_stream, r.invT = N, C.pointer(tables.st), seed, resample_stream, invT
        r.nsection, r.section_ti, r.section_tf, r.form = ns, _ptr(ti, C.c_int32), _ptr(tf, C.c_int32), form
        r.loglik_out, r.loglik_section_out = _ptr(out["loglik"], C.c_double), _ptr(out["loglik_section"], C.c_double)
        r.L_out, r.ancestors_out = _ptr(out["L"], C.c_double), _ptr(out["ancestors"], C.c_int32)
        r.lineage_transnum_out = _ptr(out.get("lineage"), C.c_int32)
        rq = Request()
        rq.kind = REQ_PF_LIKELIHOOD
        rq.model = C.pointer(model.desc)
        rq.pf = C.pointer(r)
        t = C.c_uint64()
        check(lib().beep_serve_submit(self.h, C.byref(rq), C.byref(t)))
        self._live[t.value] = (model, tables, r, rq, ti, tf, out)
        return t.value

    def poll(self, ticket: int) -> bool:
        d = C.c_int32()
        check(lib().beep_serve_poll(self.h, ticket, C.byref(d)))
        return bool(d.value)

    def wait(self, ticket: int, timeout_s: float = -1.0):
        """The request's Batch (simulation kinds) or output dict (particle filter) once done."""
        check(lib().beep_serve_wait(self.h, ticket, timeout_s))
        live = self._live[ticket]
        return live[-1] if isinstance(live[-1], dict) else live[1]

    def stats(self, ticket: int) -> dict:
        st = RequestStats()
        check(lib().beep_serve_stats(self.h, ticket, C.byref(st)))
        return {k: getattr(st, k) for k, _ in RequestStats._fields_}

    def release(self, ticket: int) -> None:
        check(lib().beep_serve_release(self.h, ticket))
        self._live.pop(ticket, None)

    def close(self):
        if self.h:
            lib().beep_server_destroy(self.h)
            self.h = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
