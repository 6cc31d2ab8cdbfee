"""beep_simulate_plain_noalloc: the plain FP64 simulation for callers that
cannot allocate device memory (an application whose own allocator or fixed
budget owns the GPU's memory).  The caller passes device buffers for the
tables, the start populations and the outputs; the working memory is the
library's fixed 64 MiB device array.

Checked through the C ABI against the ordinary entry point beep_simulate on
the same inputs, on two calls in a row (the second call must not see the
first call's leftovers): populations bit-exact, log-likelihood within the
1e-12 relative tolerance of the other parity tests.  Collected last so that a
failure here does not stop the rest of the GPU suite."""
import ctypes as C

import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import load

pytestmark = pytest.mark.gpu
L_RTOL = 1e-12


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from beep_gb300 import build
    build.build()
    return torch, capi.lib()


def device_tables(torch, tabs: capi.Tables):
    """A beep_param_tables whose pointers are device pointers (torch tensors)."""
    keep = {}
    st = capi.ParamTables()
    for k in capi.TABLE_F64_ARRAYS:
        t = torch.from_numpy(tabs.arr[k].copy()).to("cuda")
        keep[k] = t
        setattr(st, k, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)))
    for k in capi.TABLE_INT_ARRAYS:
        t = torch.from_numpy(tabs.arr[k].copy()).to("cuda")
        keep[k] = t
        setattr(st, k, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_int32)))
    st.nbeta_row, st.nefoi, st.nobs_spline = tabs.st.nbeta_row, tabs.st.nefoi, tabs.st.nobs_spline
    return st, keep


def run_noalloc(torch, L, dm, m, st, P, seed, ti, tf, pop_in=None):
    popsz = m.narea * m.ncomp * m.ndemocatpos
    Ld = torch.zeros(P, dtype=torch.float64, device="cuda")
    pd = torch.zeros(P * popsz, dtype=torch.int32, device="cuda")
    pin = None if pop_in is None else torch.from_numpy(np.ascontiguousarray(pop_in, np.int32).reshape(-1)).to("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.beep_simulate_plain_noalloc(dm.h, C.byref(st), P, seed, ti, tf,
                                       C.c_void_p(pin.data_ptr() if pin is not None else 0),
                                       C.c_void_p(Ld.data_ptr()), C.c_void_p(pd.data_ptr()), C.c_void_p(stream))
    capi.check(rc)
    return Ld.cpu().numpy(), pd.cpu().numpy().reshape(P, m.narea, m.ncomp, m.ndemocatpos)


def test_noalloc_matches_simulate_on_two_calls(setup):
    torch, L = setup
    b, m, tabs, seed = load("c0_sim")
    dm = capi.DeviceModel(m)
    st, keep = device_tables(torch, tabs[0])
    S = m.ndivision
    # call 1: the full horizon
    P1 = 16
    ref1 = dm.simulate(capi.Batch(m, tabs, P1, seed, want_pop=True))
    L1, pop1 = run_noalloc(torch, L, dm, m, st, P1, seed, 0, S)
    assert np.array_equal(pop1, ref1.pop)
    np.testing.assert_allclose(L1, ref1.L, rtol=L_RTOL, atol=0)
    # call 2: a later section from carried populations, more particles, another seed
    P2 = 24
    half = S // 2
    start = dm.simulate(capi.Batch(m, tabs, P2, seed + 1, ti=0, tf=half, want_pop=True))
    ref2 = dm.simulate(capi.Batch(m, tabs, P2, seed + 1, ti=half, tf=S, pop_in=start.pop, want_pop=True))
    L2, pop2 = run_noalloc(torch, L, dm, m, st, P2, seed + 1, half, S, pop_in=start.pop)
    assert np.array_equal(pop2, ref2.pop)
    np.testing.assert_allclose(L2, ref2.L, rtol=L_RTOL, atol=0)
    dm.close()


def test_noalloc_rejects_batches_beyond_its_memory(setup):
    torch, L = setup
    b, m, tabs, seed = load("c0_sim")
    dm = capi.DeviceModel(m)
    st, keep = device_tables(torch, tabs[0])
    rc = L.beep_simulate_plain_noalloc(dm.h, C.byref(st), 200000, seed, 0, m.ndivision, None, None, None, None)
    assert rc == 1
    assert b"working memory" in L.beep_last_error()
    dm.close()
