"""A bounded device-side wait that runs out.

The tensor-core brute force waits on mbarriers for its bulk copies and
matrix products, each wait bounded by a poll budget.  Here the budget is cut
to one poll (tk_set_device_wait_limit, host-side fault injection), so the
waits run out: the kernel must flag it, let its own copies and products
land, free its tensor memory and return; the call must come back, the
report must say TK_ETIMEOUT with every query recomputed by the exact
kernel, and the answer must still equal the oracle's.  The reference exits
the process on any device error (src/cutils.cuh:34-43)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def run(ref, q, k, mode):
    from torch_kdtree_gb300 import _lib
    from torch_kdtree_gb300._lib import LIB, check
    from torch_kdtree_gb300.nn_distance import _BRUTE_MODES, _stream_ptr
    n, d = ref.shape
    nq = q.shape[0]
    m = _BRUTE_MODES[mode]
    ws_bytes = LIB.tk_nn_distance_workspace_size(n, nq, d, k, _lib.TK_F32, m)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=ref.device)
    dd = torch.empty(nq, k, device=ref.device)
    ii = torch.empty(nq, k, dtype=torch.int32, device=ref.device)
    check(LIB.tk_nn_distance(ref.data_ptr(), n, q.data_ptr(), nq, d, k, _lib.TK_F32, m, dd.data_ptr(),
                             ii.data_ptr(), ws.data_ptr(), ws_bytes, _stream_ptr(ref.device)))
    torch.cuda.synchronize()
    flags, recomputed = ctypes.c_int(-1), ctypes.c_int(-1)
    rc = LIB.tk_nn_distance_report(ws.data_ptr(), n, nq, d, k, _lib.TK_F32, m, ctypes.byref(flags),
                                   ctypes.byref(recomputed))
    return dd, ii, rc, flags.value, recomputed.value


@pytest.mark.parametrize("mode", ["tf32", "bf16_split"])
def test_wait_that_runs_out_is_reported_and_the_answer_stays_exact(mode, oracle):
    from torch_kdtree_gb300._lib import LIB, TK_ETIMEOUT, TK_OK
    rng = np.random.default_rng(21)
    ref_np = rng.standard_normal((20000, 16)).astype(np.float32)
    q_np = rng.standard_normal((2000, 16)).astype(np.float32)
    k = 8
    bd, bi = oracle.brute(ref_np, q_np, k)
    ref = torch.from_numpy(ref_np).cuda()
    q = torch.from_numpy(q_np).cuda()
    prev = LIB.tk_set_device_wait_limit(1)
    try:
        dd, ii, rc, flags, recomputed = run(ref, q, k, mode)
    finally:
        LIB.tk_set_device_wait_limit(prev)
    assert rc == TK_ETIMEOUT and flags & 1, (rc, flags)
    assert b"wait ran out" in LIB.tk_last_error()
    assert recomputed == len(q_np)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)
    # the context is still usable, and the default budget gives a clean run
    dd, ii, rc, flags, recomputed = run(ref, q, k, mode)
    assert rc == TK_OK and flags == 0 and recomputed < len(q_np), (rc, flags, recomputed)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


def test_exact_mode_reports_nothing():
    from torch_kdtree_gb300 import _lib
    from torch_kdtree_gb300._lib import LIB, TK_OK
    flags, recomputed = ctypes.c_int(-1), ctypes.c_int(-1)
    assert LIB.tk_nn_distance_report(None, 10, 10, 3, 1, _lib.TK_F32, _lib.TK_BRUTE_EXACT, ctypes.byref(flags),
                                     ctypes.byref(recomputed)) == TK_OK
    assert flags.value == 0 and recomputed.value == 0
