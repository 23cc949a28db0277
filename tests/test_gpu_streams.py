"""Copy streams: transfers on streams 1 and 2 ordered against launches on
stream 0 with events, as the overlapped end-to-end pipeline uses them."""
import ctypes

import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu


def test_copy_streams_ordered_by_events(scl, orc):
    n = 1 << 22
    L = S.lib()
    x = orc.mod_i32(n, 1, 1001)
    hin, hout = ctypes.c_void_p(), ctypes.c_void_p()
    S.check(L.scl_host_alloc(4 * n, ctypes.byref(hin)))
    S.check(L.scl_host_alloc(4 * n, ctypes.byref(hout)))
    try:
        ctypes.memmove(hin, x.ctypes.data, 4 * n)
        d = S.DeviceArray(n, np.int32)
        p = S.Program(S.KIND_MAP, "int func(int x){ return 3 * x + 1; }", ["int", "int"])
        e_in, e_done = S.Event(), S.Event()
        for rep in range(3):
            S.check(L.scl_h2d_on(1, d.ptr, hin, 4 * n))
            e_in.record_on(1)
            e_in.wait_on(0)
            p.launch([d, d], n=n)
            e_done.record_on(0)
            e_done.wait_on(2)
            S.check(L.scl_d2h_on(2, hout, d.ptr, 4 * n))
            S.sync()
            got = np.ctypeslib.as_array(ctypes.cast(hout, ctypes.POINTER(ctypes.c_int32)), shape=(n,)).copy()
            assert np.array_equal(got, 3 * x + 1), rep
    finally:
        L.scl_host_free(hin)
        L.scl_host_free(hout)


def test_bad_stream_index_is_an_argument_error(scl):
    buf = np.zeros(4, np.int32)
    d = S.DeviceArray(4, np.int32)
    assert S.lib().scl_h2d_on(3, d.ptr, buf.ctypes.data, 16) == S.ERR_ARG
