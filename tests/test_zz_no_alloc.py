"""qsg_norm_noalloc, the allocation-free Norm: called through the C ABI and
compared with qsg_norm (the existing entry point) and with an FP64 numpy
norm, on two calls in a row.  The file name sorts last so that it also runs
after every other test; it needs nothing from them and passes alone."""
import ctypes as C

import numpy as np
import pytest

from qsim_gb300 import _native as N

# Same kernels and partition as qsg_norm: the results agree to round-off of
# the final FP64 sum (they are normally identical).
REL_TOL_SAME = 1e-12
# Against an FP64 norm of the FP32 amplitudes.
REL_TOL_FP64 = 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 5, 13, 22])
def test_norm_noalloc_matches_norm(n):
    import qsim_gb300 as q
    ctx = q.Context(0)
    ss = q.StateSpace(ctx=ctx)
    st = ss.Create(n)
    rng = np.random.default_rng(n)
    amps = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)) * 0.37
    ss.from_numpy(amps, st)
    want64 = float(np.sum(np.abs(amps.astype(np.complex64).astype(np.complex128)) ** 2))
    ref = C.c_double()
    N.check(N.lib.qsg_norm(ctx.h, st.get(), n, C.byref(ref)))
    for _ in range(2):
        out = C.c_double(-1.0)
        N.check(N.lib.qsg_norm_noalloc(ctx.h, st.get(), n, C.byref(out)))
        assert abs(out.value - ref.value) <= REL_TOL_SAME * ref.value
        assert abs(out.value - want64) <= REL_TOL_FP64 * want64


@pytest.mark.gpu
def test_norm_noalloc_rejects_bad_arguments():
    import qsim_gb300 as q
    ctx = q.Context(0)
    st = q.StateSpace(ctx=ctx).Create(3)
    out = C.c_double()
    assert N.lib.qsg_norm_noalloc(ctx.h, st.get(), 41, C.byref(out)) == 1
    assert b"qubits" in N.lib.qsg_last_error()
    assert N.lib.qsg_norm_noalloc(ctx.h, None, 3, C.byref(out)) == 1
