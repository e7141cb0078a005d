"""qsg_norm_noalloc, the Norm that allocates nothing, for callers that
cannot allocate device or pinned host memory once they run (an application
that has reserved nearly all device memory for its own pool, a fixed memory
budget, an allocator that forbids allocation behind its back).

Each case calls it first on a fresh context and checks that the context's
on-demand scratch (device and pinned) is still empty afterwards; only then is
qsg_norm, the existing entry point, called on the same state as the
reference, and the allocation-free call is repeated (two calls in a row share
the library's fixed array).  The file name sorts last so that a run that
stops at the first failure has already run every other test; the cases need
nothing from other tests and pass alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from qsim_gb300 import _native as N

# Same kernels and partition as qsg_norm: the results agree to round-off of
# the final FP64 sum (they are normally identical).
REL_TOL_SAME = 1e-12
# Against an FP64 norm of the FP32 amplitudes.
REL_TOL_FP64 = 1e-6


def scratch_bytes(ctx):
    dev, pinned = C.c_size_t(), C.c_size_t()
    N.check(N.lib.qsg_ctx_scratch_bytes(ctx.h, C.byref(dev), C.byref(pinned)))
    return dev.value, pinned.value


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
    assert scratch_bytes(ctx) == (0, 0)
    first = C.c_double(-1.0)
    N.check(N.lib.qsg_norm_noalloc(ctx.h, st.get(), n, C.byref(first)))
    # Nothing was allocated on the context by the allocation-free call.
    assert scratch_bytes(ctx) == (0, 0)
    ref = C.c_double()
    N.check(N.lib.qsg_norm(ctx.h, st.get(), n, C.byref(ref)))
    assert scratch_bytes(ctx) != (0, 0)   # the ordinary Norm did allocate
    second = C.c_double(-1.0)
    N.check(N.lib.qsg_norm_noalloc(ctx.h, st.get(), n, C.byref(second)))
    for out in (first, second):
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
    assert scratch_bytes(ctx) == (0, 0)
