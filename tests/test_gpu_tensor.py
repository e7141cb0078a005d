"""Tensor-core (tcgen05, split FP16 with a state scale) gate path against the FP64 oracle.

Tolerance: relative L2 <= 1e-5 per gate and per circuit, the same bar as the
CUDA-core path (split FP16 with FP32 accumulation keeps ~2^-22 relative error
per product); fidelity >= 1 - 1e-6 against FP64."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import qsim_gb300 as q
    from qsim_gb300 import engine as E
    from qsim_gb300 import _native as N
    ctx = q.Context(0)
    return q, E, N, ctx, q.StateSpace(ctx=ctx), q.Simulator(ctx=ctx)


def random_state(rng, n):
    a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return (a / np.linalg.norm(a)).astype(np.complex64).astype(np.complex128)


def random_unitary(rng, k):
    d = 1 << k
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return (q * (np.diag(r) / np.abs(np.diag(r)))).astype(np.complex64).astype(np.complex128)


def apply_tc(N, ctx, st, n, qs, m):
    m32 = np.ascontiguousarray(m.astype(np.complex64)).view(np.float32)
    N.check(N.lib.qsg_apply_gate_tc(ctx.h, st.get(), n, N.u32_array(qs), len(qs),
                                    m32.ctypes.data_as(N.P_f32)))


def tc_error(N, ctx):
    import ctypes as C
    e = C.c_int()
    N.check(N.lib.qsg_tc_error(ctx.h, C.byref(e)))
    return e.value


@pytest.mark.parametrize("n", [12, 13, 16])
def test_tc_six_qubit_gates(eng, oracle, n):
    q, E, N, ctx, ss, sim = eng
    rng = np.random.default_rng(40 + n)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    cases = [list(range(6)), list(range(n - 6, n)), [0, 2, 4, 6, 8, 10],
             [1, 3, 5, 7, 9, 11], sorted(rng.choice(n, 6, replace=False).tolist()),
             sorted(rng.choice(n, 6, replace=False).tolist())]
    for qs in cases:
        m = random_unitary(rng, 6)
        ref = s0.copy()
        oracle.apply_gate(ref, n, qs, m)
        ss.from_numpy(s0, st)
        apply_tc(N, ctx, st, n, qs, m)
        assert rel_l2(ss.to_numpy(st), ref) < 1e-5, qs
    assert tc_error(N, ctx) == 0


def test_tc_padded_gates(eng, oracle):
    q, E, N, ctx, ss, sim = eng
    rng = np.random.default_rng(3)
    n = 14
    s0 = random_state(rng, n)
    st = ss.Create(n)
    for k in range(0, 6):
        for _ in range(3):
            qs = sorted(rng.choice(n, k, replace=False).tolist())
            m = random_unitary(rng, k)
            ref = s0.copy()
            oracle.apply_gate(ref, n, qs, m)
            ss.from_numpy(s0, st)
            apply_tc(N, ctx, st, n, qs, m)
            assert rel_l2(ss.to_numpy(st), ref) < 1e-5, qs
    assert tc_error(N, ctx) == 0


def test_tc_non_unitary_matrix(eng, oracle):
    """M[i] = i + 1 (tests/simulator_testfixture.h:1146-1212 pattern) on a
    uniform state: large entries exercise the split-FP16 accuracy."""
    q, E, N, ctx, ss, sim = eng
    n = 12
    st = ss.Create(n)
    m = (np.arange(64 * 64) + 1).astype(np.complex128).reshape(64, 64) / 4096.0
    for qs in ([0, 1, 2, 3, 4, 5], [6, 7, 8, 9, 10, 11], [0, 3, 5, 7, 9, 11]):
        ss.SetStateUniform(st)
        apply_tc(N, ctx, st, n, qs, m)
        ref = np.full(1 << n, 1 / np.sqrt(1 << n), dtype=np.complex128)
        oracle.apply_gate(ref, n, qs, m)
        assert rel_l2(ss.to_numpy(st), ref) < 1e-5


@pytest.mark.parametrize("f", [4, 5, 6])
def test_tc_plan_matches_oracle(eng, oracle, f):
    """Fused plans with every block of >= 4 qubits on the tensor cores."""
    q, E, N, ctx, ss, sim = eng
    for c in (E.Circuit.grid(3, 5, 0, 14, 8), E.Circuit.grid(4, 4, 0, 12, 9)):
        n = c.num_qubits
        plan = E.Plan(c, max_fused_size=f, tensor_path=True, tc_min_k=4)
        assert plan.info()["num_tensor_ops"] > 0
        want = oracle.zero_state(n)
        for o in c.ops():
            oracle.apply_gate(want, n, o["qs"], o["m"])
        st = ss.Create(n)
        ss.SetStateZero(st)
        plan.run(ctx, st)
        got = ss.to_numpy(st)
        assert rel_l2(got, want) < 1e-5
        fid = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
        assert fid > 1 - 1e-6
        # Captured replay gives the same state.
        plan.capture(ctx, st)
        ss.SetStateZero(st)
        plan.replay(ctx)
        ctx.sync()
        assert rel_l2(ss.to_numpy(st), want) < 1e-5
    assert tc_error(N, ctx) == 0


def test_tc_deep_plan_keeps_norm_and_accuracy(eng, oracle):
    """A plan with ~70 tensor-core passes stays within relative L2 1e-5 of
    FP64: the tensor cores' FP32 accumulation rounds toward zero (about
    6e-7 of norm lost per pass), which the plan corrects by restoring the
    input norm after its last launch (unitary plans)."""
    q, E, N, ctx, ss, sim = eng
    c = E.Circuit.grid(4, 5, 0, 40, 21)
    n = c.num_qubits
    plan = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=2)
    assert plan.info()["num_tensor_ops"] >= 40
    want = oracle.zero_state(n)
    for o in c.ops():
        oracle.apply_gate(want, n, o["qs"], o["m"])
    st = ss.Create(n)
    ss.SetStateZero(st)
    plan.run(ctx, st)
    got = ss.to_numpy(st)
    assert abs(np.linalg.norm(got) - 1) < 1e-6
    assert rel_l2(got, want) < 1e-5
    plan.capture(ctx, st)
    ss.SetStateZero(st)
    plan.replay(ctx)
    ctx.sync()
    assert rel_l2(ss.to_numpy(st), want) < 1e-5


@pytest.mark.parametrize("n", [12, 16])
def test_tc_bounded_wait_runs_out_and_context_recovers(eng, oracle, n):
    """Failure detection without a GPU fault: the kernel's MMA thread waits
    on a barrier that nothing arrives at, with a ~1 ms clock budget; the
    wait runs out before any MMA is issued, every role leaves through the
    error exit and the host reads QSG_ERR_TIMEOUT.  The state is unchanged,
    the flag is cleared, and the next tensor-core gate on the same context
    matches the oracle."""
    import ctypes as C
    q, E, N, ctx, ss, sim = eng
    rng = np.random.default_rng(7 + n)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    ss.from_numpy(s0, st)
    rc = N.lib.qsg_tc_stall_test(ctx.h, st.get(), n, C.c_longlong(2_000_000))
    assert rc == 6, N.lib.qsg_last_error()          # QSG_ERR_TIMEOUT
    assert b"bounded wait" in N.lib.qsg_last_error()
    assert np.array_equal(ss.to_numpy(st), s0.astype(np.complex64))
    assert tc_error(N, ctx) == 0
    m = random_unitary(rng, 6)
    qs = sorted(rng.choice(n, 6, replace=False).tolist())
    apply_tc(N, ctx, st, n, qs, m)
    ref = s0.copy()
    oracle.apply_gate(ref, n, qs, m)
    assert tc_error(N, ctx) == 0
    assert rel_l2(ss.to_numpy(st), ref) <= 1e-5
    # Out-of-range budgets are argument errors, not launches.
    assert N.lib.qsg_tc_stall_test(ctx.h, st.get(), n, C.c_longlong(10)) == 1


def apply_tc2(N, ctx, st, n, qa, ma, qb, mb):
    a32 = np.ascontiguousarray(ma.astype(np.complex64)).view(np.float32)
    b32 = np.ascontiguousarray(mb.astype(np.complex64)).view(np.float32)
    return N.lib.qsg_apply_gate_tc2(ctx.h, st.get(), n, N.u32_array(qa), len(qa),
                                    a32.ctypes.data_as(N.P_f32), N.u32_array(qb),
                                    len(qb), b32.ctypes.data_as(N.P_f32))


def tc2_cases(rng, n):
    """Pairs of target sets: disjoint, interleaved, equal, partly shared,
    high qubits, padded (k < 6) and random subsets of 12 qubits that
    include qubit 0."""
    cases = [([0, 1, 2, 3, 4, 5], [6, 7, 8, 9, 10, 11]),
             ([0, 2, 4, 6, 8, 10], [1, 3, 5, 7, 9, 11]),
             ([3, 4, 5, 6, 7, 8], [3, 4, 5, 6, 7, 8]),       # one product pass
             ([1, 2, 3, 4, 5, 7], [1, 2, 3, 4, 6, 7]),       # five shared qubits
             ([2, 5, 7, n - 3, n - 2, n - 1], [0, 5, 7, 9, n - 2, n - 1]),
             ([0, 1, 2, 3, 4, 5], [3, 4, 5, 6, 7, 8]),
             (list(range(n - 6, n)), [0, 1, 2] + list(range(n - 3, n))),
             ([0, n - 1], [1, 5, n - 2]),
             ([2, n - 4, n - 3, n - 2, n - 1], [0, 1, n - 6, n - 5, n - 4])]
    for _ in range(4):
        pool = [0] + rng.choice(np.arange(1, n), 11, replace=False).tolist()
        a = sorted(rng.choice(pool, 6, replace=False).tolist())
        b = sorted(rng.choice(pool, 6, replace=False).tolist())
        cases.append((a, b))
    return cases


@pytest.mark.parametrize("n", [12, 13, 16, 22])
def test_tc2_pairs_match_oracle(eng, oracle, n):
    """Two gates in one tensor-core pass equal the two gates applied one
    after the other in FP64 (relative L2 <= 1e-5, the one-gate bar), for
    tiles of 1 tile per CTA (n <= 16) up to many (n = 22: 1024 tiles)."""
    q, E, N, ctx, ss, sim = eng
    rng = np.random.default_rng(90 + n)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    for qa, qb in tc2_cases(rng, n):
        ma = random_unitary(rng, len(qa))
        mb = random_unitary(rng, len(qb))
        ref = s0.copy()
        oracle.apply_gate(ref, n, qa, ma)
        oracle.apply_gate(ref, n, qb, mb)
        ss.from_numpy(s0, st)
        N.check(apply_tc2(N, ctx, st, n, qa, ma, qb, mb))
        assert rel_l2(ss.to_numpy(st), ref) < 1e-5, (qa, qb)
    assert tc_error(N, ctx) == 0


def test_tc2_rejects_pairs_that_do_not_fit(eng):
    """Two 6-qubit gates on 12 distinct qubits none of which is qubit 0
    leave no tile that starts at qubit 0: refused before any launch (the
    state is left as it was)."""
    q, E, N, ctx, ss, sim = eng
    n = 16
    rng = np.random.default_rng(2)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    ss.from_numpy(s0, st)
    m = random_unitary(rng, 6)
    rc = apply_tc2(N, ctx, st, n, [1, 2, 3, 4, 5, 6], m,
                   [7, 8, 9, 10, 11, 12], m)
    assert rc == 4, N.lib.qsg_last_error()         # QSG_ERR_UNSUPPORTED
    assert b"qubit 0" in N.lib.qsg_last_error()
    assert np.array_equal(ss.to_numpy(st), s0.astype(np.complex64))
    assert tc_error(N, ctx) == 0


def test_tc_plan_with_a_non_unitary_gate(eng, oracle):
    """A tensor-core plan whose circuit holds one non-unitary gate runs
    without the norm carry (a block is unitary only when all its member
    gates are, known from fusion): the oracle's state, norm included;
    the same circuit without that gate keeps the carry and its norm."""
    q, E, N, ctx, ss, sim = eng
    rng = np.random.default_rng(31)
    n = 14

    def circuit(with_bad):
        c = E.Circuit(n)
        t = 0
        for layer in range(10):
            for a in range(layer % 2, n - 1, 2):
                z = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
                u, _ = np.linalg.qr(z)
                c.add_gate(t, [a, a + 1], u)
            t += 1
            if with_bad and layer == 4:
                c.add_gate(t, [3, 4], np.diag([1.0, 0.6, 0.9, 1.3]).astype(complex))
                t += 1
        return c

    for with_bad in (True, False):
        c = circuit(with_bad)
        plan = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=1,
                      tc_pairs=2)
        want = oracle.zero_state(n)
        for o in c.ops():
            oracle.apply_gate(want, n, o["qs"], o["m"])
        st = ss.Create(n)
        ss.SetStateZero(st)
        plan.run(ctx, st)
        got = ss.to_numpy(st)
        assert rel_l2(got, want) < 1e-5, with_bad
        if not with_bad:
            assert abs(np.linalg.norm(got) - 1) < 1e-6
    assert tc_error(N, ctx) == 0


@pytest.mark.parametrize("bits", [1, 3])
def test_tc2_plans_match_oracle(eng, oracle, bits):
    """Plans whose consecutive tensor-core blocks share two-gate passes
    (every block on the tensor cores, pairs with >= `bits` run bits):
    run, captured replay and per-op profile give the oracle's state, with
    the norm carry across single and paired passes."""
    q, E, N, ctx, ss, sim = eng
    for c in (E.Circuit.grid(4, 4, 0, 16, 5), E.Circuit.grid(3, 6, 0, 14, 6)):
        n = c.num_qubits
        plan = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=1,
                      tc_pairs=bits)
        info = plan.info()
        assert info["num_tc_pairs"] > 0
        pn = plan.tc_pair_next()
        assert pn.sum() == info["num_tc_pairs"]
        assert not np.any(pn[:-1] & pn[1:])            # pairs do not overlap
        want = oracle.zero_state(n)
        for o in c.ops():
            oracle.apply_gate(want, n, o["qs"], o["m"])
        st = ss.Create(n)
        ss.SetStateZero(st)
        plan.run(ctx, st)
        got = ss.to_numpy(st)
        assert rel_l2(got, want) < 1e-5
        assert abs(np.linalg.norm(got) - 1) < 1e-6
        plan.capture(ctx, st)
        ss.SetStateZero(st)
        plan.replay(ctx)
        ctx.sync()
        assert rel_l2(ss.to_numpy(st), want) < 1e-5
        ss.SetStateZero(st)
        ms = np.asarray(plan.profile(ctx, st))
        # Profiled runs launch op by op without the norm carry.
        assert rel_l2(ss.to_numpy(st), want) < 5e-5
        # A pair is timed as its first op; its second op's interval spans
        # no launch (two events recorded back to back).
        assert np.all(ms[1:][pn[:-1] == 1] < 0.02)
    assert tc_error(N, ctx) == 0


@pytest.mark.parametrize("n", [12, 16, 20])
def test_tc_expectation_values_match_oracle(eng, oracle, n):
    """ExpectationValue on the tensor cores (the gate pass with a read-only
    epilogue that forms conj(psi_i) (M psi)_i from the tile's FP16 hi + lo
    images): Hermitian and general operators of 1..6 qubits at every
    layout class, within 1e-5 of the FP64 oracle on a normalised state."""
    import ctypes as C
    q, E, N, ctx, ss, sim = eng
    rng = np.random.default_rng(60 + n)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    ss.from_numpy(s0, st)
    out = (C.c_double * 2)()
    cases = [[0], [n - 1], [0, 1], [3, n - 2], [0, 2, 4], [1, 5, 9, n - 1],
             list(range(5)), list(range(n - 5, n)), [0, 1, 2, 3, 4, 5],
             sorted(rng.choice(n, 6, replace=False).tolist())]
    for qs in cases:
        k = len(qs)
        z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        for m in ((z + z.conj().T) / 2, z / np.sqrt(1 << k)):
            m32 = np.ascontiguousarray(m.astype(np.complex64))
            N.check(N.lib.qsg_expectation_value_tc(
                ctx.h, st.get(), n, N.u32_array(qs), k,
                m32.view(np.float32).ctypes.data_as(N.P_f32), out))
            want = oracle.expectation_value(s0, n, qs, m32.astype(np.complex128))
            got = complex(out[0], out[1])
            assert abs(got - want) <= 1e-5 * max(1.0, abs(want)), (qs, got, want)
    # The state is untouched.
    assert np.array_equal(ss.to_numpy(st), s0.astype(np.complex64))
    assert tc_error(N, ctx) == 0


def test_expectation_value_dispatch_and_overflow_fallback(eng, oracle):
    """qsg_expectation_value puts dense operators of >= 4 qubits on the
    tensor cores; a state whose amplitudes exceed the split's range (here
    multiplied by 1e5) falls back to the CUDA cores with the same answer,
    and the forced tensor-core entry reports QSG_ERR_UNSUPPORTED."""
    import ctypes as C
    q, E, N, ctx, ss, sim = eng
    n = 14
    rng = np.random.default_rng(11)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    out = (C.c_double * 2)()
    qs = [1, 4, 6, 11, 13]
    z = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
    m32 = np.ascontiguousarray(((z + z.conj().T) / 2).astype(np.complex64))
    mp = m32.view(np.float32).ctypes.data_as(N.P_f32)
    for scale in (1.0, 1e5):
        s = (s0 * scale).astype(np.complex64).astype(np.complex128)
        ss.from_numpy(s, st)
        N.check(N.lib.qsg_expectation_value(ctx.h, st.get(), n, N.u32_array(qs),
                                            5, mp, out))
        want = oracle.expectation_value(s, n, qs, m32.astype(np.complex128))
        assert abs(complex(out[0], out[1]) - want) <= 1e-5 * abs(want) + 1e-6
        rc = N.lib.qsg_expectation_value_tc(ctx.h, st.get(), n, N.u32_array(qs),
                                            5, mp, out)
        assert rc == (0 if scale == 1.0 else 4), N.lib.qsg_last_error()
    assert tc_error(N, ctx) == 0
