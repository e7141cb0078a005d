"""GPU parity of the state-vector path against the oracle and the reference's
golden outputs.  Every call goes through the C ABI (libqsim_gb300.so).

Tolerances: FP32 state vs FP64 reference, relative L2 <= 1e-5 (the bar the
reference's own FP32 path meets, see test_oracle_golden.py); FP64-accumulated
reductions within 1e-6 relative; index logic (samples, measured bits)
compared exactly, with the sample bar of >= 99.9% identical indices for
states that differ by FP32 rounding."""
import numpy as np
import pytest

from conftest import (GOLDEN_CASES, load_golden, pauli_matrix, rel_l2,
                      unpack_ops)

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def eng():
    import qsim_gb300 as q
    ctx = q.Context(0)
    return q, q.StateSpace(ctx=ctx), q.Simulator(ctx=ctx)


def random_state(rng, n):
    a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return a / np.linalg.norm(a)


def random_unitary(rng, k):
    d = 1 << k
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def c64_to_c128(a):
    return a.astype(np.complex64).astype(np.complex128)


def mat32(m):
    return np.ascontiguousarray(np.asarray(m, np.complex64)).view(np.float32)


def run_ops_gpu(ss, sim, n, ops):
    st = ss.Create(n)
    ss.SetStateZero(st)
    for o in ops:
        if o["kind"] == 0:
            sim.ApplyGate(o["qs"], mat32(o["m"]), st)
        elif o["kind"] == 1:
            sim.ApplyControlledGate(o["qs"], o["cqs"], o["cvals"], mat32(o["m"]), st)
    return st


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_final_state(eng, case):
    q, ss, sim = eng
    d = load_golden(case)
    n = int(d["n"])
    st = run_ops_gpu(ss, sim, n, unpack_ops(d))
    got = ss.to_numpy(st)
    assert rel_l2(got, d["f64"]) < TOL
    assert abs(ss.Norm(st) - 1.0) < 1e-5


@pytest.mark.parametrize("n", [1, 2, 3, 5, 6, 7, 9, 12, 15])
def test_apply_gate_every_layout(eng, oracle, n):
    """Random k-qubit unitaries (k = 0..min(6, n)) on many target sets:
    low/high targets, qubit 0 in or out (pair and non-pair layouts)."""
    q, ss, sim = eng
    rng = np.random.default_rng(100 + n)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    for k in range(0, min(6, n) + 1):
        trials = 6 if k > 0 else 1
        for _ in range(trials):
            qs = sorted(rng.choice(n, size=k, replace=False).tolist())
            m = random_unitary(rng, k)
            ref = c64_to_c128(s0)
            oracle.apply_gate(ref, n, qs, c64_to_c128(m))
            ss.from_numpy(s0, st)
            sim.ApplyGate(qs, mat32(m), st)
            got = ss.to_numpy(st)
            assert rel_l2(got, ref) < TOL, (n, qs)


def test_apply_gate_high_and_mixed_targets(eng, oracle):
    q, ss, sim = eng
    rng = np.random.default_rng(7)
    n = 18
    s0 = random_state(rng, n)
    st = ss.Create(n)
    cases = [[17], [0, 17], [16, 17], [1, 2, 3, 4], [0, 1, 2, 3],
             [4, 9, 13, 17], [5, 6, 7, 8, 9], [0, 3, 8, 12, 15, 17],
             [12, 13, 14, 15, 16, 17], [0, 1, 2, 3, 4, 5], [2, 6, 10]]
    for qs in cases:
        m = random_unitary(rng, len(qs))
        ref = c64_to_c128(s0)
        oracle.apply_gate(ref, n, qs, c64_to_c128(m))
        ss.from_numpy(s0, st)
        sim.ApplyGate(qs, mat32(m), st)
        assert rel_l2(ss.to_numpy(st), ref) < TOL, qs


@pytest.mark.parametrize("n", [4, 8, 13])
def test_controlled_gates(eng, oracle, n):
    """All control/target placements the reference's kernels distinguish:
    low and high controls, controls on qubit 0, targets low and high."""
    q, ss, sim = eng
    rng = np.random.default_rng(300 + n)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    for _ in range(40):
        k = int(rng.integers(0, min(4, n - 1) + 1))
        c = int(rng.integers(1, min(3, n - k) + 1))
        picks = rng.choice(n, size=k + c, replace=False).tolist()
        qs, cqs = sorted(picks[:k]), sorted(picks[k:])
        cvals = int(rng.integers(0, 1 << c))
        m = random_unitary(rng, k)
        ref = c64_to_c128(s0)
        oracle.apply_controlled_gate(ref, n, qs, cqs, cvals, c64_to_c128(m))
        ss.from_numpy(s0, st)
        sim.ApplyControlledGate(qs, cqs, cvals, mat32(m), st)
        assert rel_l2(ss.to_numpy(st), ref) < TOL, (qs, cqs, cvals)


def test_multi_qubit_gates_closed_form(eng, oracle):
    """Non-unitary M[i] = i + 1 (the reference's TestMultiQubitGates,
    tests/simulator_testfixture.h:1146-1212) on a uniform state, every
    contiguous target window, k = 1..6."""
    q, ss, sim = eng
    n = 8
    st = ss.Create(n)
    for k in range(1, 7):
        d = 1 << k
        m = (np.arange(d * d) + 1).astype(np.complex128).reshape(d, d)
        for q0 in range(0, n - k + 1):
            qs = list(range(q0, q0 + k))
            ss.SetStateUniform(st)
            sim.ApplyGate(qs, mat32(m), st)
            ref = np.full(1 << n, 1 / np.sqrt(1 << n), dtype=np.complex128)
            oracle.apply_gate(ref, n, qs, m)
            assert rel_l2(ss.to_numpy(st), ref) < TOL


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_expectation_values(eng, case):
    q, ss, sim = eng
    d = load_golden(case)
    if "ev64" not in d:
        pytest.skip("no expectation values")
    n = int(d["n"])
    st = ss.Create(n)
    ss.from_numpy(d["f64"], st)
    for i, ops in enumerate(d["ev_ops"]):
        qs = d["ev_qpool"][d["ev_qoff"][i]:d["ev_qoff"][i + 1]].tolist()
        ev = sim.ExpectationValue(qs, mat32(pauli_matrix(str(ops))), st)
        assert abs(ev - d["ev64"][i]) < 1e-5


def test_expectation_values_random(eng, oracle):
    q, ss, sim = eng
    rng = np.random.default_rng(11)
    for n in (3, 9, 14):
        s0 = random_state(rng, n)
        st = ss.Create(n)
        ss.from_numpy(s0, st)
        for k in range(1, min(6, n) + 1):
            for _ in range(3):
                qs = sorted(rng.choice(n, size=k, replace=False).tolist())
                m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
                ref = oracle.expectation_value(c64_to_c128(s0), n, qs, c64_to_c128(m))
                ev = sim.ExpectationValue(qs, mat32(m), st)
                assert abs(ev - ref) < 1e-5 * max(1.0, abs(ref)), (n, qs)


def test_hermitian_expectation_values(eng, oracle):
    """Hermitian operators of 1..3 qubits take the tile kernel's Hermitian
    mode (the diagonal and twice the real part of the upper triangle, half
    the products): against the FP64 oracle, with and without qubit 0 among
    the targets, and against the general mode on the same matrix made
    non-Hermitian by a 1e-30 imaginary part on one diagonal entry."""
    q, ss, sim = eng
    rng = np.random.default_rng(13)
    for n in (3, 9, 14, 20):
        s0 = random_state(rng, n)
        st = ss.Create(n)
        ss.from_numpy(s0, st)
        for k in (1, 2, 3):
            for with0 in (True, False):
                if k + (0 if with0 else 1) > n:
                    continue
                pool = list(range(n)) if with0 else list(range(1, n))
                qs = sorted(rng.choice(pool, size=k, replace=False).tolist())
                if with0 and 0 not in qs:
                    qs = sorted([0] + qs[1:])
                z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
                h = c64_to_c128((z + z.conj().T) / 2)
                ref = oracle.expectation_value(c64_to_c128(s0), n, qs, h)
                ev = sim.ExpectationValue(qs, mat32(h), st)
                assert abs(ev - ref) < 1e-5 * max(1.0, abs(ref)), (n, k, qs)
                assert ev.imag == 0.0
                g = h.copy()
                g[0, 0] += 1e-30j
                evg = sim.ExpectationValue(qs, mat32(g), st)
                assert abs(ev - evg) < 1e-5 * max(1.0, abs(ref)), (n, k, qs)


def test_monomial_expectation_values(eng, oracle):
    """Monomial operators (one nonzero per row at column r ^ xm: Pauli
    strings, diagonal gates, phased permutations) take the one-pass kernel;
    it agrees with the FP64 oracle and with the dense tile-kernel path on the
    same operator (made dense by a zero-valued perturbation that the monomial
    test rejects: one off-pattern entry of 1e-30)."""
    q, ss, sim = eng
    rng = np.random.default_rng(12)
    for n in (2, 7, 13, 16):
        s0 = random_state(rng, n)
        st = ss.Create(n)
        ss.from_numpy(s0, st)
        for k in range(1, min(6, n) + 1):
            dim = 1 << k
            for xm in sorted({0, 1, dim - 1, int(rng.integers(dim))}):
                qs = sorted(rng.choice(n, size=k, replace=False).tolist())
                m = np.zeros((dim, dim), np.complex128)
                ph = np.exp(1j * rng.uniform(0, 2 * np.pi, dim)) * rng.uniform(0.5, 1.5, dim)
                for r in range(dim):
                    m[r, r ^ xm] = ph[r]
                ref = oracle.expectation_value(c64_to_c128(s0), n, qs, c64_to_c128(m))
                ev = sim.ExpectationValue(qs, mat32(m), st)
                assert abs(ev - ref) < 1e-5 * max(1.0, abs(ref)), (n, k, xm, qs)
                md = m.copy()
                md[0, (0 ^ xm) ^ 1 if dim > 1 else 0] += 1e-30
                evd = sim.ExpectationValue(qs, mat32(md), st)
                assert abs(ev - evd) < 1e-5 * max(1.0, abs(ref)), (n, k, xm)


@pytest.mark.parametrize("n", [13, 20])
def test_monomial_kernel_forms(eng, oracle, n):
    """Monomial operators over whole tiles of work take the kernel that
    derives a thread's units, signs and table rows from one base unit:
    without a partner unit (Z only, or X on qubit 0), with a near partner
    (flipped qubits 1..10) and with a far one (a flipped qubit >= 11,
    paired on the highest; also with flips of qubits 9 and 10, whose unit
    bits 8, 9 are the thread's own unit offsets).  Each Pauli string (sign
    form) and a monomial with random entries on the same pattern (table
    form) against the FP64 oracle, and against the same operator with a
    1e-30 off-pattern entry (the dense path)."""
    q, ss, sim = eng
    rng = np.random.default_rng(21 + n)
    s0 = random_state(rng, n)
    st = ss.Create(n)
    ss.from_numpy(s0, st)
    cases = [([2, 5], "ZZ"), ([0, 7], "XZ"), ([0, 3, 6], "YIZ"),
             ([3], "X"), ([0, 5, 8], "XYZ"), ([1, 10], "YX"),
             ([9, 10, 12], "XYZ"), ([0, 2, 9, 12], "YZXX"),
             ([4, 11], "ZY"), ([0, 1, 6, 9, 10, 12], "XYZXYZ")]
    for qs, word in cases:
        pm = pauli_matrix(word)
        dim = len(pm)
        xm = int(np.flatnonzero(pm[0])[0])
        tm = np.zeros_like(pm)
        for r in range(dim):
            tm[r, r ^ xm] = complex(rng.normal(), rng.normal())
        for m in (pm, tm):
            ref = oracle.expectation_value(c64_to_c128(s0), n, qs, c64_to_c128(m))
            ev = sim.ExpectationValue(qs, mat32(m), st)
            assert abs(ev - ref) < 1e-5 * max(1.0, abs(ref)), (n, qs, word)
            md = m.copy()
            md[0, 1 if md[0, 1] == 0 else 0] += 1e-30
            evd = sim.ExpectationValue(qs, mat32(md), st)
            assert abs(ev - evd) < 1e-5 * max(1.0, abs(ref)), (n, qs, word)


def test_norm_inner_product_add_multiply(eng):
    q, ss, sim = eng
    rng = np.random.default_rng(5)
    for n in (0, 1, 4, 10, 17):
        a = c64_to_c128(random_state(rng, n) * 1.7)
        b = c64_to_c128(random_state(rng, n))
        sa, sb = ss.Create(n), ss.Create(n)
        ss.from_numpy(a, sa)
        ss.from_numpy(b, sb)
        assert abs(ss.Norm(sa) - np.vdot(a, a).real) < 1e-6
        ip = ss.InnerProduct(sa, sb)
        assert abs(ip - np.vdot(a, b)) < 1e-6
        assert abs(ss.RealInnerProduct(sa, sb) - np.vdot(a, b).real) < 1e-6
        assert ss.Add(sa, sb)
        assert rel_l2(ss.to_numpy(sb), a + b) < TOL
        ss.Multiply(0.5, sb)
        assert rel_l2(ss.to_numpy(sb), 0.5 * (a + b)) < TOL
    s1, s2 = ss.Create(3), ss.Create(4)
    assert np.isnan(ss.InnerProduct(s1, s2).real)
    assert not ss.Add(s1, s2)


def test_set_state_and_amplitudes(eng):
    q, ss, sim = eng
    for n in (0, 3, 11):
        st = ss.Create(n)
        ss.SetStateZero(st)
        v = ss.to_numpy(st)
        assert v[0] == 1 and np.count_nonzero(v) == 1
        ss.SetStateUniform(st)
        assert np.allclose(ss.to_numpy(st), 1 / np.sqrt(1 << n))
        ss.SetAllZeros(st)
        assert np.count_nonzero(ss.to_numpy(st)) == 0
        ss.SetAmpl(st, (1 << n) - 1, 0.25, -0.5)
        assert ss.GetAmpl(st, (1 << n) - 1) == complex(0.25, -0.5)
    n = 6
    st = ss.Create(n)
    ss.SetStateZero(st)
    ss.BulkSetAmpl(st, 0b101, 0b001, complex(2, 3))
    v = ss.to_numpy(st)
    idx = np.arange(1 << n)
    sel = (idx & 0b101) == 0b001
    assert np.all(v[sel] == complex(2, 3))
    assert v[0] == 1 and np.count_nonzero(v[~sel]) == 1
    ss.BulkSetAmpl(st, 0b101, 0b001, 0.0, 1.0, exclude=True)
    v = ss.to_numpy(st)
    assert np.all(v[~sel] == 1j) and np.all(v[sel] == complex(2, 3))


@pytest.mark.parametrize("case", ["rand12_k6", "rand14_k2", "ctrl11", "small6"])
def test_samples_match_reference(eng, case):
    """Sample(state, m, seed): identical uniforms to the reference
    (mt19937(seed), uniform_real_distribution, sorted), CDF search on the
    device.  On the reference's own state cast to FP32, >= 99.9% of indices
    are identical to the reference's FP64 samples."""
    q, ss, sim = eng
    d = load_golden(case)
    n = int(d["n"])
    st = ss.Create(n)
    ss.from_numpy(d["f64"], st)
    got = np.array(ss.Sample(st, d["s64"].size, int(d["sample_seed"])), np.uint64)
    assert np.mean(got == d["s64"]) >= 0.999


def test_samples_exact_against_oracle_on_same_state(eng, oracle):
    q, ss, sim = eng
    rng = np.random.default_rng(9)
    for n in (1, 5, 13, 16):
        s = c64_to_c128(random_state(rng, n))
        st = ss.Create(n)
        ss.from_numpy(s, st)
        want = oracle.sample(s.copy(), n, 3000, 77)
        got = np.array(ss.Sample(st, 3000, 77), np.uint64)
        assert np.mean(got == want) >= 0.999
        assert np.all(np.diff(got.astype(np.int64)) >= 0)


def test_samples_and_measure_with_two_level_prefix(eng, oracle):
    """States of >= 26 qubits (more than 4096 chunks) take the two-level
    chunk prefix.  27 qubits: each of 2000 samples and 3 measurements must
    be the index whose CDF interval holds its threshold r = u * norm (u the
    same sorted mt19937 uniforms).  At 2^27 terms the sequential FP64 CDF of
    the host (the oracle's scan, np.cumsum) drifts by up to about one
    amplitude's probability (7e-9 here), so the check allows 2e-8 of slack
    at both ends of the interval; a wrong prefix would be off by a chunk's
    probability (6e-5)."""
    import ctypes as C
    from qsim_gb300 import _native as N
    q, ss, sim = eng
    n = 27
    rng = np.random.default_rng(27)
    st = ss.Create(n)
    ss.SetStateUniform(st)
    for _ in range(6):
        k = int(rng.integers(1, 4))
        qs = sorted(rng.choice(n, size=k, replace=False).tolist())
        sim.ApplyGate(qs, mat32(random_unitary(rng, k)), st)
    s = ss.to_numpy(st)
    cdf = np.cumsum(np.abs(s) ** 2)
    total = cdf[-1]
    slack = 2e-8

    def holds(k, r):
        lo = 0.0 if k == 0 else cdf[k - 1]
        return lo - slack <= r <= cdf[k] + slack

    m = 2000
    u = np.zeros(m)
    oracle.L.orc_generate_random_values(m, 5, 1.0,
                                        u.ctypes.data_as(C.POINTER(C.c_double)))
    got = np.array(ss.Sample(st, m, 5), np.uint64)
    assert np.all(np.diff(got.astype(np.int64)) >= 0)
    bad = [j for j in range(m) if not holds(int(got[j]), u[j] * total)]
    assert not bad, (len(bad), bad[:5])
    for uu in (0.0, 0.3, 0.999999):
        bits = C.c_uint64()
        N.check(N.lib.qsg_measure(ss.ctx.h, st.get(), n, (1 << n) - 1, uu, 0,
                                  C.byref(bits)))
        assert holds(int(bits.value), uu * total)


def test_sample_edge_cases(eng):
    q, ss, sim = eng
    st = ss.Create(10)
    ss.SetStateZero(st)
    assert ss.Sample(st, 0, 1) == []
    assert set(ss.Sample(st, 100, 3)) == {0}
    ss.SetAllZeros(st)
    ss.SetAmpl(st, 1023, 1.0, 0.0)
    assert set(ss.Sample(st, 50, 3)) == {1023}


def test_partial_norms_and_find_measured_bits(eng, oracle):
    q, ss, sim = eng
    rng = np.random.default_rng(21)
    n = 16
    s = c64_to_c128(random_state(rng, n))
    st = ss.Create(n)
    ss.from_numpy(s, st)
    pn = ss.PartialNorms(st)
    chunk = (1 << n) // pn.size
    p = np.abs(s) ** 2
    # FP32 products and per-thread partial sums, FP64 accumulation.
    assert np.allclose(pn, p.reshape(pn.size, chunk).sum(1), rtol=1e-6, atol=1e-12)
    for m in (0, pn.size // 2, pn.size - 1):
        r = 0.6 * pn[m]
        cs = np.cumsum(p[m * chunk:(m + 1) * chunk])
        want = m * chunk + int(np.argmax(r < cs))
        assert ss.FindMeasuredBits(m, r, (1 << n) - 1, st) == want
        assert ss.FindMeasuredBits(m, r, 0b11, st) == want & 0b11


def test_measurement_sequence_matches_reference(eng):
    """Measure(qubits, mt19937(seed), state) repeated: same bits as the
    reference and the same collapsed state (lib/statespace.h:84-140)."""
    q, ss, sim = eng
    d = load_golden("rand14_k2")
    n = int(d["n"])
    st = ss.Create(n)
    ss.from_numpy(d["f64"], st)
    rgen = q.Rng(int(d["meas_seed"]))
    qs = d["meas_qs"].tolist()
    for want in d["meas_bits"]:
        res = ss.Measure(qs, rgen, st)
        assert res.valid and res.bits == int(want)
        assert res.bitstring == [(int(want) >> qq) & 1 for qq in qs]
    assert rel_l2(ss.to_numpy(st), d["meas_state"]) < TOL
    bad = ss.Measure([n], rgen, st)
    assert not bad.valid


def test_collapse(eng, oracle):
    q, ss, sim = eng
    rng = np.random.default_rng(3)
    n = 12
    s = c64_to_c128(random_state(rng, n))
    st = ss.Create(n)
    ss.from_numpy(s, st)
    mr = q.MeasurementResult(mask=0b1000100001, bits=0b1000000001, valid=True)
    ss.Collapse(mr, st)
    ref = s.copy()
    oracle.collapse(ref, n, mr.mask, mr.bits)
    assert rel_l2(ss.to_numpy(st), ref) < TOL


def test_errors_are_status_codes(eng):
    q, ss, sim = eng
    st = ss.Create(5)
    with pytest.raises(q.QsgError) as e:
        sim.ApplyGate([5], mat32(np.eye(2)), st)
    assert e.value.status == 1
    with pytest.raises(q.QsgError) as e:
        sim.ApplyGate([2, 1], mat32(np.eye(4)), st)
    assert e.value.status == 1
    with pytest.raises(q.QsgError) as e:
        sim.ApplyGate(list(range(7)), mat32(np.eye(128)), ss.Create(8))
    assert e.value.status == 4
    with pytest.raises(q.QsgError) as e:
        sim.ApplyControlledGate([1], [1], 1, mat32(np.eye(2)), st)
    assert e.value.status == 1
    big = ss.Create(39)  # 4 TiB: more than the device holds
    assert ss.IsNull(big)
    ok = ss.Create(3)
    assert not ss.IsNull(ok)
