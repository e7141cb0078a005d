"""Unitary calculator (lib/unitaryspace_basic.h, lib/unitary_calculator_basic.h).

CPU: the oracle's restatement (a 2n-qubit state whose gates act on the
column bits) equals the reference's own UnitaryCalculatorBasic<double> on the
golden circuits (tests/golden/unitary*.npz, made by make_golden.py), and
from the identity entry (i, j) is (Gm ... G1)[j][i].  GPU: the engine's
unitaries through the C ABI against those goldens (relative L2 <= 1e-5, the
FP32 bar of the state-vector tests), entry access, the identity, fused
(CUDA-core and tensor-core) plans, and argument errors."""
import numpy as np
import pytest

from conftest import UNITARY_CASES, load_golden, rel_l2, unpack_ops

TOL = 1e-5


def golden_unitary(d):
    n = int(d["n"])
    return n, d["u64"].reshape(1 << n, 1 << n)


def circuit_matrix(n, ops):
    """Product Gm ... G1 of the ops on n qubits (bit q of an index is qubit
    q; bit j of a gate's matrix index is its qs[j])."""
    d = 1 << n
    c = np.eye(d, dtype=np.complex128)
    idx = np.arange(d)
    for o in ops:
        qs, cqs = o["qs"], o.get("cqs", [])
        k = len(qs)
        g = np.zeros((d, d), dtype=np.complex128)
        for col in range(d):
            ok = all(((col >> q) & 1) == ((o["cvals"] >> i) & 1)
                     for i, q in enumerate(cqs))
            if not ok:
                g[col, col] = 1.0
                continue
            sub = sum(((col >> q) & 1) << j for j, q in enumerate(qs))
            base = col & ~sum(1 << q for q in qs)
            for r in range(1 << k):
                row = base | sum(((r >> j) & 1) << q for j, q in enumerate(qs))
                g[row, col] = o["m"][r, sub]
        c = g @ c
    del idx
    return c


@pytest.mark.parametrize("case", UNITARY_CASES)
def test_oracle_unitary_matches_reference(case, oracle):
    d = load_golden(case)
    n, want = golden_unitary(d)
    got = oracle.unitary(n, unpack_ops(d))
    assert rel_l2(got.ravel(), want.ravel()) < 1e-12


@pytest.mark.parametrize("case", UNITARY_CASES[:2])
def test_reference_layout_is_the_transposed_circuit_matrix(case):
    d = load_golden(case)
    n, want = golden_unitary(d)
    c = circuit_matrix(n, unpack_ops(d))
    assert np.allclose(want, c.T, atol=1e-10)


# ------------------------------------------------------------------ GPU --

@pytest.fixture(scope="module")
def uc():
    from qsim_gb300 import api
    from qsim_gb300 import unitary as U
    ctx = api.Context()
    return U.UnitarySpace(ctx=ctx), U.UnitaryCalculator(ctx=ctx), ctx


def mat32(m):
    return np.ascontiguousarray(np.asarray(m, np.complex64)).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("case", UNITARY_CASES)
def test_gpu_unitary_matches_reference(case, uc):
    us, calc, _ = uc
    d = load_golden(case)
    n, want = golden_unitary(d)
    u = us.CreateUnitary(n)
    us.SetIdentity(u)
    for o in unpack_ops(d):
        if o["kind"] == 0:
            calc.ApplyGate(o["qs"], mat32(o["m"]), u)
        else:
            calc.ApplyControlledGate(o["qs"], o["cqs"], o["cvals"], mat32(o["m"]), u)
    got = us.to_numpy(u)
    assert rel_l2(got.ravel(), want.ravel()) < TOL
    # GetEntry reads the reference's (i, j).
    for i, j in ((0, 0), (1, 2), ((1 << n) - 1, 3 % (1 << n))):
        assert abs(us.GetEntry(u, i, j) - want[i, j]) < 1e-5


@pytest.mark.gpu
def test_gpu_identity_entries_and_zeros(uc):
    us, calc, _ = uc
    n = 4
    u = us.CreateUnitary(n)
    us.SetIdentity(u)
    assert np.array_equal(us.to_numpy(u), np.eye(1 << n))
    us.SetEntry(u, 3, 5, 0.25 - 0.5j)
    assert us.GetEntry(u, 3, 5) == 0.25 - 0.5j
    assert us.to_numpy(u)[3, 5] == 0.25 - 0.5j
    v = us.CreateUnitary(n)
    us.CopyUnitary(u, v)
    assert np.array_equal(us.to_numpy(v), us.to_numpy(u))
    us.SetAllZeros(u)
    assert not us.to_numpy(u).any()


@pytest.mark.gpu
@pytest.mark.parametrize("n,f,tc,pairs", [(5, 4, False, 0), (7, 3, False, 0),
                                          (12, 6, True, 0), (12, 6, True, 1)])
def test_gpu_unitary_from_fused_plan(uc, oracle, n, f, tc, pairs):
    """A fused plan applied to the unitary (tensor-core blocks on tcgen05
    for the 12-qubit circuit: a 2^24-entry unitary; with `pairs`, blocks
    two at a time in two-gate passes) equals the unfused oracle unitary."""
    us, calc, ctx = uc
    from qsim_gb300 import engine as E
    c = E.Circuit.chain(n, 4, 30 + n) if n < 12 else E.Circuit.grid(3, 4, 0, 3, 5)
    plan = E.Plan(c, max_fused_size=f, tensor_path=tc, tc_min_k=2,
                  tc_pairs=pairs)
    if tc:
        assert plan.info()["num_tensor_ops"] > 0
    if pairs:
        assert plan.info()["num_tc_pairs"] > 0
    u = us.CreateUnitary(n)
    us.SetIdentity(u)
    calc.RunPlan(plan, u)
    ops = [o for o in c.ops() if o["kind"] in (0, 1)]
    want = oracle.unitary(n, ops)
    assert rel_l2(us.to_numpy(u).ravel(), want.ravel()) < TOL


@pytest.mark.gpu
def test_gpu_unitary_argument_errors(uc):
    us, calc, _ = uc
    from qsim_gb300._native import QsgError
    u = us.CreateUnitary(3)
    with pytest.raises(QsgError):
        calc.ApplyGate([3], mat32(np.eye(2)), u)        # qubit >= n
    with pytest.raises(QsgError):
        us.GetEntry(u, 8, 0)                            # row out of range
    with pytest.raises(QsgError):
        us.CreateUnitary(21)                            # 2n > 40
