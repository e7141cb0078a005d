"""Hybrid Schrodinger-Feynman simulation (lib/hybrid.h, lib/run_qsimh.h).

Fixtures (tests/golden/make_golden.py): hybrid_known.npz holds the
reference's own known-answer runs (tests/hybrid_testfixture.h: circuits,
parts, prefix/root splits, SplitLattice counts and expected amplitudes, read
from the reference's test file and checked against the reference there);
hybrid{6,8,10}.npz hold the reference's QSimHRunner amplitudes (double) of
seeded circuits for several prefix/root/suffix splits.

CPU: the Schmidt terms rebuild every gate, SplitLattice counts, the FP64
oracle (oracle/hybrid_oracle.py) equals the fixtures and, summed over all
paths, the state-vector amplitudes; unsupported operations are errors.
GPU: the engine's amplitudes through the C ABI against the fixtures
(absolute 2e-6 on the known answers, whose expected values carry 1e-6;
relative L2 1e-5 on the seeded cases), every device-batch split against the
others, and a 24-qubit circuit on the tensor-core path against the full
state vector."""
import os
import sys

import numpy as np
import pytest

from conftest import load_golden, rel_l2

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import hybrid_oracle as HO  # noqa: E402

RANDOM_CASES = ["hybrid6", "hybrid8", "hybrid10"]


def known_runs():
    d = load_golden("hybrid_known")
    out = []
    for i in range(int(d["count"])):
        out.append(dict(text=str(d[f"text{i}"]), parts=d[f"parts{i}"].tolist(),
                        counts=d[f"counts{i}"].tolist(), prefix=int(d[f"prefix{i}"]),
                        np=int(d[f"np{i}"]), nr=int(d[f"nr{i}"]), want=d[f"want{i}"]))
    return out


def circuit_ops(c):
    ops = c.ops()
    for i, o in enumerate(ops):
        o["schmidt"] = c.schmidt(i) if len(o["qs"]) == 2 else []
    return ops


@pytest.fixture(scope="module")
def E():
    from qsim_gb300 import engine
    return engine


def test_schmidt_terms_rebuild_the_gates(E):
    rng = np.random.default_rng(3)
    c = E.Circuit(4)
    specs = [("id2", ()), ("cz", ()), ("cnot", ()), ("cx", ()), ("sw", ()),
             ("is", ()), ("cp", (0.7,)), ("cp", (-2.1,)),
             ("fs", (0.9, 0.5)), ("fs", (-0.4, -1.3)), ("fs", (2.5, 3.9))]
    t = 0
    for name, ps in specs:
        for qs in ([0, 2], [3, 1]):
            c.add_named(t, name, qs, ps)
            t += 1
    c.add_named(t, "h", [0])
    for i, o in enumerate(c.ops()):
        terms = c.schmidt(i)
        if len(o["qs"]) == 1:
            assert terms == []
            continue
        assert len(terms) in (1, 2, 4)
        u = sum(np.kron(b, a) for a, b in terms)   # bit 0 <-> first qubit
        assert np.abs(u - o["m"]).max() < 1e-12
    del rng


def test_split_counts_match_reference(E):
    from qsim_gb300 import hybrid
    for r in known_runs()[::4]:
        info = hybrid.split_lattice(E.Circuit.parse(r["text"]), r["parts"])
        ops0, ops1, gx, n0, n1 = r["counts"]
        assert (info["num_ops0"], info["num_ops1"], info["num_gatexs"],
                info["num_qubits0"], info["num_qubits1"]) == (ops0, ops1, gx, n0, n1)


def test_oracle_matches_reference_known_answers(E):
    for r in known_runs():
        c = E.Circuit.parse(r["text"])
        got = HO.hybrid_amplitudes(c.num_qubits, circuit_ops(c), r["parts"],
                                   range(len(r["want"])), r["prefix"], r["np"],
                                   r["nr"])
        assert np.abs(got - r["want"]).max() < 2e-6


@pytest.mark.parametrize("case", RANDOM_CASES)
def test_oracle_matches_reference(E, case):
    d = load_golden(case)
    c = E.Circuit.parse(str(d["text"]))
    ops = circuit_ops(c)
    for (np_, nr, prefix), want in zip(d["runs"].tolist(), d["amps"]):
        got = HO.hybrid_amplitudes(int(d["n"]), ops, d["parts"].tolist(),
                                   d["bits"], prefix, np_, nr)
        assert np.abs(got - want).max() < 1e-10


def test_oracle_full_path_sum_is_the_state_vector(E, oracle):
    d = load_golden("hybrid8")
    c = E.Circuit.parse(str(d["text"]))
    n = c.num_qubits
    s = oracle.zero_state(n)
    for o in c.ops():
        oracle.apply_gate(s, n, o["qs"], o["m"])
    got = HO.hybrid_amplitudes(n, circuit_ops(c), d["parts"].tolist(),
                               d["bits"], 0, 0, 0)
    assert np.abs(got - s[d["bits"].astype(np.int64)]).max() < 1e-12


@pytest.mark.parametrize("text", [
    "3\n0 h 0\n1 c 0 1 x 2\n",          # controlled gate
    "3\n0 h 0\n1 m 0 1\n",              # measurement
])
def test_unsupported_operations_are_errors(E, text):
    from qsim_gb300 import hybrid
    from qsim_gb300._native import QsgError
    with pytest.raises(QsgError):
        hybrid.split_lattice(E.Circuit.parse(text), [0, 1, 1])


def test_bad_parts_are_errors(E):
    from qsim_gb300 import hybrid
    from qsim_gb300._native import QsgError
    c = E.Circuit.parse("3\n0 h 0\n1 cz 0 2\n")
    for parts in ([0, 1], [0, 2, 1], [1, 1, 1]):
        with pytest.raises(QsgError):
            hybrid.split_lattice(c, parts)


# ------------------------------------------------------------------ GPU --

@pytest.fixture(scope="module")
def ctx():
    import qsim_gb300 as q
    return q.Context(0)


@pytest.mark.gpu
def test_gpu_known_answers(E, ctx):
    from qsim_gb300 import hybrid
    for r in known_runs():
        c = E.Circuit.parse(r["text"])
        got, info = hybrid.run(ctx, c, r["parts"], range(len(r["want"])),
                               prefix=r["prefix"], num_prefix_gatexs=r["np"],
                               num_root_gatexs=r["nr"])
        assert np.abs(got - r["want"]).max() < 2e-6
        assert info["num_gatexs"] == r["counts"][2]


@pytest.mark.gpu
@pytest.mark.parametrize("case", RANDOM_CASES)
def test_gpu_matches_reference(E, ctx, case):
    from qsim_gb300 import hybrid
    d = load_golden(case)
    c = E.Circuit.parse(str(d["text"]))
    for (np_, nr, prefix), want in zip(d["runs"].tolist(), d["amps"]):
        for f in (2, 4):
            got, _ = hybrid.run(ctx, c, d["parts"].tolist(), d["bits"],
                                prefix=prefix, num_prefix_gatexs=np_,
                                num_root_gatexs=nr, max_fused_size=f)
            assert np.linalg.norm(want) > 1e-3
            assert rel_l2(got, want) < 1e-5


@pytest.mark.gpu
def test_gpu_batch_splits_agree(E, ctx):
    """Suffix path bits batched on the device or looped on the host, root
    gates or suffix gates: the same sum."""
    from qsim_gb300 import hybrid
    d = load_golden("hybrid10")
    c = E.Circuit.parse(str(d["text"]))
    parts, bits = d["parts"].tolist(), d["bits"]
    want = d["amps"][0]                      # all paths, no prefix
    seen = set()
    for nr in (0, 2):
        for mb in (1, 3, 6, 40):
            got, info = hybrid.run(ctx, c, parts, bits, num_root_gatexs=nr,
                                   max_batch_bits=mb)
            seen.add(info["batch_bits"])
            assert rel_l2(got, want) < 1e-5
    assert len(seen) >= 3
    # Results accumulate onto the caller's array, as the reference's do.
    acc = want.copy()
    hybrid.run(ctx, c, parts, bits, results=acc)
    assert rel_l2(acc, 2 * want) < 1e-5


@pytest.mark.gpu
def test_gpu_tensor_core_parts_match_state_vector(E, ctx):
    """24-qubit 6x4 grid, depth 8, cut between rows 3 and 4 (parts of 12
    qubits, 8 fSim gates on the cut = 16 path bits): hybrid amplitudes on
    the tensor-core path (parts of 12 qubits plus the path qubits) against
    the engine's full state vector."""
    import qsim_gb300 as q
    from qsim_gb300 import hybrid
    c = E.Circuit.grid(6, 4, 0, 8, 3)
    n = c.num_qubits
    parts = [0] * 12 + [1] * 12
    info0 = hybrid.split_lattice(c, parts)
    assert info0["num_gatexs"] == 8
    rng = np.random.default_rng(5)
    bits = rng.choice(1 << n, 512, replace=False).astype(np.uint64)
    got, info = hybrid.run(ctx, c, parts, bits, max_fused_size=6,
                           tensor_path=True, num_root_gatexs=min(2, info0["num_gatexs"]))
    ss = q.StateSpace(ctx=ctx)
    st = ss.Create(n)
    ss.SetStateZero(st)
    E.Plan(c, max_fused_size=4).run(ctx, st)
    want = ss.to_numpy(st)[bits.astype(np.int64)]
    assert rel_l2(got, want) < 2e-5
    assert info["batch_bits"] > 0
