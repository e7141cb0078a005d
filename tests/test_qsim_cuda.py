"""The qsim_cuda-compatible module (qsim_gb300.qsim_cuda) against the
reference's own Python extension (pybind_interface/pybind_main.cpp with the
basic CPU factory, built from its sources by `make -C oracle pybind`).

The fixture tests/golden/pybind_module.npz (written by make_golden.py
pybind) holds circuits described as builder calls and the reference module's
outputs for them: one 4-qubit circuit per Cirq gate kind (final state), a
10-qubit circuit of every builder (gates with random parameters, controls,
diagonal and matrix gates) with its final states from |0>, a basis state and
a state vector, amplitudes of bitstrings, 500 samples, expectation values of
Pauli sums (one on 8 qubits, one the identity) and moment expectation
values, a circuit with measurements (qsim_sample bits for 3 seeds), and a
noisy circuit (Pauli-mixture, amplitude-damping and two-qubit channels)
with one trajectory's state, amplitudes and samples per seed, expectation
values over 8 and 4 repetitions, and measurement bits per seed, and an
8-qubit circuit of Cirq gates cut into halves (6 gates on the cut) with
qsimh_simulate's amplitudes for five prefix/root splits.

CPU: the module exports every name of the reference module's simulator and
builder interface with the same enum values; the gate matrices, applied by
the FP64 oracle, reproduce the reference's states.  GPU: every entry point
through the engine against the fixture (states relative L2 <= 1e-5, the
FP32 bar of the other tests; amplitudes and expectation values within 2e-6;
samples >= 99 % identical; measurement bits equal)."""
import json

import numpy as np
import pytest

from conftest import load_golden, rel_l2

# Every entry point of the reference module is built.
NOT_BUILT = set()


@pytest.fixture(scope="module")
def fx():
    d = load_golden("pybind_module")
    return {k: json.loads(str(v)) for k, v in d.items()}


@pytest.fixture(scope="module")
def Q():
    from qsim_gb300 import qsim_cuda
    return qsim_cuda


def build(Q, n, desc):
    c = Q.Circuit()
    c.num_qubits = n
    for d in desc:
        if d["t"] == "gate":
            Q.add_gate(getattr(Q, d["kind"]), d["time"], d["qubits"], d["params"], c)
        elif d["t"] == "diag":
            Q.add_diagonal_gate(d["time"], d["qubits"], d["angles"], c)
        elif d["t"] == "matrix":
            Q.add_matrix_gate(d["time"], d["qubits"], d["matrix"], c)
        elif d["t"] == "ctrl":
            Q.control_last_gate(d["qubits"], d["values"], c)
        elif d["t"] == "meas":
            Q.add_measurement(d["time"], d["qubits"], c)
        elif d["t"] == "chan":
            Q.add_channel(d["time"], d["qubits"], [tuple(k) for k in d["kops"]], c)
    return c


def opsums(Q, spec):
    out = []
    for strings, count in spec:
        ops = []
        for weight, terms in strings:
            s = Q.OpString()
            s.weight = complex(*weight)
            for kind, qs in terms:
                Q.add_gate_to_opstring(getattr(Q, kind), qs, s)
            ops.append(s)
        out.append((ops, count))
    return out


def options(c, **kw):
    return dict(dict(c=c, f=2, s=1, t=1, v=0, z=0), **kw)


def cplx(v):
    return np.asarray(v, np.float32).view(np.complex64).astype(np.complex128)


def oracle_state(Q, oracle, c):
    n = c.num_qubits
    s = oracle.zero_state(n)
    for o in c.ops:
        qs, m = Q._sorted(o["qs"], o["m"])
        if o["kind"] == 1:
            cq = o["cqs"]
            order = sorted(range(len(cq)), key=lambda i: cq[i])
            cv = sum(((o["cvals"] >> i) & 1) << j for j, i in enumerate(order))
            oracle.apply_controlled_gate(s, n, qs, sorted(cq), cv, m)
        elif o["kind"] == 0:
            oracle.apply_gate(s, n, qs, m)
    return s


def test_module_interface_matches_reference(fx, Q):
    missing = [x for x in fx["names"] if x not in NOT_BUILT and not hasattr(Q, x)]
    assert missing == []
    for name, v in fx["kind_values"].items():
        assert int(getattr(Q, name)) == v, name


def test_gate_matrices_reproduce_reference_states(fx, Q, oracle):
    """Each Cirq gate kind with random parameters, applied by the FP64
    oracle from this module's matrices, gives the reference module's state."""
    for case in fx["gate_kinds"]:
        c = build(Q, 4, case["desc"])
        assert rel_l2(oracle_state(Q, oracle, c), cplx(case["fs"])) < 1e-6, \
            case["desc"][-1]


def test_mixed_circuit_on_the_oracle(fx, Q, oracle):
    """Controls, diagonal and matrix gates of the 10-qubit circuit through
    this module's builders, applied by the oracle: the reference's state."""
    m = fx["mixed"]
    c = build(Q, m["n"], m["desc"])
    assert rel_l2(oracle_state(Q, oracle, c), cplx(m["fs0"])) < 1e-6


def test_qsimh_terms_on_the_oracle(fx, Q):
    """The Schmidt terms given to the engine for the Cirq gates on the cut,
    summed over paths by the FP64 hybrid oracle: the reference module's
    qsimh amplitudes, also for partial sums over fixed prefixes."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
    import hybrid_oracle as HO
    h = fx["hybrid"]
    n = h["n"]
    ec = Q._hybrid_circuit(build(Q, n, h["desc"]))
    ops = ec.ops()
    for i, o in enumerate(ops):
        o["schmidt"] = ec.schmidt(i) if len(o["qs"]) == 2 else []
    parts = [1 if q in h["k"] else 0 for q in range(n)]
    bits = Q._bitstrings(h["btxt"], n)
    for r in h["runs"]:
        got = HO.hybrid_amplitudes(n, ops, parts, bits, r["w"], r["p"], r["r"])
        want = np.array([complex(*a) for a in r["amps"]])
        assert np.abs(got - want).max() < 2e-6, (r["p"], r["r"], r["w"])


def test_bitstring_parsing(Q):
    assert Q._bitstrings("011\n100\n", 3) == [0b110, 0b001]
    with pytest.raises(ValueError):
        Q._bitstrings("01\n", 3)


# ------------------------------------------------------------------ GPU --

@pytest.mark.gpu
def test_gpu_every_gate_kind(fx, Q):
    for case in fx["gate_kinds"]:
        c = build(Q, 4, case["desc"])
        got = Q.qsim_simulate_fullstate(options(c), 0)
        assert got.dtype == np.float32 and got.size == 32
        assert rel_l2(cplx(got), cplx(case["fs"])) < 1e-5, case["desc"][-1]


@pytest.mark.gpu
def test_gpu_mixed_circuit_entry_points(fx, Q):
    m = fx["mixed"]
    c = build(Q, m["n"], m["desc"])
    assert rel_l2(cplx(Q.qsim_simulate_fullstate(options(c), 0)), cplx(m["fs0"])) < 1e-5
    vec = np.asarray(m["vec"], np.float32)
    assert rel_l2(cplx(Q.qsim_simulate_fullstate(options(c), vec)),
                  cplx(m["fs_vec"])) < 1e-5
    assert rel_l2(cplx(Q.qsim_simulate_fullstate(options(c), 37)),
                  cplx(m["fs_basis"])) < 1e-5
    amps = np.array(Q.qsim_simulate(options(c, i=m["btxt"])))
    want = np.array([complex(*a) for a in m["amps"]])
    assert np.abs(amps - want).max() < 2e-6
    smp = np.array(Q.qsim_sample_final(options(c, s=5), 500))
    assert np.mean(smp == np.array(m["samples"])) >= 0.99
    evs = np.array(Q.qsim_simulate_expectation_values(
        options(c), opsums(Q, m["opsums"]), 0))
    want = np.array([complex(*e) for e in m["evs"]])
    assert np.abs(evs - want).max() < 2e-6
    mevs = Q.qsim_simulate_moment_expectation_values(
        options(c), [(end, opsums(Q, sp)) for end, sp in m["moments"]], 0)
    for row, wrow in zip(mevs, m["mevs"]):
        assert np.abs(np.array(row) - np.array([complex(*e) for e in wrow])).max() < 2e-6


@pytest.mark.gpu
def test_gpu_measurement_bits(fx, Q):
    m = fx["measure"]
    c = build(Q, m["n"], m["desc"])
    for seed, want in m["seeds"].items():
        assert Q.qsim_sample(options(c, s=int(seed))) == want


@pytest.mark.gpu
def test_gpu_noisy_circuit_entry_points(fx, Q):
    """The reference's trajectories for the same seeds: the same Kraus
    choices, so the same states (FP32 bar), amplitudes, samples, averaged
    expectation values and measurement bits."""
    m = fx["noisy"]
    n = m["n"]
    c = build(Q, n, m["desc"])
    vec = np.asarray(m["vec"], np.float32)
    for seed in m["fs"]:
        o = options(c, s=int(seed), r=1)
        assert rel_l2(cplx(Q.qtrajectory_simulate_fullstate(o, 0)),
                      cplx(m["fs"][seed])) < 1e-5, seed
        assert rel_l2(cplx(Q.qtrajectory_simulate_fullstate(o, vec)),
                      cplx(m["fs_vec"][seed])) < 1e-5, seed
        amps = np.array(Q.qtrajectory_simulate(options(c, s=int(seed), i=m["btxt"])))
        want = np.array([complex(*a) for a in m["amps"][seed]])
        assert np.abs(amps - want).max() < 2e-6
        smp = np.array(Q.qtrajectory_sample_final(o, 200))
        assert np.mean(smp == np.array(m["samples"][seed])) >= 0.99
    evs = np.array(Q.qtrajectory_simulate_expectation_values(
        options(c, r=8), opsums(Q, m["opsums"]), 0))
    want = np.array([complex(*e) for e in m["evs"]])
    assert np.abs(evs - want).max() < 2e-6
    mevs = Q.qtrajectory_simulate_moment_expectation_values(
        options(c, r=4), [(end, opsums(Q, sp)) for end, sp in m["moments"]], 0)
    for row, wrow in zip(mevs, m["mevs"]):
        assert np.abs(np.array(row) - np.array([complex(*e) for e in wrow])).max() < 2e-6
    mc = build(Q, n, m["mdesc"])
    for seed, want in m["mbits"].items():
        assert Q.qtrajectory_sample(options(mc, s=int(seed), r=1)) == want


@pytest.mark.gpu
def test_gpu_qsimh(fx, Q):
    h = fx["hybrid"]
    c = build(Q, h["n"], h["desc"])
    for r in h["runs"]:
        got = np.array(Q.qsimh_simulate(options(c, i=h["btxt"], k=h["k"], w=r["w"],
                                                p=r["p"], r=r["r"])))
        want = np.array([complex(*a) for a in r["amps"]])
        assert np.abs(got - want).max() < 2e-6, (r["p"], r["r"], r["w"])
