"""Precision of every engine form against the FP64 state-vector oracle.

Workloads (seeded synthetic circuits with the configurations' shapes):

* grid random circuit, sqrt(X)/sqrt(Y)/sqrt(W) + fSim(pi/2, pi/6), depth
  20: the plain CUDA-core plan (max_fused_size 4), the tensor-core plans
  (f = 6 with blocks of >= 5 qubits on tcgen05, and every block on
  tcgen05) and the learned planner's plan.  Bar: relative L2 <= 1e-5 and
  fidelity >= 1 - 1e-6 against FP64.
* layered U3 + CZ/CNOT circuit with 8 controlled gates per layer, 40
  layers, then 64 Pauli strings of weight 1..6: every expectation value
  (FP32 state, FP64 reductions) within 1e-5 of the FP64 value, the weighted
  sum within 1e-4.

By default the grid is 4x6 (24 qubits) and the layered circuit has 20
qubits; QSG_FULL_SIZE=1 runs the full sizes (5x6 grid = 30 qubits, FP64
oracle 16 GiB on the host; layered circuit on 28 qubits).  The 30-qubit grid
circuit's plain, tensor-core and learned forms are checked at full size in
every run (test_headline_circuit_30q_against_fp64).  Each test prints
one JSON line with the measured errors (pytest -s shows it)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FULL = os.environ.get("QSG_FULL_SIZE", "0") == "1"
CHUNK = 1 << 24


@pytest.fixture(scope="module")
def eng():
    import qsim_gb300 as q
    from qsim_gb300 import engine as E
    ctx = q.Context(0)
    return q, E, ctx, q.StateSpace(ctx=ctx), q.Simulator(ctx=ctx)


def oracle_state(oracle, c):
    return oracle.run_ops_fp64_fused(c.num_qubits, c.ops())


def state_c64(ss, st):
    """The device state as a complex64 host array (no FP64 copy: 8 GiB at
    30 qubits)."""
    buf = np.empty(ss.MinSize(st.num_qubits()), dtype=np.float32)
    ss.Copy(st, buf)
    return buf[: 2 << st.num_qubits()].view(np.complex64)


def errors(got, want):
    """(relative L2, fidelity) of a complex64 state against a complex128
    one, accumulated in FP64 over chunks (no full-size temporaries)."""
    d2 = w2 = g2 = 0.0
    ip = 0j
    for i in range(0, want.size, CHUNK):
        g = got[i:i + CHUNK].astype(np.complex128)
        w = want[i:i + CHUNK]
        d2 += float(np.vdot(g - w, g - w).real)
        w2 += float(np.vdot(w, w).real)
        g2 += float(np.vdot(g, g).real)
        ip += complex(np.vdot(w, g))
    return float(np.sqrt(d2 / w2)), float(abs(ip) ** 2 / (w2 * g2))


def test_grid_circuit_forms_against_fp64(eng, oracle):
    q, E, ctx, ss, sim = eng
    from qsim_gb300 import learned as L
    rows, cols = (5, 6) if FULL else (4, 6)
    c = E.Circuit.grid(rows, cols, 0, 20, 1)
    n = c.num_qubits
    want = oracle_state(oracle, c)
    forms = {
        "plain_f4": E.Plan(c, max_fused_size=4),
        "tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5),
        "tc_f6_all": E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=1),
        "learned_tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True,
                                tc_min_k=2, cost_model=L.CostMLP.load()),
        "learned_tc_f6_pairs": E.Plan(c, max_fused_size=6, tensor_path=True,
                                      tc_min_k=2, cost_model=L.CostMLP.load(),
                                      tc_pairs=3),
    }
    assert forms["learned_tc_f6_pairs"].info()["num_tc_pairs"] > 0
    st = ss.Create(n)
    out = {"workload": f"grid{rows}x{cols} ({n} qubits) depth 20, seed 1",
           "forms": {}}
    for name, plan in forms.items():
        ss.SetStateZero(st)
        plan.run(ctx, st)
        rel, fid = errors(state_c64(ss, st), want)
        out["forms"][name] = {"rel_l2": rel, "fidelity": fid,
                              "passes": len(plan)}
    print(json.dumps(out))
    for name, r in out["forms"].items():
        assert r["rel_l2"] <= 1e-5, name
        assert r["fidelity"] >= 1 - 1e-6, name


def test_headline_circuit_30q_against_fp64(eng, oracle):
    """The 30-qubit 5x6 grid depth-20 circuit (seed 1) at its full size in
    every default run: the plain CUDA-core f = 4 plan, the split-FP16
    tensor-core f = 6 plan, the learned planner's plan and the same with
    two-gate tensor-core passes (the form the headline time is measured
    on), each against the FP64 oracle (one-qubit gates folded into
    two-qubit gates in FP64, 16 GiB on the host).  Bar: relative L2 <= 1e-5
    and fidelity >= 1 - 1e-6."""
    q, E, ctx, ss, sim = eng
    from qsim_gb300 import learned as L
    c = E.Circuit.grid(5, 6, 0, 20, 1)
    n = c.num_qubits
    want = oracle.run_ops_fp64_fused(n, c.ops())
    forms = {
        "plain_f4": E.Plan(c, max_fused_size=4),
        "tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5),
        "learned_tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True,
                                tc_min_k=2, cost_model=L.CostMLP.load()),
        "learned_tc_f6_pairs": E.Plan(c, max_fused_size=6, tensor_path=True,
                                      tc_min_k=2, cost_model=L.CostMLP.load(),
                                      tc_pairs=3),
    }
    st = ss.Create(n)
    out = {"workload": "grid5x6 (30 qubits) depth 20, seed 1", "forms": {}}
    for name, plan in forms.items():
        ss.SetStateZero(st)
        plan.run(ctx, st)
        rel, fid = errors(state_c64(ss, st), want)
        out["forms"][name] = {"rel_l2": rel, "fidelity": fid,
                              "passes": len(plan)}
    del st
    print(json.dumps(out))
    for name, r in out["forms"].items():
        assert r["rel_l2"] <= 1e-5, name
        assert r["fidelity"] >= 1 - 1e-6, name


def test_layered_controlled_expectations_against_fp64(eng, oracle):
    q, E, ctx, ss, sim = eng
    from conftest import pauli_matrix
    n = 28 if FULL else 20
    c = E.Circuit.layered_u3(n, 40, 8, 3)
    want = oracle_state(oracle, c)
    st = ss.Create(n)
    ss.SetStateZero(st)
    E.Plan(c, max_fused_size=4).run(ctx, st)
    rel, fid = errors(state_c64(ss, st), want)
    worst, tot, tot_ref = 0.0, 0.0, 0.0
    for qs, letters, coeff in E.pauli_sum(n, 64, 6, 5):
        m = pauli_matrix(letters)
        ev = sim.ExpectationValue(
            qs, np.ascontiguousarray(m.astype(np.complex64)).view(np.float32), st)
        evr = oracle.expectation_value(want, n, qs, m)
        worst = max(worst, abs(ev - evr))
        tot += coeff * ev.real
        tot_ref += coeff * evr.real
    print(json.dumps({"workload": f"layered U3 ({n} qubits) 40 layers, 8 "
                      "controlled gates per layer, 64 Pauli strings",
                      "state_rel_l2": rel, "state_fidelity": fid,
                      "ev_max_abs_err": worst,
                      "pauli_sum_abs_err": abs(tot - tot_ref)}))
    assert rel <= 1e-5 and fid >= 1 - 1e-6
    assert worst < 1e-5
    assert abs(tot - tot_ref) < 1e-4
