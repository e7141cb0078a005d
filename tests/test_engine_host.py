"""CPU tests of the host engine: text parser and gate library against the
reference, fusion plans against the unfused circuit (the plan may change
speed, never the state), planner quality against the reference's
MultiQubitGateFuser, and the synthetic workload generators."""
import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_l2


@pytest.fixture(scope="module")
def E():
    from qsim_gb300 import engine
    return engine


def oracle_run_circuit(oracle, n, ops):
    s = oracle.zero_state(n)
    for o in ops:
        if o["kind"] == 0:
            oracle.apply_gate(s, n, o["qs"], o["m"])
        elif o["kind"] == 1:
            oracle.apply_controlled_gate(s, n, o["qs"], o["cqs"], o["cvals"], o["m"])
    return s


def test_parser_and_gate_library_match_reference(E, oracle):
    """Every gate of the text format, qubits in both orders, controlled
    gates: parsed here and applied by the oracle, the state equals the
    reference's CircuitQsimParser + SimulatorBasic<double> state."""
    d = load_golden("text_gates9")
    c = E.Circuit.parse(str(d["text"]))
    n = int(d["n"])
    assert c.num_qubits == n
    s = oracle_run_circuit(oracle, n, c.ops())
    assert rel_l2(s, d["f64"]) < 1e-12


@pytest.mark.parametrize("text", [
    "3\n0 foo 0\n",                 # unknown gate
    "3\n0 h 3\n",                   # qubit out of range
    "3\n0 cz 1 1\n",                # repeated qubit
    "3\n1 h 0\n0 x 0\n",            # out of time order on qubit 0
    "3\n0 h 0\n1 m 0\n0 x 1\n",     # crosses a measurement boundary
    "3\n0 rx 0\n",                  # missing parameter
    "3\n0 h 0 1\n",                 # trailing characters
    "3\n0 c 1 m 0\n",               # controlled measurement
    "0\n",                          # no qubits
])
def test_parser_rejects_invalid_input(E, text):
    from qsim_gb300 import QsgError
    with pytest.raises(QsgError):
        E.Circuit.parse(text)


def test_parser_maxtime(E):
    c = E.Circuit.parse("2\n0 h 0\n1 cz 0 1\n2 x 1\n", maxtime=1)
    assert len(c) == 2


def test_named_gates_are_unitary(E):
    c = E.Circuit(3)
    for name, qs, ps in [("h", [0], []), ("t", [1], []), ("x_1_2", [2], []),
                         ("y_1_2", [0], []), ("hz_1_2", [1], []),
                         ("rxy", [0], [0.3, 1.1]), ("fs", [2, 0], [1.2, -0.4]),
                         ("cp", [1, 2], [0.7]), ("is", [0, 2], []),
                         ("cnot", [2, 1], []), ("u3", [1], [0.1, 0.2, 0.3])]:
        c.add_named(0, name, qs, ps)
    for o in c.ops():
        m = o["m"]
        assert np.allclose(m @ m.conj().T, np.eye(m.shape[0]), atol=1e-12)
        assert o["qs"] == sorted(o["qs"])


def test_cnot_control_order(E, oracle):
    """cnot q0 q1 with q0 > q1: control stays on q0 after qubit sorting."""
    c = E.Circuit(2)
    c.add_named(0, "x", [1])
    c.add_named(1, "cnot", [1, 0])
    s = oracle_run_circuit(oracle, 2, c.ops())
    assert abs(s[3]) == pytest.approx(1.0)


def small_circuits(E):
    yield "grid3x4", E.Circuit.grid(3, 4, 0, 14, 3)
    yield "grid2x4p2", E.Circuit.grid(2, 4, 2, 10, 4)
    yield "chain11", E.Circuit.chain(11, 12, 5)
    yield "u3ctrl10", E.Circuit.layered_u3(10, 6, 3, 6)


@pytest.mark.parametrize("f", [1, 2, 3, 4, 5, 6])
def test_fused_plan_equals_unfused(E, oracle, f):
    """The fused plan's matrices (FP64) reproduce the unfused circuit's
    state to 1e-12 (reference test: tests/fuser_mqubit_test.cc:264-365)."""
    for name, c in small_circuits(E):
        n = c.num_qubits
        want = oracle_run_circuit(oracle, n, c.ops())
        plan = E.Plan(c, max_fused_size=f)
        s = oracle.zero_state(n)
        covered = 0
        for o in plan.ops():
            assert len(o["qs"]) <= max(f, 2) or o["kind"] != 0
            covered += o["members"]
            if o["kind"] == 0:
                oracle.apply_gate(s, n, o["qs"], o["m"])
            elif o["kind"] == 1:
                oracle.apply_controlled_gate(s, n, o["qs"], o["cqs"], o["cvals"], o["m"])
        assert covered == len(c)
        assert rel_l2(s, want) < 1e-12, (name, f)


def test_fused_plan_with_measurements_keeps_order(E):
    c = E.Circuit.parse("3\n0 h 0\n0 h 1\n1 cz 0 1\n2 m 0 1\n3 h 2\n3 x 0\n4 m 2\n")
    plan = E.Plan(c, max_fused_size=4)
    kinds = [o["kind"] for o in plan.ops()]
    assert kinds.count(2) == 2
    first_m = kinds.index(2)
    # Gates before the first measurement are fused into ops before it.
    assert all(k == 0 for k in kinds[:first_m])
    assert sum(o["members"] for o in plan.ops()) == len(c)


def test_planner_pass_counts_vs_reference_fuser(E):
    """Fused-op counts at max_fused_size 4, 5 and 6 on the seeded grid
    circuits are within 10% of (or below) the reference fuser's counts."""
    d = load_golden("fuser_mqubit_counts")
    for name in ("grid5x6d20", "grid4x5d14", "grid5x6p2d24"):
        c = E.Circuit.grid(*[int(x) for x in d[name + "_args"]])
        ref = d[name]  # f = 2..6
        for f in (4, 5, 6):
            mine = len(E.Plan(c, max_fused_size=f))
            assert mine <= 1.1 * ref[f - 2] + 1, (name, f, mine, ref[f - 2])


def test_multi_start_fusion_is_deterministic_and_fewest(E):
    """Tensor-core plans try several seed windows on parallel host threads
    and keep the fewest blocks (the first of equal ones): the same plan on
    every call, never more blocks than any single window."""
    c = E.Circuit.grid(5, 6, 0, 20, 1)
    plans = [E.Plan(c, max_fused_size=6, tensor_path=True) for _ in range(3)]
    sig = [[(o["qs"], o["members"]) for o in p.ops()] for p in plans]
    assert sig[0] == sig[1] == sig[2]
    assert len(plans[0]) == 36
    for w in (2, 3, 4, 6, 8, 12):
        single = E.Plan(c, max_fused_size=6, seeds=w)
        assert len(plans[0]) <= len(single)


def test_grid_generator_invariants(E):
    rows, cols, cycles = 4, 5, 14
    c = E.Circuit.grid(rows, cols, 0, cycles, 11)
    ops = c.ops()
    n = rows * cols
    one = [o for o in ops if len(o["qs"]) == 1]
    two = [o for o in ops if len(o["qs"]) == 2]
    assert len(one) == n * cycles
    # No qubit repeats its previous single-qubit gate.
    last = {}
    for o in one:
        key = o["m"].round(12).tobytes()
        assert last.get(o["qs"][0]) != key
        last[o["qs"][0]] = key
    # Each cycle's couplers are nearest neighbours and disjoint.
    by_time = {}
    for o in two:
        by_time.setdefault(o["time"], []).append(o["qs"])
        a, b = o["qs"]
        ra, ca, rb, cb = a // cols, a % cols, b // cols, b % cols
        assert abs(ra - rb) + abs(ca - cb) == 1
    for t, pairs in by_time.items():
        flat = [q for p in pairs for q in p]
        assert len(flat) == len(set(flat))
    # Deterministic by seed, different across seeds.
    c2 = E.Circuit.grid(rows, cols, 0, cycles, 11)
    assert all(np.array_equal(a["m"], b["m"]) for a, b in zip(ops, c2.ops()))
    c3 = E.Circuit.grid(rows, cols, 0, cycles, 12)
    assert not all(np.array_equal(a["m"], b["m"]) for a, b in zip(ops, c3.ops()))


def test_layered_u3_generator(E):
    c = E.Circuit.layered_u3(28, 40, 8, 3)
    ops = c.ops()
    ctrl = [o for o in ops if o["kind"] == 1]
    assert len(ctrl) == 40 * 8
    assert all(1 <= len(o["cqs"]) <= 2 and len(o["qs"]) == 1 for o in ctrl)
    u3 = [o for o in ops if o["kind"] == 0 and len(o["qs"]) == 1]
    assert len(u3) == 28 * 40
    # Times are ordered per qubit.
    last = {}
    for o in ops:
        for q in o["qs"] + o["cqs"]:
            assert o["time"] >= last.get(q, -1)
            last[q] = o["time"]


def test_pauli_sum(E):
    terms = E.pauli_sum(28, 64, 6, 9)
    assert len(terms) == 64
    for qs, letters, coeff in terms:
        assert 1 <= len(qs) <= 6 and qs == sorted(qs) and len(set(qs)) == len(qs)
        assert set(letters) <= set("XYZ") and -1 <= coeff <= 1


def test_learned_plan_absorbs_controlled_gates_and_keeps_the_state(E, oracle):
    """With the cost model, the planner may absorb controlled gates into
    blocks (as dense gates on targets and controls); the plan still applies
    the same circuit (FP64 oracle, unfused vs plan ops), and it has fewer
    controlled passes and fewer passes than the fixed fuser at f = 6."""
    from qsim_gb300 import learned as L
    m = L.CostMLP.load()
    c = E.Circuit.layered_u3(12, 8, 8, 5)
    n = c.num_qubits
    want = oracle.run_ops(n, c.ops())
    fixed = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5)
    learned = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=2,
                     cost_model=m)
    got = oracle_run_circuit(oracle, n, learned.ops())
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12
    ctrl = lambda p: sum(1 for o in p.ops() if o["kind"] == 1)  # noqa: E731
    assert ctrl(learned) < ctrl(fixed)
    assert len(learned) < len(fixed)


def run_bits(a, b):
    """Run bits of the two-gate tile of two padded 6-qubit target sets: the
    union completed with the lowest other qubits to 12, then the longest
    prefix 0..b-1 it holds with the rest above b (-1 without qubit 0)."""
    u = sorted(set(a) | set(b))
    q = 0
    while len(u) < 12:
        if q not in u:
            u.append(q)
        q += 1
    u.sort()
    h = next(h for h in range(13) if sum(x >= 12 - h for x in u) == h)
    return 12 - h if 12 - h >= 1 else -1


def pair_tile(a, b):
    """The two-gate tile of two padded 6-qubit target sets: their union
    completed with the lowest other qubits to 12."""
    u = set(a) | set(b)
    q = 0
    while len(u) < 12:
        u.add(q)
        q += 1
    return u


def pair_factor(a, b):
    """Measured cost of a two-gate pass relative to two one-gate passes by
    the shape of its tile (the planner's table): run bits rb, and for short
    runs the tile's other qubits below 12 (near) and in 12..20 (mid)."""
    u = pair_tile(a, b)
    rb = 0
    while rb in u:
        rb += 1
    if rb >= 4:
        return 0.80
    near = sum(1 for q in u if rb <= q < 12)
    mid = sum(1 for q in u if 12 <= q < 21)
    if rb == 3:
        return 0.87 if near >= 1 else 1.28
    if rb == 2:
        if near >= 2 or (near == 1 and mid >= 2):
            return 0.95
        return 1.28 if near == 1 else 2.49
    return 1.11 if rb == 1 else 2.49


def test_pair_factor_by_tile_shape(E):
    """The planner's pair cost by tile shape, at the geometries measured on
    the GB300: long runs 0.80 whatever the rest of the tile; 64-byte runs
    (3 run bits) need another tile qubit below 12, 32-byte runs (2) two of
    them or one and a spread of middle qubits; otherwise the pass costs more
    than two (1.28-2.49) and is never chosen."""
    hi = [21, 22, 23, 24, 25, 26, 27, 28, 29]
    assert pair_factor([0, 2, 5, 24, 26, 28], [1, 3, 23, 25, 27, 29]) == 0.80
    assert pair_factor([0, 2, 22, 24, 26, 28], [1, 3, 23, 25, 27, 29]) == 0.80
    assert pair_factor([0, 2, 22, 24, 26, 28], [1, 9, 23, 25, 27, 29]) == 0.87
    assert pair_factor([0, 2, 22, 24, 26, 28], [1, 12, 23, 25, 27, 29]) == 1.28
    assert pair_factor([0, 6] + hi[:4], [1] + hi[4:]) == 1.28
    assert pair_factor([0, 12] + hi[:4], [1] + hi[4:]) == 2.49
    assert pair_factor([12, 13, 14, 15, 16, 17], [0, 6, 12, 18, 24, 30]) == 0.95
    assert pair_factor([0, 4, 10, 16, 22, 28], [4, 5, 11, 17, 23, 29]) == 0.95
    # The 32-qubit pair that ran at 2.0x two passes in a learned plan.
    assert pair_factor([24, 25, 26, 27, 28, 29], [12, 18, 24, 25, 30, 31]) > 2


def test_pairs_only_where_the_tile_shape_pays(E):
    """Two consecutive 6-qubit tensor-core blocks share a pass only when
    their tile's shape was measured faster than two passes: qubits 0..11
    pair; a tile of qubits 0, 1, 12, 18, 24..31 (two run bits, no other
    tile qubit below 12: 2.0x two passes on the GB300) does not."""
    rng = np.random.default_rng(4)

    def u64():
        z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
        return np.linalg.qr(z)[0]

    for qa, qb, pairs in (([0, 1, 2, 3, 4, 5], [6, 7, 8, 9, 10, 11], 1),
                          ([24, 25, 26, 27, 28, 29], [12, 18, 24, 25, 30, 31], 0),
                          ([0, 2, 22, 24, 26, 28], [1, 9, 23, 25, 27, 29], 1),
                          ([0, 2, 22, 24, 26, 28], [1, 12, 23, 25, 27, 29], 0)):
        c = E.Circuit(32)
        c.add_gate(0, qa, u64())
        c.add_gate(1, qb, u64())
        plan = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5,
                      tc_pairs=2)
        assert len(plan) == 2
        assert plan.info()["num_tc_pairs"] == pairs, (qa, qb)


def test_bench_pair_factor_is_the_planners():
    """bench.py predicts plan times with the planner's pair table: its
    mirror agrees with this file's on random pairs of 6-qubit target sets
    (whose planner consistency test_two_gate_pass_pairing checks)."""
    import importlib
    import sys
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    rng = np.random.default_rng(3)
    n = 30
    seen = set()
    for _ in range(400):
        a = sorted(rng.choice(n, 6, replace=False).tolist())
        b = sorted(rng.choice(n, 6, replace=False).tolist())
        if len(set(a) | set(b)) > 12:
            continue
        f = pair_factor(a, b)
        assert bench.pair_cost_factor(n, a, b) == f, (a, b)
        seen.add(f)
    assert len(seen) >= 3


@pytest.mark.parametrize("bits", [1, 3, 5])
def test_two_gate_pass_pairing(E, bits):
    """Pairs of consecutive tensor-core blocks marked for two-gate passes:
    no op in two pairs, both ops 6-qubit tensor-core gates, their tile has
    >= `bits` run bits and a pair is predicted faster than two passes, the
    set of pairs has the largest predicted saving (checked here by the same
    recursion over the chain of consecutive ops), and the plan costs no
    more passes than the plan chosen without pairs (the fixed planner
    compares its candidates by passes, a pair at its measured cost)."""
    c = E.Circuit.grid(5, 6, 0, 20, 1)
    base = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5)
    plan = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5,
                  tc_pairs=bits)
    pn = plan.tc_pair_next()
    assert plan.info()["num_tc_pairs"] == int(pn.sum())
    ops = plan.ops()
    gain = [0.0] * len(ops)
    for i in range(len(ops) - 1):
        if (ops[i]["path"] == 1 and ops[i + 1]["path"] == 1
                and len(ops[i]["qs"]) == 6 and len(ops[i + 1]["qs"]) == 6):
            rb = run_bits(ops[i]["qs"], ops[i + 1]["qs"])
            if rb >= bits:
                gain[i] = max(0.0, 2 * (1 - pair_factor(ops[i]["qs"],
                                                        ops[i + 1]["qs"])))
    cost = 0.0
    i = 0
    while i < len(ops):
        if pn[i]:
            assert gain[i] > 0
            assert i + 1 < len(ops) and not pn[i + 1]
            cost += 2 - gain[i]
            i += 2
        else:
            cost += 1
            i += 1
    assert cost <= len(base) + 1e-9
    best = [0.0] * (len(ops) + 2)
    for i in range(len(ops) - 1, -1, -1):
        best[i] = max(best[i + 1], (gain[i] + best[i + 2]) if gain[i] > 0 else 0)
    assert abs(sum(gain[i] for i in np.flatnonzero(pn)) - best[0]) < 1e-9
    assert int(pn.sum()) > 0
    assert E.Plan(c, max_fused_size=6, tensor_path=True,
                  tc_min_k=5).info()["num_tc_pairs"] == 0
