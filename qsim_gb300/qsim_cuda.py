"""qsim's Python extension interface (the ``qsim_cuda`` module that qsimcirq
loads for ``use_gpu=True``: pybind_interface/pybind_main.h and
pybind_main.cpp) on the GB300 engine.

Same names, arguments and results as the reference module: ``Circuit``
(``num_qubits``), ``OpString`` (``weight``), the Cirq gate kinds (``kXPowGate``
... with the reference's enum values, lib/gates_cirq.h:30-78), the circuit
builders (``add_gate``, ``add_diagonal_gate``, ``add_matrix_gate``,
``add_measurement``, ``control_last_gate``, ``add_gate_to_opstring``,
``add_matrix_gate_to_opstring``) and the simulators taking the options dict
(``"c"`` circuit, ``"i"`` bitstrings as lines of 0/1 with qubit 0 first,
``"f"`` max fused size, ``"s"`` seed, ``"t"``, ``"v"``, ``"z"``):
``qsim_simulate``, ``qsim_simulate_fullstate``, ``qsim_sample``,
``qsim_sample_final``, ``qsim_simulate_expectation_values`` and
``qsim_simulate_moment_expectation_values``, and for noisy circuits
(``add_channel``) the ``qtrajectory_*`` counterparts on the engine's
trajectory runner, and ``qsimh_simulate`` on the hybrid simulator
(``qsim_gb300.hybrid``) with the reference's Schmidt terms of the Cirq
two-qubit gates.

Gate matrices follow Cirq's definitions (eigen-decomposed power gates
U(t, s) = sum_k exp(i pi t (theta_k + s)) P_k), in the reference's layout:
bit j of a matrix index belongs to the j-th listed qubit, so a two-qubit
Cirq gate on (q0, q1) acts with q0 as bit 0; matrix gates and diagonal gates
take Cirq's big-endian order (first qubit most significant) as the
reference does (lib/gates_cirq.h MatrixGate, TwoQubitDiagonalGate).
"""
from __future__ import annotations

import enum
import math
from typing import Dict, List

import numpy as np

# ---------------------------------------------------------------- kinds --

_KIND_NAMES = [
    "kI1", "kI2", "kI", "kXPowGate", "kYPowGate", "kZPowGate", "kHPowGate",
    "kCZPowGate", "kCXPowGate", "krx", "kry", "krz", "kH", "kS", "kCZ", "kCX",
    "kT", "kX", "kY", "kZ", "kPhasedXPowGate", "kPhasedXZGate", "kXXPowGate",
    "kYYPowGate", "kZZPowGate", "kXX", "kYY", "kZZ", "kSwapPowGate",
    "kISwapPowGate", "kriswap", "kSWAP", "kISWAP", "kPhasedISwapPowGate",
    "kgivens", "kFSimGate", "kTwoQubitDiagonalGate",
    "kThreeQubitDiagonalGate", "kCCZPowGate", "kCCXPowGate", "kCSwapGate",
    "kCCZ", "kCCX", "kMatrixGate1", "kMatrixGate2", "kMatrixGate",
    "kGlobalPhaseGate",
]
GateKind = enum.IntEnum("GateKind", [(n, i) for i, n in enumerate(_KIND_NAMES)])
globals().update({k.name: k for k in GateKind})


class OtherGateKind(enum.IntEnum):
    kMeasurement = 100002


kMeasurement = OtherGateKind.kMeasurement

# ---------------------------------------------------------- gate matrices --

_I = np.eye(2, dtype=np.complex128)
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
_Z = np.diag([1.0, -1.0]).astype(np.complex128)
_P0 = np.diag([1.0, 0.0]).astype(np.complex128)
_P1 = np.diag([0.0, 1.0]).astype(np.complex128)
_HM = (_X + _Z) / math.sqrt(2)


def _kron(*ms):
    """Kronecker product with the FIRST factor on bit 0 (the first listed
    qubit): _kron(A, B)[(a0 + 2 b0), (a1 + 2 b1)] = A[a0, a1] B[b0, b1]."""
    out = np.eye(1, dtype=np.complex128)
    for m in ms:
        out = np.kron(m, out)
    return out


def _power(components, t, s=0.0):
    """Cirq EigenGate: sum_k exp(i pi t (theta_k + s)) P_k."""
    return sum(np.exp(1j * math.pi * t * (theta + s)) * p
               for theta, p in components)


def _proj(v):
    v = np.asarray(v, dtype=np.complex128)
    return np.outer(v, v.conj())


def _pauli_pow(p, t, s):
    d = p.shape[0]
    e = np.eye(d, dtype=np.complex128)
    return _power([(0.0, (e + p) / 2), (1.0, (e - p) / 2)], t, s)


def _zpow(t, s=0.0):
    return _power([(0.0, _P0), (1.0, _P1)], t, s)


def _xpow(t, s=0.0):
    return _pauli_pow(_X, t, s)


def _cpow(target_proj, t, s, ncontrols):
    """Controlled power gate: the phase exp(i pi t) on controls = 1 and the
    target projector; controls are the first listed qubits."""
    p = _kron(*([_P1] * ncontrols), target_proj)
    e = np.eye(p.shape[0], dtype=np.complex128)
    return _power([(0.0, e - p), (1.0, p)], t, s)


def _iswap_pow(t, s=0.0):
    # |01> (q0 = 1) is index 1, |10> (q1 = 1) index 2 in this layout.
    plus = np.zeros(4)
    plus[1] = plus[2] = math.sqrt(0.5)
    minus = np.zeros(4)
    minus[1], minus[2] = math.sqrt(0.5), -math.sqrt(0.5)
    return _power([(0.0, np.diag([1.0, 0, 0, 1.0]).astype(np.complex128)),
                   (0.5, _proj(plus)), (-0.5, _proj(minus))], t, s)


def _swap_pow(t, s=0.0):
    anti = np.zeros(4)
    anti[1], anti[2] = math.sqrt(0.5), -math.sqrt(0.5)
    pa = _proj(anti)
    return _power([(0.0, np.eye(4) - pa), (1.0, pa)], t, s)


def _phased_iswap(p, t):
    # exp(-i pi p) on q0 = 1, exp(i pi p) on q1 = 1, around ISWAP^t.
    d = np.diag(np.exp(1j * math.pi * p * np.array([0, -1, 1, 0])))
    return d @ _iswap_pow(t) @ d.conj().T


def _fsim(theta, phi):
    c, s = math.cos(theta), math.sin(theta)
    return np.array([[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0],
                     [0, 0, 0, np.exp(-1j * phi)]], dtype=np.complex128)


def _diagonal(angles, k):
    """Diagonal gate; angles in Cirq's big-endian order (first qubit most
    significant), missing angles 0."""
    a = list(angles) + [0.0] * ((1 << k) - len(angles))
    d = np.empty(1 << k, dtype=np.complex128)
    for i in range(1 << k):
        big = sum(((i >> j) & 1) << (k - 1 - j) for j in range(k))
        d[i] = np.exp(1j * a[big])
    return np.diag(d)


def _cswap():
    m = np.zeros((8, 8), dtype=np.complex128)
    for i in range(8):
        j = i
        if i & 1:  # control (first qubit) set: exchange bits 1 and 2
            j = (i & 1) | ((i >> 1 & 1) << 2) | ((i >> 2 & 1) << 1)
        m[j, i] = 1
    return m


def gate_matrix(kind: int, nq: int, params: Dict[str, float]) -> np.ndarray:
    """Matrix of a Cirq gate kind on `nq` listed qubits (bit j <-> j-th
    qubit), as lib/gates_cirq.h's Create functions build it."""
    k = GateKind(kind)

    def e():
        return params["exponent"]

    def gs():
        return params["global_shift"]

    if k in (GateKind.kI1, GateKind.kI2, GateKind.kI):
        return np.eye(1 << nq, dtype=np.complex128)
    if k == GateKind.kXPowGate:
        return _xpow(e(), gs())
    if k == GateKind.kYPowGate:
        return _pauli_pow(_Y, e(), gs())
    if k == GateKind.kZPowGate:
        return _zpow(e(), gs())
    if k == GateKind.kHPowGate:
        return _pauli_pow(_HM, e(), gs())
    if k == GateKind.kCZPowGate:
        return _cpow(_P1, e(), gs(), 1)
    if k == GateKind.kCXPowGate:
        return _cpow((_I - _X) / 2, e(), gs(), 1)
    if k == GateKind.krx:
        return _xpow(params["phi"] / math.pi, -0.5)
    if k == GateKind.kry:
        return _pauli_pow(_Y, params["phi"] / math.pi, -0.5)
    if k == GateKind.krz:
        return _zpow(params["phi"] / math.pi, -0.5)
    if k == GateKind.kH:
        return _HM.copy()
    if k == GateKind.kS:
        return _zpow(0.5)
    if k == GateKind.kT:
        return _zpow(0.25)
    if k == GateKind.kX:
        return _X.copy()
    if k == GateKind.kY:
        return _Y.copy()
    if k == GateKind.kZ:
        return _Z.copy()
    if k == GateKind.kCZ:
        return _cpow(_P1, 1.0, 0.0, 1)
    if k == GateKind.kCX:
        return _cpow((_I - _X) / 2, 1.0, 0.0, 1)
    if k == GateKind.kPhasedXPowGate:
        p = params["phase_exponent"]
        return _zpow(p) @ _xpow(e(), gs()) @ _zpow(-p)
    if k == GateKind.kPhasedXZGate:
        a = params["axis_phase_exponent"]
        return (_zpow(params["z_exponent"]) @ _zpow(a)
                @ _xpow(params["x_exponent"]) @ _zpow(-a))
    if k in (GateKind.kXXPowGate, GateKind.kYYPowGate, GateKind.kZZPowGate):
        p = {GateKind.kXXPowGate: _X, GateKind.kYYPowGate: _Y,
             GateKind.kZZPowGate: _Z}[k]
        return _pauli_pow(_kron(p, p), e(), gs())
    if k in (GateKind.kXX, GateKind.kYY, GateKind.kZZ):
        p = {GateKind.kXX: _X, GateKind.kYY: _Y, GateKind.kZZ: _Z}[k]
        return _kron(p, p)
    if k == GateKind.kSwapPowGate:
        return _swap_pow(e(), gs())
    if k == GateKind.kISwapPowGate:
        return _iswap_pow(e(), gs())
    if k == GateKind.kriswap:
        return _iswap_pow(2 * params["phi"] / math.pi)
    if k == GateKind.kSWAP:
        return _swap_pow(1.0)
    if k == GateKind.kISWAP:
        return _iswap_pow(1.0)
    if k == GateKind.kPhasedISwapPowGate:
        return _phased_iswap(params["phase_exponent"], e())
    if k == GateKind.kgivens:
        return _phased_iswap(0.25, 2 * params["phi"] / math.pi)
    if k == GateKind.kFSimGate:
        return _fsim(params["theta"], params["phi"])
    if k == GateKind.kCCZPowGate:
        return _cpow(_P1, e(), gs(), 2)
    if k == GateKind.kCCXPowGate:
        return _cpow((_I - _X) / 2, e(), gs(), 2)
    if k == GateKind.kCSwapGate:
        return _cswap()
    if k == GateKind.kCCZ:
        return _cpow(_P1, 1.0, 0.0, 2)
    if k == GateKind.kCCX:
        return _cpow((_I - _X) / 2, 1.0, 0.0, 2)
    raise ValueError("GateKind not supported.")


_NQ = {GateKind.kI1: 1, GateKind.kI2: 2, GateKind.kCZPowGate: 2,
       GateKind.kCXPowGate: 2, GateKind.kCZ: 2, GateKind.kCX: 2,
       GateKind.kXXPowGate: 2, GateKind.kYYPowGate: 2, GateKind.kZZPowGate: 2,
       GateKind.kXX: 2, GateKind.kYY: 2, GateKind.kZZ: 2,
       GateKind.kSwapPowGate: 2, GateKind.kISwapPowGate: 2,
       GateKind.kriswap: 2, GateKind.kSWAP: 2, GateKind.kISWAP: 2,
       GateKind.kPhasedISwapPowGate: 2, GateKind.kgivens: 2,
       GateKind.kFSimGate: 2, GateKind.kCCZPowGate: 3,
       GateKind.kCCXPowGate: 3, GateKind.kCSwapGate: 3, GateKind.kCCZ: 3,
       GateKind.kCCX: 3}

# ------------------------------------------------------------- circuits --


class Circuit:
    """Circuit<Operation<float>> of the reference module: ``num_qubits`` and
    the operations in order (each a dict: "kind" 0 gate / 1 controlled /
    2 measurement, "time", "qs" as listed, "m" with bit j <-> qs[j],
    "cqs", "cvals")."""

    def __init__(self):
        self.num_qubits = 0
        self.ops: List[dict] = []


class OpString:
    """OpString<float> (lib/expect.h): ``weight`` times the product of its
    gates."""

    def __init__(self):
        self.weight = 1.0 + 0.0j
        self.ops: List[dict] = []


def _gate(kind, time, qubits, params):
    qs = [int(q) for q in qubits]
    k = GateKind(kind)
    if k in (GateKind.kMatrixGate1, GateKind.kMatrixGate2, GateKind.kMatrixGate,
             GateKind.kTwoQubitDiagonalGate, GateKind.kThreeQubitDiagonalGate,
             GateKind.kGlobalPhaseGate):
        raise ValueError("GateKind not supported.")
    want = _NQ.get(k, 0 if k == GateKind.kI else 1)
    if want and len(qs) != want:
        raise ValueError(f"{k.name} acts on {want} qubits")
    ps = {str(a): float(v) for a, v in params.items()}
    return dict(kind=0, time=int(time), qs=qs, m=gate_matrix(k, len(qs), ps),
                cqs=[], cvals=0, gate=k, params=ps)


def _matrix_gate(time, qubits, matrix):
    qs = [int(q) for q in qubits]
    m = np.asarray(matrix, dtype=np.float64)
    if len(qs) == 0:
        # Global phase gate: matrix = (cos, sin) of the phase.
        return dict(kind=0, time=int(time), qs=[], cqs=[], cvals=0,
                    m=np.array([[m[0] + 1j * m[1]]]))
    if len(qs) > 6:
        raise ValueError("Only up to 6-qubit matrix gates are supported.")
    d = 1 << len(qs)
    c = (m[0::2] + 1j * m[1::2]).reshape(d, d)
    # Cirq's order: the first listed qubit is the most significant bit.
    return dict(kind=0, time=int(time), qs=qs[::-1], m=c, cqs=[], cvals=0)


def add_gate(gate_kind, time, qubits, params, circuit: Circuit) -> None:
    circuit.ops.append(_gate(gate_kind, time, qubits, params))


def add_diagonal_gate(time, qubits, angles, circuit: Circuit) -> None:
    qs = [int(q) for q in qubits]
    if len(qs) not in (2, 3):
        raise ValueError("Only 2- or 3-qubit diagonal gates are supported.")
    circuit.ops.append(dict(kind=0, time=int(time), qs=qs, cqs=[], cvals=0,
                            m=_diagonal([float(a) for a in angles], len(qs))))


def add_matrix_gate(time, qubits, matrix, circuit: Circuit) -> None:
    circuit.ops.append(_matrix_gate(time, qubits, matrix))


def add_measurement(time, qubits, circuit: Circuit) -> None:
    circuit.ops.append(dict(kind=2, time=int(time), qs=[int(q) for q in qubits],
                            m=None, cqs=[], cvals=0))


def control_last_gate(qubits, values, circuit: Circuit) -> None:
    """Gate::ControlledBy(qubits, values): value i belongs to qubits[i]
    (lib/gate.h:106-146)."""
    op = circuit.ops[-1]
    if op["kind"] != 0:
        raise ValueError("the last operation is not a gate")
    cv = 0
    for i, v in enumerate(values):
        cv |= (int(v) & 1) << i
    op.update(kind=1, cqs=[int(q) for q in qubits], cvals=cv)


def add_channel(time, qubits, prob_matrix_unitary_triples,
                circuit: Circuit) -> None:
    """A noisy-circuit channel (pybind_main.cpp add_channel): Kraus
    operators given as (lower-bound probability, matrix in Cirq's qubit
    order, is unitary)."""
    kops = []
    cqs = None
    for prob, mat, unitary in prob_matrix_unitary_triples:
        g = _matrix_gate(time, qubits, mat)
        qs, m = _sorted(g["qs"], g["m"])
        cqs = qs
        kops.append((bool(unitary), float(prob), m))
    circuit.ops.append(dict(kind=3, time=int(time), qs=cqs or [], kops=kops,
                            m=None, cqs=[], cvals=0))


def add_gate_to_opstring(gate_kind, qubits, opstring: OpString) -> None:
    opstring.ops.append(_gate(gate_kind, 0, qubits, {}))


def add_matrix_gate_to_opstring(qubits, matrix, opstring: OpString) -> None:
    opstring.ops.append(_matrix_gate(0, qubits, matrix))

# ----------------------------------------------------------- simulation --


def _ctx():
    from .api import default_context
    return default_context()


def _sorted(qs, m):
    """Qubits ascending with the matrix permuted to match (bit j <-> qs[j])."""
    qs = list(qs)
    order = sorted(range(len(qs)), key=lambda j: qs[j])
    if order == list(range(len(qs))):
        return qs, m
    k = len(qs)
    pos = [0] * k
    for new, old in enumerate(order):
        pos[old] = new
    d = 1 << k
    perm = np.array([sum(((i >> j) & 1) << pos[j] for j in range(k))
                     for i in range(d)])
    out = np.empty_like(m)
    out[np.ix_(perm, perm)] = m
    return [qs[j] for j in order], out


def _engine_circuit(num_qubits, ops):
    from . import engine as E
    c = E.Circuit(num_qubits)
    for o in ops:
        if o["kind"] == 2:
            c.add_measurement(o["time"], o["qs"])
        elif o["kind"] == 1:
            c.add_controlled_gate(o["time"], o["qs"], o["cqs"], o["cvals"], o["m"])
        else:
            c.add_gate(o["time"], o["qs"], o["m"])
    return c


def _noisy_circuit(num_qubits, ops):
    """The engine's noisy circuit: runs of gates appended as circuits, each
    channel as a general Kraus channel."""
    from . import engine as E
    nc = E.NoisyCircuit(num_qubits)
    run = []
    for o in list(ops) + [None]:
        if o is not None and o["kind"] != 3:
            run.append(o)
            continue
        if run:
            nc.append(_engine_circuit(num_qubits, run))
            run = []
        if o is not None:
            nc.add_kraus_channel(o["time"], o["qs"], o["kops"])
    return nc


def _max_fused(options):
    return max(1, min(6, int(options.get("f", 2))))


def _bitstrings(text: str, n: int) -> List[int]:
    """BitstringsFromStream (lib/bitstring.h:37-66): one bitstring per line,
    its first character is qubit 0."""
    out = []
    for line in text.split("\n"):
        if not line:
            continue
        p, b = 0, 0
        while p < min(len(line), 128) and line[p] in "01":
            b |= (ord(line[p]) - 48) << p
            p += 1
        if p != n:
            raise ValueError(f"wrong bitstring length: got {p}; should be {n}.")
        out.append(b)
    return out


def _embed(m, gqs, qs):
    """Matrix of a gate on `gqs` (bit j <-> gqs[j]) on the qubits `qs`
    (sorted, bit j <-> qs[j])."""
    u, k = len(qs), len(gqs)
    pos = [qs.index(q) for q in gqs]
    d = 1 << u
    out = np.zeros((d, d), dtype=np.complex128)
    mask = sum(1 << p for p in pos)
    for col in range(d):
        sub = sum(((col >> p) & 1) << j for j, p in enumerate(pos))
        base = col & ~mask
        for r in range(1 << k):
            row = base | sum(((r >> j) & 1) << p for j, p in enumerate(pos))
            out[row, col] = m[r, sub]
    return out


class _Run:
    """SimulatorHelper (pybind_main.cpp): one state, the circuit run from an
    input state with measurements drawn from mt19937(seed), seed + 1 after
    every run."""

    def __init__(self, options):
        from . import api
        self.circuit: Circuit = options["c"]
        self.n = self.circuit.num_qubits
        self.f = _max_fused(options)
        self.seed = int(options.get("s", 0))
        self.ctx = _ctx()
        self.ss = api.StateSpace(ctx=self.ctx)
        self.sim = api.Simulator(ctx=self.ctx)
        self.state = self.ss.Create(self.n)

    def init(self, input_state):
        if isinstance(input_state, (int, np.integer)):
            self.ss.SetAllZeros(self.state)
            self.ss.SetAmpl(self.state, int(input_state), 1.0, 0.0)
        else:
            v = np.asarray(input_state, dtype=np.float32)
            self.ss.from_numpy(v[: 2 << self.n].view(np.complex64), self.state)

    def run_ops(self, ops):
        from . import engine as E
        bits = []
        if ops:
            plan = E.Plan(_engine_circuit(self.n, ops), max_fused_size=self.f)
            bits = plan.run(self.ctx, self.state, seed=self.seed)
        self.seed += 1
        return bits

    def run_noisy(self, ops, from_state=True, collect_mea_stat=False):
        """QuantumTrajectorySimulator::RunOnce with repetition = seed on the
        current state (from_state) or from |0..0>; returns its stats."""
        from . import engine as E
        stats = np.zeros(0, dtype=np.uint64)
        if ops:
            traj = E.Trajectories(_noisy_circuit(self.n, ops),
                                  max_fused_size=self.f, collect_kop_stat=False,
                                  collect_mea_stat=collect_mea_stat)
            if from_state:
                stats = traj.run_from(self.ctx, self.state, self.seed)
            else:
                stats = traj.run(self.ctx, self.state, self.seed)
        self.seed += 1
        return stats

    def expectation_values(self, opsums_and_qubit_counts):
        out = []
        for opsum, count in opsums_and_qubit_counts:
            if count == 0:
                out.append(complex(sum(complex(s.weight) for s in opsum)))
                continue
            total = 0j
            for s in opsum:
                total += complex(s.weight) * self._opstring_ev(s, count)
            out.append(total)
        return out

    def _opstring_ev(self, s: OpString, count: int) -> complex:
        qs = sorted({q for o in s.ops for q in o["qs"]})
        if not qs:
            return 1.0 + 0j
        if count <= 6 and len(qs) <= 6:
            m = np.eye(1 << len(qs), dtype=np.complex128)
            for o in s.ops:
                m = _embed(o["m"], o["qs"], qs) @ m
            m32 = np.ascontiguousarray(m.astype(np.complex64)).view(np.float32)
            return complex(self.sim.ExpectationValue(qs, m32, self.state))
        scratch = self.ss.Create(self.n)
        self.ss.Copy(self.state, scratch)
        for o in s.ops:
            gq, gm = _sorted(o["qs"], o["m"])
            self.sim.ApplyGate(gq, np.ascontiguousarray(
                gm.astype(np.complex64)).view(np.float32), scratch)
        return complex(self.ss.InnerProduct(self.state, scratch))


def qsim_simulate(options) -> List[complex]:
    """Amplitudes of the bitstrings options["i"] after the circuit from
    |0...0> (QSimRunner::Run with a measure callback)."""
    r = _Run(options)
    bits = _bitstrings(options["i"], r.n)
    r.ss.SetStateZero(r.state)
    r.run_ops(r.circuit.ops)
    amps = r.ss.to_numpy(r.state)
    return [complex(amps[b]) for b in bits]


def qsim_simulate_fullstate(options, input_state=0) -> np.ndarray:
    """Final state (interleaved float32, normal order) from a basis state
    (int) or a state vector (float32 array)."""
    r = _Run(options)
    r.init(input_state)
    r.run_ops(r.circuit.ops)
    amps = np.ascontiguousarray(r.ss.to_numpy(r.state), dtype=np.complex64)
    return amps.view(np.float32).copy()


def qsim_sample_final(options, num_samples: int) -> List[int]:
    """StateSpace::Sample of the final state (seed s + 1: the run used s)."""
    r = _Run(options)
    r.init(0)
    r.run_ops(r.circuit.ops)
    return [int(x) for x in r.ss.Sample(r.state, int(num_samples), r.seed)]


def qsim_sample(options) -> List[int]:
    """Measurement results of the circuit's measurement gates, one bit per
    measured qubit in the gates' qubit order, concatenated."""
    r = _Run(options)
    r.ss.SetStateZero(r.state)
    bits = r.run_ops(r.circuit.ops)
    out = []
    meas = [o for o in r.circuit.ops if o["kind"] == 2]
    for o, b in zip(meas, bits):
        out.extend(int((int(b) >> q) & 1) for q in o["qs"])
    return out


def qsim_simulate_expectation_values(options, opsums_and_qubit_counts,
                                     input_state=0) -> List[complex]:
    """Expectation values of the opsums on the final state."""
    r = _Run(options)
    r.init(input_state)
    r.run_ops(r.circuit.ops)
    return r.expectation_values(opsums_and_qubit_counts)


def qsim_simulate_moment_expectation_values(options, opsums_and_qubit_counts,
                                            input_state=0):
    """Expectation values after parts of the circuit: entry (end, opsums) is
    evaluated after ops [previous end, end)."""
    r = _Run(options)
    r.init(input_state)
    out, begin = [], 0
    for end, counts in opsums_and_qubit_counts:
        r.run_ops(r.circuit.ops[begin:int(end)])
        out.append(r.expectation_values(counts))
        begin = int(end)
    return out


# -------------------------------------------------- noisy circuits -------


def qtrajectory_simulate(options) -> List[complex]:
    """Amplitudes of the bitstrings options["i"] after one trajectory
    (repetition s) of the noisy circuit from |0...0>."""
    r = _Run(options)
    bits = _bitstrings(options["i"], r.n)
    r.run_noisy(r.circuit.ops, from_state=False)
    amps = r.ss.to_numpy(r.state)
    return [complex(amps[b]) for b in bits]


def qtrajectory_simulate_fullstate(options, input_state=0) -> np.ndarray:
    """Final state of one trajectory (repetition s) from the input state."""
    r = _Run(options)
    r.init(input_state)
    r.run_noisy(r.circuit.ops)
    amps = np.ascontiguousarray(r.ss.to_numpy(r.state), dtype=np.complex64)
    return amps.view(np.float32).copy()


def qtrajectory_sample_final(options, num_samples: int) -> List[int]:
    """Samples of the final state of one trajectory (seed s + 1)."""
    r = _Run(options)
    r.init(0)
    r.run_noisy(r.circuit.ops)
    return [int(x) for x in r.ss.Sample(r.state, int(num_samples), r.seed)]


def qtrajectory_sample(options) -> List[int]:
    """Measurement results of one trajectory (repetition s), one bit per
    measured qubit in the gates' qubit order, concatenated."""
    from . import engine as E
    r = _Run(options)
    stats = r.run_noisy(r.circuit.ops, from_state=False, collect_mea_stat=True)
    vals = E.Trajectories.samples(stats)
    out = []
    meas = [o for o in r.circuit.ops if o["kind"] == 2]
    for o, v in zip(meas, vals):
        out.extend(int((int(v) >> q) & 1) for q in o["qs"])
    return out


def qtrajectory_simulate_expectation_values(options, opsums_and_qubit_counts,
                                            input_state=0) -> List[complex]:
    """Expectation values averaged over options["r"] trajectories
    (repetitions s, s + 1, ...), each from the input state."""
    r = _Run(options)
    reps = int(options["r"])
    acc = np.zeros(len(opsums_and_qubit_counts), dtype=np.complex128)
    for _ in range(reps):
        r.init(input_state)
        r.run_noisy(r.circuit.ops)
        acc += np.array(r.expectation_values(opsums_and_qubit_counts))
    return [complex(x) for x in acc / reps]


def qtrajectory_simulate_moment_expectation_values(
        options, opsums_and_qubit_counts, input_state=0):
    """Moment expectation values averaged over options["r"] trajectories."""
    r = _Run(options)
    reps = int(options["r"])
    acc = [np.zeros(len(c), dtype=np.complex128) for _, c in opsums_and_qubit_counts]
    for _ in range(reps):
        r.init(input_state)
        begin = 0
        for i, (end, counts) in enumerate(opsums_and_qubit_counts):
            r.run_noisy(r.circuit.ops[begin:int(end)])
            acc[i] += np.array(r.expectation_values(counts))
            begin = int(end)
    return [[complex(x) for x in a / reps] for a in acc]


# ------------------------------------------------------------------ qsimh --

_H = 0.5
_IS2 = math.sqrt(0.5)
_C = 0.5 + 0.5j
# First Schmidt factor (on the gate's first listed qubit) of the Cirq
# two-qubit gates, as lib/gates_cirq.h's SchmidtDecomp functions choose
# them: a path of the hybrid simulator picks one term per gate on the cut,
# so partial sums over fixed prefix bits equal the reference's only with the
# same terms.  The second factors follow from the gate matrix (projection
# onto these mutually orthogonal first factors).
_FIRST = {
    GateKind.kI2: [_I],
    GateKind.kCZPowGate: [_P0, _P1], GateKind.kCZ: [_P0, _P1],
    GateKind.kCXPowGate: [_P0, _P1], GateKind.kCX: [_P0, _P1],
    GateKind.kXXPowGate: [_I, _X], GateKind.kYYPowGate: [_I, _Y],
    GateKind.kZZPowGate: [_I, _Z],
    GateKind.kXX: [_X], GateKind.kYY: [_Y], GateKind.kZZ: [_Z],
    GateKind.kSwapPowGate: [_H * _I, _H * _X, _H * _Y, _H * _Z],
    GateKind.kISwapPowGate: [_H * _I, _H * _X, _H * _Y, _H * _Z],
    GateKind.kriswap: [_H * _I, _H * _X, _H * _Y, _H * _Z],
    GateKind.kPhasedISwapPowGate: [_H * _I, _H * _X, _H * _Y, _H * _Z],
    GateKind.kgivens: [_H * _I, _H * _X, _H * _Y, _H * _Z],
    GateKind.kSWAP: [_IS2 * _I, _IS2 * _X, _IS2 * _Y, _IS2 * _Z],
    GateKind.kISWAP: [_IS2 * _I, _C * _X, _C * _Y, _IS2 * _Z],
}


def _schmidt_terms(kind, m):
    """[(A_k, B_k)] with A_k on the first listed qubit (bit 0 of m)."""
    terms = []
    u = m.reshape(2, 2, 2, 2)          # [b, a, b', a'] for index a + 2 b
    for a in _FIRST[kind]:
        b = np.einsum("xy,bxcy->bc", a.conj(), u) / np.sum(np.abs(a) ** 2)
        terms.append((a, b))
    return terms


def _hybrid_circuit(c: Circuit):
    """The engine circuit of a qsimh run: gates only; two-qubit Cirq gates
    carry the reference's Schmidt terms (fSim as the engine's named fs
    gate, whose terms are the same)."""
    from . import engine as E
    ec = E.Circuit(c.num_qubits)
    i = 0
    for o in c.ops:
        if o["kind"] != 0:
            raise ValueError("measurement, controlled or other non-matrix "
                             "gates are not supported by qsimh.")
        k = o.get("gate")
        if len(o["qs"]) == 2 and k == GateKind.kFSimGate:
            ec.add_named(o["time"], "fs", o["qs"],
                         (o["params"]["theta"], o["params"]["phi"]))
        else:
            ec.add_gate(o["time"], o["qs"], o["m"])
            if len(o["qs"]) == 2 and k in _FIRST:
                terms = _schmidt_terms(k, o["m"])
                if o["qs"][0] > o["qs"][1]:      # engine: A on the lower qubit
                    terms = [(b, a) for a, b in terms]
                ec.set_schmidt(i, terms)
        i += 1
    return ec


def qsimh_simulate(options) -> List[complex]:
    """Amplitudes of the bitstrings options["i"] by the hybrid simulator
    (pybind_main.cpp qsimh_simulate): options["k"] lists the qubits of part
    1, "w" the prefix, "p" and "r" the numbers of prefix and root gates on
    the cut.  Errors are printed and give an empty list, as the reference's
    module does."""
    import sys
    from . import hybrid
    from ._native import QsgError
    c: Circuit = options["c"]
    n = c.num_qubits
    try:
        bits = _bitstrings(options["i"], n)
        parts = [0] * n
        for q in options["k"]:
            if int(q) >= n:
                raise ValueError("Invalid arguments are provided for arg k.")
            parts[int(q)] = 1
        amps, _ = hybrid.run(_ctx(), _hybrid_circuit(c), parts, bits,
                             prefix=int(options["w"]),
                             num_prefix_gatexs=int(options["p"]),
                             num_root_gatexs=int(options["r"]),
                             max_fused_size=_max_fused(options))
    except (QsgError, ValueError) as e:
        print(e, file=sys.stderr)
        return []
    return [complex(np.complex64(a)) for a in amps]
