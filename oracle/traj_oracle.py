"""TEST INFRASTRUCTURE ONLY: CPU restatement of quantum trajectories.

Restates, in FP64 and without fusion, the noise channels of
lib/channels_cirq.h and the Kraus-operator sampling of
QuantumTrajectorySimulator::RunIteration (lib/qtrajectory.h:240-387):

* one std::mt19937(rep) per repetition and one
  uniform_real_distribution<double>(0, 1) draw per operation (a measurement
  draws uniform(0, norm) inside StateSpace::VirtualMeasure,
  lib/statespace.h:97-140);
* a channel first walks its Kraus operators with the lower-bound
  probabilities (:305-327); if none is chosen, the state is normalised when a
  non-unitary operator was applied since the last normalisation, and each
  non-unitary operator's probability becomes <psi|K^dagger K|psi> (:331-380),
  falling back to the most probable one when round-off leaves r above the
  total;
* measurements normalise first when needed (:278-283), and the final state
  is normalised when the last applied operators were not all unitary.

Deferring operators, as the reference does, changes only when they are
applied, not the state that any decision sees, so the ops are applied as
they come.  Used by tests/ only, as the checker of the GPU engine; it is
itself pinned against the reference's own trajectory outputs
(tests/golden/traj_*.npz).  Linear-algebra primitives and the RNG come from
oracle/qsim_oracle.c through the `orc` object of tests/conftest.py.
"""
from __future__ import annotations

import math

import numpy as np

PX = np.array([[0, 1], [1, 0]], np.complex128)
PY = np.array([[0, -1j], [1j, 0]], np.complex128)
PZ = np.array([[1, 0], [0, -1]], np.complex128)


def _f32(x):
    return float(np.float32(x))


def channel_kops(code: int, q: int, p: float, fp32: bool = True, qs=None):
    """Kraus operators of a one-qubit channel of lib/channels_cirq.h as
    (unitary, prob, [(qubits, matrix)], kd_k diagonal or None).  With fp32,
    matrix and kd_k entries hold the single-precision values of the
    reference's float channels, else those of its double channels.  Code 6:
    the reference's multi-qubit depolarizing factory on the channel qubits
    `qs` (:147-189), whose Pauli of index digit j acts on register qubit j."""
    rnd = np.float32 if fp32 else np.float64
    if code == 6:
        k = len(qs)
        p1, p2 = 1 - p, p / 3
        out = []
        for i in range(4 ** k):
            prob, ops = 1.0, []
            for j in range(k):
                pauli = (i >> (2 * j)) & 3
                if pauli == 0:
                    prob *= p1
                else:
                    prob *= p2
                    ops.append(([j], (PX, PY, PZ)[pauli - 1]))
            out.append((True, prob, ops, None))
        return out
    if code == 0:  # depolarizing, :127-199
        p1, p2 = 1 - p, p / 3
        return [(True, p1, [], None), (True, p2, [([q], PX)], None),
                (True, p2, [([q], PY)], None), (True, p2, [([q], PZ)], None)]
    if code in (1, 2):  # amplitude / phase damping, :274-345
        p1 = 1 - p
        r, s = rnd(math.sqrt(p1)), rnd(math.sqrt(p))
        k0 = np.array([[1, 0], [0, r]], np.complex128)
        if code == 1:
            k1 = np.array([[0, s], [0, 0]], np.complex128)
        else:
            k1 = np.array([[0, 0], [0, s]], np.complex128)
        return [(False, p1, [([q], k0)], [1.0, float(r * r)]),
                (False, 0.0, [([q], k1)], [0.0, float(s * s)])]
    if code == 3:  # bit flip, :425-447
        return [(True, 1 - p, [], None), (True, p, [([q], PX)], None)]
    if code == 4:  # phase flip, :393-415
        return [(True, 1 - p, [], None), (True, p, [([q], PZ)], None)]
    if code == 5:  # reset, :359-380
        return [(False, 0.0, [([q], np.array([[1, 0], [0, 0]], np.complex128))],
                 [1.0, 0.0]),
                (False, 0.0, [([q], np.array([[0, 1], [0, 0]], np.complex128))],
                 [0.0, 1.0])]
    raise ValueError(code)


def _normalize(orc, s, n):
    a = 1.0 / math.sqrt(orc.norm(s, n))
    s *= a


def run_trajectory(orc, n: int, ops, rep: int,
                   normalize_before_mea_gates: bool = True, fp32: bool = True):
    """ops: list of dicts, either gates {"kind": 0|1|2, qs, cqs, cvals, m}
    or channels {"channel": code, "q": q, "p": p}.  Returns (final state,
    stat samples).  `fp32` selects the channel constants (channel_kops)."""
    s = orc.zero_state(n)
    g = orc.mt(rep & 0xFFFFFFFF)
    unitary = True
    stats = []
    for op in ops:
        if "channel" not in op and op["kind"] == 2:
            if not unitary and normalize_before_mea_gates:
                _normalize(orc, s, n)
                unitary = True
            mask = 0
            for q in op["qs"]:
                mask |= 1 << q
            norm = orc.norm(s, n)
            r = orc.L.orc_uniform(g, norm)
            bits = orc.find_index(s, n, r) & mask
            orc.collapse(s, n, mask, bits)
            stats.append(bits)
            continue
        r = orc.L.orc_canonical(g)
        if "channel" not in op:
            if op["kind"] == 0:
                orc.apply_gate(s, n, op["qs"], op["m"])
            else:
                orc.apply_controlled_gate(s, n, op["qs"], op["cqs"],
                                          op["cvals"], op["m"])
            stats.append(0)
            continue
        kops = channel_kops(op["channel"], op["q"], op["p"], fp32,
                            op.get("qs"))
        cp = 0.0
        chosen = None
        for i, (uni, prob, kops_ops, _) in enumerate(kops):
            cp += prob
            if r < cp:
                chosen = i
                unitary = unitary and uni
                break
        if chosen is None:
            if not unitary:
                _normalize(orc, s, n)
                unitary = True
            max_prob, max_index = 0.0, 0
            for i, (uni, prob, kops_ops, kd) in enumerate(kops):
                if uni:
                    continue
                ev = orc.expectation_value(s, n, [op["q"]], np.diag(kd)).real
                if ev > max_prob:
                    max_prob, max_index = ev, i
                cp += ev - prob
                if r < cp or i == len(kops) - 1:
                    chosen = i if r < cp else max_index
                    unitary = False
                    break
        if chosen is None:
            continue
        for qs, m in kops[chosen][2]:
            orc.apply_gate(s, n, qs, m)
        stats.append(chosen)
    if not unitary:
        _normalize(orc, s, n)
    return s, stats


def ops_from_fixture(d, unpack_ops):
    """The op list of a tests/golden/traj_*.npz fixture."""
    gates = iter(unpack_ops(d))
    ops = []
    qmask = d["op_qmask"] if "op_qmask" in d else np.zeros(len(d["op_q"]))
    for code, q, p, qm in zip(d["op_channel"], d["op_q"], d["op_p"], qmask):
        if code < 0:
            ops.append(next(gates))
        else:
            qs = [b for b in range(64) if (int(qm) >> b) & 1] or [int(q)]
            ops.append(dict(channel=int(code), q=int(q), p=float(p), qs=qs))
    return ops
