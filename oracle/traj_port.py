"""TEST INFRASTRUCTURE ONLY: the timed CPU baseline of the batched noisy
trajectories ("port" of the reference's CPU trajectory simulator).

Restates QuantumTrajectorySimulator::RunIteration
(lib/qtrajectory.h:240-387) in FP32 on the host cores, the shape the
reference runs on its CPU simulators:

* one std::mt19937(rep) and one uniform_real_distribution<double>(0, 1) draw
  per operation (oracle/qsim_oracle.c orc_canonical);
* gates and chosen Kraus operators are deferred and applied fused when the
  state is needed (ApplyDeferredOps, :417-447).  The reference fuses the
  deferred list with its fuser at max_fused_size 2 by default
  (QuantumTrajectorySimulator::Parameter derives from the fuser's
  Parameter); here every one-qubit operator is folded into the next
  two-qubit gate on its qubit (one pass per two-qubit gate, the rest
  flushed when the state is needed);
* a channel first walks its Kraus operators with their lower-bound
  probabilities (:305-327); when none is chosen it applies the deferred
  operators, normalises if a non-unitary operator was applied (a Norm and a
  Multiply pass), and computes <psi|K^dagger K|psi> for each non-unitary
  operator (one pass each, :331-380);
* the final state is normalised when the last operators were non-unitary.

Gate passes use orc_port_apply_gate_f32 (the lane-batched restatement of the
reference's SIMD simulators); norms, expectation values and scaling use the
oracle's FP32-state reductions.  Channel constants follow
oracle/traj_oracle.py (lib/channels_cirq.h).  Only bench.py's CPU-baseline
leg and tests/ use this file.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from traj_oracle import channel_kops

P = C.POINTER


def noisy_ops(clean_ops, n, p_depol, gamma, cycle_len=2):
    """The engine's MakeNoisy rule (lib/circuit_noisy.h:33-64: a
    depolarizing channel on every qubit of every operation; plus amplitude
    damping on every qubit after each cycle of `cycle_len` time steps):
    a list of gates {"qs", "m"} and channels {"channel", "q", "p"}."""
    ops = []
    for i, o in enumerate(clean_ops):
        t = o["time"]
        ops.append(dict(qs=list(o["qs"]), m=np.asarray(o["m"], np.complex128)))
        if p_depol > 0:
            for q in list(o["qs"]) + list(o.get("cqs", [])):
                ops.append(dict(channel=0, q=int(q), p=p_depol))
        last = (i + 1 == len(clean_ops)
                or clean_ops[i + 1]["time"] // cycle_len != t // cycle_len)
        if gamma > 0 and last:
            for q in range(n):
                ops.append(dict(channel=1, q=q, p=gamma))
    return ops


class TrajectoryPort:
    """One n-qubit FP32 host state and the reference's trajectory loop."""

    def __init__(self, lib, n: int):
        self.L = lib
        self.n = n
        self.s = np.zeros(2 << n, np.float32)
        self.sp = self.s.ctypes.data_as(P(C.c_float))
        lib.orc_port_apply_gate_f32.argtypes = [P(C.c_float), C.c_uint,
                                                P(C.c_uint), C.c_uint,
                                                P(C.c_float)]
        lib.orc_port_norm_f32.restype = C.c_double
        lib.orc_port_norm_f32.argtypes = [P(C.c_float), C.c_uint]
        lib.orc_port_scale_f32.argtypes = [P(C.c_float), C.c_uint, C.c_float]
        lib.orc_port_diag1_ev_f32.restype = C.c_double
        lib.orc_port_diag1_ev_f32.argtypes = [P(C.c_float), C.c_uint, C.c_uint,
                                              C.c_double, C.c_double]
        lib.orc_canonical.restype = C.c_double
        lib.orc_canonical.argtypes = [C.c_void_p]
        lib.orc_mt_seed.argtypes = [C.c_void_p, C.c_uint32]
        lib.orc_mt_size.restype = C.c_size_t
        self.g = C.create_string_buffer(lib.orc_mt_size())
        self.pending = {}

    def _apply(self, qs, m):
        m32 = np.ascontiguousarray(np.asarray(m, np.complex64)).view(np.float32)
        qa = (C.c_uint * max(1, len(qs)))(*qs)
        self.L.orc_port_apply_gate_f32(self.sp, self.n, qa, len(qs),
                                       m32.ctypes.data_as(P(C.c_float)))

    def _defer(self, qs, m):
        if len(qs) == 1:
            q = qs[0]
            self.pending[q] = m @ self.pending[q] if q in self.pending else m
        elif len(qs) == 2:
            a, b = qs
            pa = self.pending.pop(a, np.eye(2))
            pb = self.pending.pop(b, np.eye(2))
            self._apply(qs, m @ np.kron(pb, pa))
        else:
            for q in qs:
                if q in self.pending:
                    self._apply([q], self.pending.pop(q))
            self._apply(qs, m)

    def _flush(self):
        for q in sorted(self.pending):
            self._apply([q], self.pending[q])
        self.pending.clear()

    def _normalize(self):
        nrm = self.L.orc_port_norm_f32(self.sp, self.n)
        self.L.orc_port_scale_f32(self.sp, self.n, 1.0 / math.sqrt(nrm))

    def run(self, ops, rep: int) -> list:
        """One trajectory from |0...0>; returns the Kraus-operator indices
        chosen at the channels."""
        self.s[:] = 0
        self.s[0] = 1
        self.pending.clear()
        self.L.orc_mt_seed(self.g, rep & 0xFFFFFFFF)
        unitary = True
        choices = []
        for op in ops:
            r = self.L.orc_canonical(self.g)
            if "channel" not in op:
                self._defer(op["qs"], op["m"])
                continue
            kops = channel_kops(op["channel"], op["q"], op["p"], True,
                                op.get("qs"))
            cp, chosen = 0.0, None
            for i, (uni, prob, _, _) in enumerate(kops):
                cp += prob
                if r < cp:
                    chosen = i
                    unitary = unitary and uni
                    break
            if chosen is None:
                self._flush()
                if not unitary:
                    self._normalize()
                    unitary = True
                max_prob, max_index = 0.0, 0
                for i, (uni, prob, _, kd) in enumerate(kops):
                    if uni:
                        continue
                    ev = self.L.orc_port_diag1_ev_f32(self.sp, self.n, op["q"],
                                                      kd[0], kd[1])
                    if ev > max_prob:
                        max_prob, max_index = ev, i
                    cp += ev - prob
                    if r < cp or i == len(kops) - 1:
                        chosen = i if r < cp else max_index
                        unitary = False
                        break
            for qs, m in kops[chosen][2]:
                self._defer(list(qs), m)
            choices.append(chosen)
        self._flush()
        if not unitary:
            self._normalize()
        return choices

    def state(self):
        return self.s[: 2 << self.n].view(np.complex64)


def time_batch(lib, circuits, reps_per_circuit: int, sample_reps: int,
               p_depol: float, gamma: float, cycle_len: int = 2):
    """Bounded sample of a trajectory batch: for each distinct qubit count
    the first circuit of that size runs `sample_reps` repetitions; the
    batch's time is estimated as sum over its circuits of
    reps_per_circuit x the mean sampled time at the circuit's qubit count.
    circuits: list of (n, clean ops).  Returns (estimated seconds, sample
    description, per-n mean seconds)."""
    by_n = {}
    for n, clean in circuits:
        by_n.setdefault(n, clean)
    mean_s = {}
    for n, clean in sorted(by_n.items()):
        port = TrajectoryPort(lib, n)
        ops = noisy_ops(clean, n, p_depol, gamma, cycle_len)
        port.run(ops, 10**6)   # warm-up (page faults of the state)
        ts = []
        for rep in range(sample_reps):
            t0 = time.perf_counter()
            port.run(ops, rep)
            ts.append(time.perf_counter() - t0)
        mean_s[n] = float(np.mean(ts))
    total = sum(reps_per_circuit * mean_s[n] for n, _ in circuits)
    desc = (f"{sample_reps} repetitions of one circuit per qubit count "
            f"({len(by_n)} counts), FP32 port of RunIteration on the host "
            f"cores; batch time = sum over the {len(circuits)} circuits of "
            f"{reps_per_circuit} x the mean time at that qubit count")
    return total, desc, mean_s
