"""Host-side engine objects exposed through the C ABI: random numbers now,
circuits, fusion plans and runners as they are added."""
from __future__ import annotations

import numpy as np

from . import _native as N


class Rng:
    """std::mt19937(seed) with uniform_real_distribution<double> draws, the
    generator the reference passes to Measure (lib/statespace.h:97-140)."""

    def __init__(self, seed: int):
        self.h = N.lib.qsg_rng_create(seed & 0xFFFFFFFF)

    def next_u32(self) -> int:
        return int(N.lib.qsg_rng_next_u32(self.h))

    def uniform(self, max_value: float) -> float:
        return float(N.lib.qsg_rng_uniform(self.h, max_value))

    def __del__(self):
        try:
            N.lib.qsg_rng_destroy(self.h)
        except Exception:
            pass


def generate_random_values(num: int, seed: int, max_value: float) -> np.ndarray:
    """GenerateRandomValues (lib/util.h:67-85) without the sentinel."""
    out = np.empty(max(1, num), dtype=np.float64)
    N.lib.qsg_generate_random_values(num, seed & 0xFFFFFFFF, max_value,
                                     out.ctypes.data_as(N.P_f64))
    return out[:num]


import ctypes as C

from ._native import check

KIND_GATE, KIND_CONTROLLED, KIND_MEASURE = 0, 1, 2


def _u32(xs):
    return N.u32_array(xs)


def _c128(m):
    a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    return a, a.view(np.float64).ctypes.data_as(N.P_f64)


class Circuit:
    """Operation list (lib/circuit.h) built through the engine's C ABI."""

    def __init__(self, num_qubits: int = 0, _handle=None):
        if _handle is not None:
            self.h = _handle
        else:
            h = C.c_void_p()
            check(N.lib.qsg_circuit_create(num_qubits, C.byref(h)))
            self.h = h

    # ---- constructors ------------------------------------------------------
    @classmethod
    def parse(cls, text: str, maxtime: int = 0xFFFFFFFF) -> "Circuit":
        h = C.c_void_p()
        check(N.lib.qsg_circuit_parse(text.encode(), maxtime, C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def grid(cls, rows, cols, extra, cycles, seed) -> "Circuit":
        h = C.c_void_p()
        check(N.lib.qsg_circuit_grid(rows, cols, extra, cycles, seed, C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def chain(cls, n, cycles, seed) -> "Circuit":
        h = C.c_void_p()
        check(N.lib.qsg_circuit_chain(n, cycles, seed, C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def layered_u3(cls, n, layers, num_controlled, seed) -> "Circuit":
        h = C.c_void_p()
        check(N.lib.qsg_circuit_layered_u3(n, layers, num_controlled, seed,
                                           C.byref(h)))
        return cls(_handle=h)

    # ---- building ----------------------------------------------------------
    def add_gate(self, time, qs, matrix):
        _, mp = _c128(matrix)
        check(N.lib.qsg_circuit_add_gate(self.h, time, _u32(qs), len(qs), mp))

    def add_controlled_gate(self, time, qs, cqs, cvals, matrix):
        _, mp = _c128(matrix)
        check(N.lib.qsg_circuit_add_controlled_gate(
            self.h, time, _u32(qs), len(qs), _u32(cqs), len(cqs), cvals, mp))

    def add_measurement(self, time, qs):
        check(N.lib.qsg_circuit_add_measurement(self.h, time, _u32(qs), len(qs)))

    def add_named(self, time, name, qs, params=()):
        p = (C.c_double * max(1, len(params)))(*params)
        check(N.lib.qsg_circuit_add_named_gate(self.h, time, name.encode(),
                                               _u32(qs), len(qs), p, len(params)))

    # ---- inspection --------------------------------------------------------
    @property
    def num_qubits(self) -> int:
        n = C.c_uint()
        check(N.lib.qsg_circuit_info(self.h, C.byref(n), None))
        return n.value

    def __len__(self) -> int:
        m = C.c_uint64()
        check(N.lib.qsg_circuit_info(self.h, None, C.byref(m)))
        return m.value

    def op(self, i: int) -> dict:
        kind, time, k, nc = C.c_int(), C.c_uint(), C.c_uint(), C.c_uint()
        check(N.lib.qsg_circuit_get_op(self.h, i, C.byref(kind), C.byref(time),
                                       C.byref(k), None, C.byref(nc), None,
                                       None, None))
        qs = (C.c_uint * 64)()
        cqs = (C.c_uint * 64)()
        cv = C.c_uint64()
        d = 1 << k.value
        m = np.zeros(d * d, dtype=np.complex128)
        check(N.lib.qsg_circuit_get_op(self.h, i, None, None, None, qs, None,
                                       cqs, C.byref(cv),
                                       m.view(np.float64).ctypes.data_as(N.P_f64)))
        return dict(kind=kind.value, time=time.value, qs=list(qs[:k.value]),
                    cqs=list(cqs[:nc.value]), cvals=cv.value,
                    m=m.reshape(d, d) if kind.value != KIND_MEASURE else None)

    def ops(self):
        return [self.op(i) for i in range(len(self))]

    def set_schmidt(self, i: int, terms):
        """Schmidt terms of two-qubit op i: a list of (A, B) 2x2 factors, A
        on the op's first (lower) qubit, summing to the op's matrix."""
        buf = np.zeros(16 * max(1, len(terms)), dtype=np.float64)
        c = buf.view(np.complex128)
        for j, (a, b) in enumerate(terms):
            c[8 * j:8 * j + 4] = np.asarray(a, np.complex128).ravel()
            c[8 * j + 4:8 * j + 8] = np.asarray(b, np.complex128).ravel()
        check(N.lib.qsg_circuit_set_schmidt(self.h, i, len(terms),
                                            buf.ctypes.data_as(N.P_f64)))

    def schmidt(self, i: int):
        """Operator Schmidt terms of op i (two-qubit named gates): a list of
        (A, B), A the 2x2 factor on the op's first qubit; [] otherwise."""
        t = C.c_uint()
        check(N.lib.qsg_circuit_get_schmidt(self.h, i, C.byref(t), None))
        buf = np.zeros(16 * max(1, t.value), dtype=np.float64)
        check(N.lib.qsg_circuit_get_schmidt(self.h, i, C.byref(t),
                                            buf.ctypes.data_as(N.P_f64)))
        c = buf.view(np.complex128)
        return [(c[8 * j:8 * j + 4].reshape(2, 2).copy(),
                 c[8 * j + 4:8 * j + 8].reshape(2, 2).copy())
                for j in range(t.value)]

    def __del__(self):
        try:
            N.lib.qsg_circuit_destroy(self.h)
        except Exception:
            pass


def pauli_sum(n, count, max_weight, seed):
    w = (C.c_uint * count)()
    q = (C.c_uint * (count * max_weight))()
    letters = C.create_string_buffer(count * max_weight + 1)
    co = (C.c_double * count)()
    check(N.lib.qsg_pauli_sum(n, count, max_weight, seed, w, q, letters, co))
    raw = letters.raw
    out = []
    for i in range(count):
        qs = list(q[i * max_weight:i * max_weight + w[i]])
        ls = raw[i * max_weight:i * max_weight + w[i]].decode()
        out.append((qs, ls, co[i]))
    return out


class PlanCache:
    """Fused plans keyed by circuit content (qsg_plan_cache): a repeated
    circuit, given as a Circuit or as qsim text, skips parsing and fusion,
    and a plan without measurements replays the CUDA graph captured on its
    first run on the same state."""

    def __init__(self, capacity: int = 64):
        h = C.c_void_p()
        check(N.lib.qsg_plan_cache_create(capacity, C.byref(h)))
        self.h = h
        self._ctxs = []   # device buffers of cached plans belong to these

    @staticmethod
    def _opts(max_fused_size, tensor_path, tc_min_k, seeds, cost_model,
              tc_pairs=0):
        if cost_model is not None and hasattr(cost_model, "h"):
            cost_model = cost_model.h.value
        return N.FuseOptions(max_fused_size, seeds, int(tensor_path), tc_min_k,
                             cost_model, tc_pairs)

    def run(self, ctx, circuit, state, seed: int = 1, max_meas: int = 1024,
            max_fused_size: int = 4, tensor_path: bool = False,
            tc_min_k: int = 5, seeds: int = 0, cost_model=None,
            maxtime: int = 0xFFFFFFFF, tc_pairs: int = 0):
        """QSimRunner::Run of `circuit` (a Circuit, or qsim text as str) on
        `state`; returns (measured bits, hit)."""
        if not any(c is ctx for c in self._ctxs):
            self._ctxs.append(ctx)
        o = self._opts(max_fused_size, tensor_path, tc_min_k, seeds, cost_model,
                       tc_pairs)
        bits = np.zeros(max_meas, dtype=np.uint64)
        nm, hit = C.c_uint64(), C.c_int()
        if isinstance(circuit, str):
            check(N.lib.qsg_plan_cache_run_text(
                ctx.h, self.h, circuit.encode(), maxtime, C.byref(o),
                state.get(), seed, bits.ctypes.data_as(N.P_u64), max_meas,
                C.byref(nm), C.byref(hit)))
        else:
            check(N.lib.qsg_plan_cache_run(
                ctx.h, self.h, circuit.h, C.byref(o), state.get(), seed,
                bits.ctypes.data_as(N.P_u64), max_meas, C.byref(nm),
                C.byref(hit)))
        return bits[:nm.value], bool(hit.value)

    def stats(self):
        v = [C.c_uint64() for _ in range(5)]
        check(N.lib.qsg_plan_cache_stats(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("hits", "misses", "evictions", "captures", "size"),
                        (x.value for x in v)))

    def clear(self):
        check(N.lib.qsg_plan_cache_clear(self.h))

    def __del__(self):
        try:
            N.lib.qsg_plan_cache_destroy(self.h)
        except Exception:
            pass


class Plan:
    """Fused plan (MultiQubitGateFuser output) ready to run on the GPU."""

    def __init__(self, circuit: Circuit, max_fused_size: int = 4,
                 tensor_path: bool = False, tc_min_k: int = 5, seeds: int = 0,
                 cost_model=None, unfused: bool = False, tc_pairs: int = 0):
        """tc_pairs: minimum run bits of two-gate tensor-core passes (0: one
        pass per block).  The planner weighs each pair by the saving
        measured for its tile's shape (run bits, and for short runs the
        tile's other low qubits) and takes only pairs predicted faster than
        two passes."""
        self.circuit = circuit
        h = C.c_void_p()
        if unfused:
            check(N.lib.qsg_plan_create_unfused(circuit.h, C.byref(h)))
        else:
            if cost_model is not None and hasattr(cost_model, "h"):
                cost_model = cost_model.h.value   # a learned.CostMLP
            o = N.FuseOptions(max_fused_size, seeds, int(tensor_path), tc_min_k,
                              cost_model, tc_pairs)
            check(N.lib.qsg_plan_create(circuit.h, C.byref(o), C.byref(h)))
        self.h = h

    def info(self):
        n, k, t = C.c_uint64(), C.c_uint(), C.c_uint64()
        check(N.lib.qsg_plan_info(self.h, C.byref(n), C.byref(k), C.byref(t)))
        pairs = C.c_uint64()
        check(N.lib.qsg_plan_tc_pairs(self.h, C.byref(pairs), None))
        return dict(num_ops=n.value, max_k=k.value, num_tensor_ops=t.value,
                    num_tc_pairs=pairs.value)

    def tc_pair_next(self) -> np.ndarray:
        """Per op: 1 if it starts a two-gate tensor-core pass."""
        n = self.info()["num_ops"]
        out = np.zeros(max(1, n), dtype=np.uint8)
        check(N.lib.qsg_plan_tc_pairs(self.h, None,
                                      out.ctypes.data_as(C.POINTER(C.c_ubyte))))
        return out[:n]

    def __len__(self):
        return self.info()["num_ops"]

    def op(self, i: int) -> dict:
        kind, k, nc, path = C.c_int(), C.c_uint(), C.c_uint(), C.c_int()
        nm = C.c_uint64()
        check(N.lib.qsg_plan_get_op(self.h, i, C.byref(kind), C.byref(k), None,
                                    C.byref(nc), None, None, C.byref(path),
                                    C.byref(nm), None))
        qs = (C.c_uint * 64)()
        cqs = (C.c_uint * 64)()
        cv = C.c_uint64()
        d = 1 << k.value
        m = np.zeros(d * d, dtype=np.complex128)
        check(N.lib.qsg_plan_get_op(self.h, i, None, None, qs, None, cqs,
                                    C.byref(cv), None, None,
                                    m.view(np.float64).ctypes.data_as(N.P_f64)))
        return dict(kind=kind.value, qs=list(qs[:k.value]),
                    cqs=list(cqs[:nc.value]), cvals=cv.value, path=path.value,
                    members=nm.value,
                    m=m.reshape(d, d) if kind.value != KIND_MEASURE else None)

    def ops(self):
        return [self.op(i) for i in range(len(self))]

    def set_schmidt(self, i: int, terms):
        """Schmidt terms of two-qubit op i: a list of (A, B) 2x2 factors, A
        on the op's first (lower) qubit, summing to the op's matrix."""
        buf = np.zeros(16 * max(1, len(terms)), dtype=np.float64)
        c = buf.view(np.complex128)
        for j, (a, b) in enumerate(terms):
            c[8 * j:8 * j + 4] = np.asarray(a, np.complex128).ravel()
            c[8 * j + 4:8 * j + 8] = np.asarray(b, np.complex128).ravel()
        check(N.lib.qsg_circuit_set_schmidt(self.h, i, len(terms),
                                            buf.ctypes.data_as(N.P_f64)))

    def schmidt(self, i: int):
        """Operator Schmidt terms of op i (two-qubit named gates): a list of
        (A, B), A the 2x2 factor on the op's first qubit; [] otherwise."""
        t = C.c_uint()
        check(N.lib.qsg_circuit_get_schmidt(self.h, i, C.byref(t), None))
        buf = np.zeros(16 * max(1, t.value), dtype=np.float64)
        check(N.lib.qsg_circuit_get_schmidt(self.h, i, C.byref(t),
                                            buf.ctypes.data_as(N.P_f64)))
        c = buf.view(np.complex128)
        return [(c[8 * j:8 * j + 4].reshape(2, 2).copy(),
                 c[8 * j + 4:8 * j + 8].reshape(2, 2).copy())
                for j in range(t.value)]

    def run(self, ctx, state, seed: int = 1, max_meas: int = 1024):
        self._ctx = ctx   # the plan's device buffers belong to this context
        bits = np.zeros(max_meas, dtype=np.uint64)
        nm = C.c_uint64()
        check(N.lib.qsg_plan_run(ctx.h, self.h, state.get(), seed,
                                 bits.ctypes.data_as(N.P_u64), max_meas,
                                 C.byref(nm)))
        return bits[:nm.value]

    def capture(self, ctx, state):
        self._ctx = ctx   # the plan's device buffers belong to this context
        check(N.lib.qsg_plan_capture(ctx.h, self.h, state.get()))

    def profile(self, ctx, state):
        """Per-op milliseconds (CUDA events around each launch)."""
        self._ctx = ctx   # the plan's device buffers belong to this context
        n = len(self)
        ms = np.zeros(max(1, n), dtype=np.float32)
        check(N.lib.qsg_plan_profile(ctx.h, self.h, state.get(),
                                     ms.ctypes.data_as(N.P_f32), n))
        return ms[:n]

    def replay(self, ctx):
        self._ctx = ctx   # the plan's device buffers belong to this context
        check(N.lib.qsg_plan_replay(ctx.h, self.h))

    def __del__(self):
        try:
            N.lib.qsg_plan_destroy(self.h)
        except Exception:
            pass


# ---- noisy circuits and trajectories ---------------------------------------

CHANNEL_DEPOLARIZING, CHANNEL_AMPLITUDE_DAMPING, CHANNEL_PHASE_DAMPING = 0, 1, 2
CHANNEL_BIT_FLIP, CHANNEL_PHASE_FLIP, CHANNEL_RESET = 3, 4, 5
# The reference's multi-qubit depolarizing factory: Pauli of digit j on
# register qubit j (lib/channels_cirq.h:147-189).
CHANNEL_DEPOLARIZING_REGISTER = 6
NO_STAT = np.uint64(0xFFFFFFFFFFFFFFFF)


class NoisyCircuit:
    """Circuit with channels (lib/circuit_noisy.h, lib/channels_cirq.h)."""

    def __init__(self, num_qubits: int = 0, _handle=None):
        if _handle is not None:
            self.h = _handle
        else:
            h = C.c_void_p()
            check(N.lib.qsg_noisy_create(num_qubits, C.byref(h)))
            self.h = h

    @classmethod
    def make(cls, circuit: Circuit, p_depol: float, gamma: float = 0.0,
             cycle_len: int = 2) -> "NoisyCircuit":
        """MakeNoisy with depolarizing(p_depol) after each op's qubits and,
        with gamma > 0, amplitude damping(gamma) on every qubit after each
        cycle of `cycle_len` clean time steps."""
        h = C.c_void_p()
        check(N.lib.qsg_noisy_make(circuit.h, p_depol, gamma, cycle_len,
                                   C.byref(h)))
        return cls(_handle=h)

    def append(self, circuit: Circuit):
        check(N.lib.qsg_noisy_append_circuit(self.h, circuit.h))

    def _append_one(self, build):
        c = Circuit(self.info()["num_qubits"])
        build(c)
        self.append(c)

    def add_gate(self, time, qs, matrix):
        self._append_one(lambda c: c.add_gate(time, qs, matrix))

    def add_controlled_gate(self, time, qs, cqs, cvals, matrix):
        self._append_one(lambda c: c.add_controlled_gate(time, qs, cqs, cvals,
                                                         matrix))

    def add_measurement(self, time, qs):
        self._append_one(lambda c: c.add_measurement(time, qs))

    def add_channel(self, kind: int, time: int, qs, p: float = 0.0):
        check(N.lib.qsg_noisy_add_channel(self.h, kind, time, _u32(qs),
                                          len(qs), p))

    def add_kraus_channel(self, time: int, qs, kops):
        """kops: list of (unitary: bool, prob: float, matrix 2^k x 2^k)."""
        mats = np.ascontiguousarray(
            np.stack([np.asarray(m, np.complex128).reshape(-1) for _, _, m in kops]))
        uni = (C.c_int * len(kops))(*[int(u) for u, _, _ in kops])
        pr = (C.c_double * len(kops))(*[float(p) for _, p, _ in kops])
        check(N.lib.qsg_noisy_add_kraus_channel(
            self.h, time, _u32(qs), len(qs), len(kops), uni, pr,
            mats.view(np.float64).ctypes.data_as(N.P_f64)))

    def info(self):
        n, m, c = C.c_uint(), C.c_uint64(), C.c_uint64()
        check(N.lib.qsg_noisy_info(self.h, C.byref(n), C.byref(m), C.byref(c)))
        return dict(num_qubits=n.value, num_ops=m.value, num_channels=c.value)

    def __len__(self):
        return self.info()["num_ops"]

    def op(self, i: int) -> dict:
        ch, t, nq, nk = C.c_int(), C.c_uint(), C.c_uint(), C.c_uint()
        qs = (C.c_uint * 64)()
        check(N.lib.qsg_noisy_get_op(self.h, i, C.byref(ch), C.byref(t),
                                     C.byref(nq), qs, C.byref(nk)))
        return dict(is_channel=bool(ch.value), time=t.value,
                    qs=list(qs[:nq.value]), num_kops=nk.value)

    def __del__(self):
        try:
            N.lib.qsg_noisy_destroy(self.h)
        except Exception:
            pass


class Trajectories:
    """QuantumTrajectorySimulator for one noisy circuit (lib/qtrajectory.h)."""

    def __init__(self, noisy: NoisyCircuit, max_fused_size: int = 4,
                 seeds: int = 0, collect_kop_stat: bool = True,
                 collect_mea_stat: bool = True,
                 normalize_before_mea_gates: bool = True,
                 tensor_path: bool = False, tc_min_k: int = 5):
        self.noisy = noisy
        o = N.TrajOptions(max_fused_size, seeds, int(collect_kop_stat),
                          int(collect_mea_stat), int(normalize_before_mea_gates),
                          int(tensor_path), tc_min_k)
        h = C.c_void_p()
        check(N.lib.qsg_traj_create(noisy.h, C.byref(o), C.byref(h)))
        self.h = h

    def info(self):
        n, m, f = C.c_uint(), C.c_uint64(), C.c_uint64()
        check(N.lib.qsg_traj_info(self.h, C.byref(n), C.byref(m), C.byref(f)))
        return dict(num_qubits=n.value, num_ops=m.value, num_fused_ops=f.value)

    def run(self, ctx, state, rep: int) -> np.ndarray:
        """RunOnce: trajectory `rep` into `state`; per-op statistics."""
        stats = np.zeros(max(1, self.info()["num_ops"]), dtype=np.uint64)
        check(N.lib.qsg_traj_run(ctx.h, self.h, state.get(), rep,
                                 stats.ctypes.data_as(N.P_u64)))
        return stats

    def run_from(self, ctx, state, rep: int) -> np.ndarray:
        """RunOnce on `state` as given (not reset to |0..0>)."""
        stats = np.zeros(max(1, self.info()["num_ops"]), dtype=np.uint64)
        check(N.lib.qsg_traj_run_from(ctx.h, self.h, state.get(), rep,
                                      stats.ctypes.data_as(N.P_u64)))
        return stats

    @staticmethod
    def samples(stats: np.ndarray) -> np.ndarray:
        """The reference's stat.samples: entries other than NO_STAT."""
        return stats[stats != NO_STAT]


def run_trajectory_batch(runners, items, num_streams: int = 8, device: int = 0,
                         out_states=None, big_qubits: int = 0,
                         big_streams: int = 1, return_launches: bool = False):
    """RunBatch over items [(runner index, rep)] on concurrent streams.
    Returns (per-item stats list, latency_ms array, wall seconds) and, with
    return_launches, the number of kernels launched."""
    nr = len(runners)
    rh = (C.c_void_p * max(1, nr))(*[r.h.value for r in runners])
    ir = np.ascontiguousarray([i for i, _ in items], dtype=np.uint32)
    rp = np.ascontiguousarray([r for _, r in items], dtype=np.uint64)
    sizes = [runners[i].info()["num_ops"] for i, _ in items]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    stats = np.zeros(max(1, int(offs[-1])), dtype=np.uint64)
    lat = np.zeros(max(1, len(items)), dtype=np.float32)
    wall = C.c_double()
    launches = C.c_uint64()
    outs = None
    if out_states is not None:
        outs = (C.c_void_p * len(items))(*[s.get() if s is not None else None
                                           for s in out_states])
    o = N.BatchOptions(num_streams, big_qubits, big_streams)
    check(N.lib.qsg_traj_run_batch(
        device, rh, nr, ir.ctypes.data_as(N.P_u32), rp.ctypes.data_as(N.P_u64),
        len(items), C.byref(o), stats.ctypes.data_as(N.P_u64), outs,
        lat.ctypes.data_as(N.P_f32), C.byref(wall), C.byref(launches)))
    per = [stats[offs[i]:offs[i + 1]] for i in range(len(items))]
    if return_launches:
        return per, lat[:len(items)], wall.value, launches.value
    return per, lat[:len(items)], wall.value


def run_trajectory_batch_packed(runners, items, ctas_per_sm: int = 0,
                                max_qubits: int = 0, host_threads: int = 0,
                                num_streams: int = 8, device: int = 0,
                                out_states=None, tile_kib: int = 0,
                                overlap: bool = False):
    """RunBatch as one persistent kernel over a packed batch
    (qsg_traj_run_packed).  Returns (per-item stats list, latency_ms array,
    wall seconds, launches, info dict)."""
    nr = len(runners)
    rh = (C.c_void_p * max(1, nr))(*[r.h.value for r in runners])
    ir = np.ascontiguousarray([i for i, _ in items], dtype=np.uint32)
    rp = np.ascontiguousarray([r for _, r in items], dtype=np.uint64)
    sizes = [runners[i].info()["num_ops"] for i, _ in items]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    stats = np.zeros(max(1, int(offs[-1])), dtype=np.uint64)
    lat = np.zeros(max(1, len(items)), dtype=np.float32)
    wall = C.c_double()
    launches = C.c_uint64()
    outs = None
    if out_states is not None:
        outs = (C.c_void_p * len(items))(*[s.get() if s is not None else None
                                           for s in out_states])
    o = N.PackedOptions(ctas_per_sm, max_qubits, host_threads, tile_kib,
                        int(overlap), N.BatchOptions(num_streams, 0, 0))
    info = N.PackedInfo()
    check(N.lib.qsg_traj_run_packed(
        device, rh, nr, ir.ctypes.data_as(N.P_u32), rp.ctypes.data_as(N.P_u64),
        len(items), C.byref(o), stats.ctypes.data_as(N.P_u64), outs,
        lat.ctypes.data_as(N.P_f32), C.byref(wall), C.byref(launches),
        C.byref(info)))
    per = [stats[offs[i]:offs[i + 1]] for i in range(len(items))]
    inf = {f: getattr(info, f) for f, _ in N.PackedInfo._fields_}
    return per, lat[:len(items)], wall.value, launches.value, inf
