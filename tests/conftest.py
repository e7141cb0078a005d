"""Shared fixtures: the oracle (CPU restatement, test infrastructure), golden
fixtures made from the reference, and GPU gating."""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def gpu_available() -> bool:
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            rt = C.CDLL("/usr/local/cuda/lib64/libcudart.so")
        except OSError:
            return False
    n = C.c_int(0)
    return rt.cudaGetDeviceCount(C.byref(n)) == 0 and n.value > 0


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


# ---------------------------------------------------------------- oracle --
class Oracle:
    """ctypes view of oracle/qsim_oracle.c (test infrastructure only)."""

    def __init__(self):
        if not os.path.exists(ORACLE_SO):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")],
                           check=True, capture_output=True)
        L = C.CDLL(ORACLE_SO)
        P = C.POINTER
        dp, fp, up, u64p = P(C.c_double), P(C.c_float), P(C.c_uint), P(C.c_uint64)
        for name, res, args in [
            ("orc_apply_gate_f64", None, [dp, C.c_uint, up, C.c_uint, dp]),
            ("orc_apply_controlled_gate_f64", None,
             [dp, C.c_uint, up, C.c_uint, up, C.c_uint, C.c_uint64, dp]),
            ("orc_expectation_value_f64", None,
             [dp, C.c_uint, up, C.c_uint, dp, dp]),
            ("orc_apply_gate_f32", None, [fp, C.c_uint, up, C.c_uint, fp]),
            ("orc_apply_gate_lanes_f64", None, [dp, C.c_uint, up, C.c_uint, dp]),
            ("orc_port_apply_gate_f32", None, [fp, C.c_uint, up, C.c_uint, fp]),
            ("orc_norm_f64", C.c_double, [dp, C.c_uint]),
            ("orc_inner_product_f64", None, [dp, dp, C.c_uint, dp]),
            ("orc_mt_seed", None, [C.c_void_p, C.c_uint32]),
            ("orc_mt_next", C.c_uint32, [C.c_void_p]),
            ("orc_canonical", C.c_double, [C.c_void_p]),
            ("orc_uniform", C.c_double, [C.c_void_p, C.c_double]),
            ("orc_mt_size", C.c_size_t, []),
            ("orc_generate_random_values", None,
             [C.c_uint64, C.c_uint32, C.c_double, dp]),
            ("orc_sample_f64", None, [dp, C.c_uint, C.c_uint64, C.c_uint32, u64p]),
            ("orc_find_index_f64", C.c_uint64, [dp, C.c_uint, C.c_double]),
            ("orc_collapse_f64", None, [dp, C.c_uint, C.c_uint64, C.c_uint64]),
            ("orc_num_threads", C.c_int, []),
            ("orc_set_num_threads", None, [C.c_int]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        self.L = L

    @staticmethod
    def _u32(xs):
        xs = list(xs)
        return (C.c_uint * max(1, len(xs)))(*xs)

    @staticmethod
    def _dp(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    def zero_state(self, n):
        s = np.zeros(1 << n, dtype=np.complex128)
        s[0] = 1
        return s

    def apply_gate(self, s, n, qs, m):
        m = np.ascontiguousarray(np.asarray(m, np.complex128)).view(np.float64)
        self.L.orc_apply_gate_f64(self._dp(s), n, self._u32(qs), len(qs), self._dp(m))

    def apply_controlled_gate(self, s, n, qs, cqs, cvals, m):
        m = np.ascontiguousarray(np.asarray(m, np.complex128)).view(np.float64)
        self.L.orc_apply_controlled_gate_f64(self._dp(s), n, self._u32(qs), len(qs),
                                             self._u32(cqs), len(cqs), cvals, self._dp(m))

    def expectation_value(self, s, n, qs, m):
        m = np.ascontiguousarray(np.asarray(m, np.complex128)).view(np.float64)
        out = np.zeros(2)
        self.L.orc_expectation_value_f64(self._dp(s), n, self._u32(qs), len(qs),
                                         self._dp(m), self._dp(out))
        return complex(out[0], out[1])

    def norm(self, s, n):
        return self.L.orc_norm_f64(self._dp(s), n)

    def sample(self, s, n, m, seed):
        out = np.zeros(max(1, m), dtype=np.uint64)
        self.L.orc_sample_f64(self._dp(s), n, m, seed,
                              out.ctypes.data_as(C.POINTER(C.c_uint64)))
        return out[:m]

    def mt(self, seed):
        buf = C.create_string_buffer(self.L.orc_mt_size())
        self.L.orc_mt_seed(buf, seed)
        return buf

    def find_index(self, s, n, r):
        return int(self.L.orc_find_index_f64(self._dp(s), n, r))

    def collapse(self, s, n, mask, bits):
        self.L.orc_collapse_f64(self._dp(s), n, mask, bits)

    def unitary(self, n, ops):
        """The reference's UnitaryCalculatorBasic from the identity
        (lib/unitary_calculator_basic.h:126-259): entry (i, j) at index
        i * 2^n + j, each gate applied to every row over the column bits at
        its qubits, i.e. the oracle's state-vector gate on qubits < n of a
        2n-qubit state.  Returns the (2^n, 2^n) complex128 matrix."""
        d = 1 << n
        u = np.zeros(d * d, dtype=np.complex128)
        u[np.arange(d) * d + np.arange(d)] = 1.0
        for o in ops:
            if o["kind"] == 0:
                self.apply_gate(u, 2 * n, o["qs"], o["m"])
            elif o["kind"] == 1:
                self.apply_controlled_gate(u, 2 * n, o["qs"], o["cqs"],
                                           o["cvals"], o["m"])
        return u.reshape(d, d)

    def apply_gate_lanes(self, s, n, qs, m):
        """orc_apply_gate_f64 restated lane-batched (same sums, vectorised):
        the fast path for large states."""
        m = np.ascontiguousarray(np.asarray(m, np.complex128)).view(np.float64)
        self.L.orc_apply_gate_lanes_f64(self._dp(s), n, self._u32(qs), len(qs),
                                        self._dp(m))

    def run_ops_fp64_fused(self, n, ops):
        """FP64 final state from |0...0> with every one-qubit gate folded
        into the next two-qubit gate on its qubit, the matrix products in
        FP64: QSimRunner with the reference's BasicGateFuser
        (lib/fuser_basic.h: one-qubit gates fused into their neighbouring
        two-qubit gates) on SimulatorBasic<For, double>
        (lib/simulator_basic.h:31).  Controlled gates and gates on more
        qubits are applied as they are, after the one-qubit gates pending on
        their qubits.  A 30-qubit grid circuit of depth 20 takes ~270 passes
        instead of ~840."""
        s = self.zero_state(n)
        pending = {}

        def flush(qs):
            for q in qs:
                m = pending.pop(q, None)
                if m is not None:
                    self.apply_gate_lanes(s, n, [q], m)

        for o in ops:
            if o["kind"] == 0 and len(o["qs"]) == 1:
                q = o["qs"][0]
                m = np.asarray(o["m"], np.complex128)
                pending[q] = m @ pending[q] if q in pending else m
            elif o["kind"] == 0 and len(o["qs"]) == 2:
                a, b = o["qs"]
                pa = pending.pop(a, np.eye(2))
                pb = pending.pop(b, np.eye(2))
                m = np.asarray(o["m"], np.complex128) @ np.kron(pb, pa)
                self.apply_gate_lanes(s, n, [a, b], m)
            elif o["kind"] == 0:
                flush(o["qs"])
                self.apply_gate_lanes(s, n, o["qs"], o["m"])
            elif o["kind"] == 1:
                flush(list(o["qs"]) + list(o["cqs"]))
                qs, m = expand_controlled(o["qs"], o["cqs"], o["cvals"], o["m"])
                self.apply_gate_lanes(s, n, qs, m)
            else:
                flush(o.get("qs", ()))
        flush(sorted(pending))
        return s

    def run_ops(self, n, ops):
        s = self.zero_state(n)
        for o in ops:
            if o["kind"] == 0:
                self.apply_gate(s, n, o["qs"], o["m"])
            elif o["kind"] == 1:
                self.apply_controlled_gate(s, n, o["qs"], o["cqs"], o["cvals"], o["m"])
        return s


def expand_controlled(qs, cqs, cvals, m):
    """A controlled gate as a dense gate on sorted(qs + cqs): the identity
    except where the control bits equal cvals (bit i <-> cqs[i],
    lib/gate.h:37-70), where the target matrix acts (bit j <-> qs[j])."""
    u = sorted(list(qs) + list(cqs))
    pos = {q: i for i, q in enumerate(u)}
    k, d = len(qs), 1 << len(u)
    m = np.asarray(m, np.complex128)
    x = np.arange(d)
    tid = np.zeros(d, np.int64)
    cv = np.zeros(d, np.int64)
    for j, q in enumerate(qs):
        tid |= ((x >> pos[q]) & 1) << j
    for i, q in enumerate(cqs):
        cv |= ((x >> pos[q]) & 1) << i
    full = np.zeros((d, d), np.complex128)
    same_c = cv[:, None] == cv[None, :]
    on = same_c & (cv[:, None] == cvals)
    full[on] = m[tid[:, None], tid[None, :]][on]
    off = same_c & (cv[:, None] != cvals) & (tid[:, None] == tid[None, :])
    full[off] = 1.0
    return u, full


@pytest.fixture(scope="session")
def oracle():
    return Oracle()


# ---------------------------------------------------------------- golden --
def unpack_ops(d):
    ops = []
    for i, kind in enumerate(d["kinds"]):
        qs = d["qpool"][d["qoff"][i]:d["qoff"][i + 1]].tolist()
        cqs = d["cpool"][d["coff"][i]:d["coff"][i + 1]].tolist()
        mf = d["mpool"][d["moff"][i]:d["moff"][i + 1]]
        m = mf.view(np.complex64).astype(np.complex128).reshape(
            1 << len(qs), 1 << len(qs)) if mf.size else None
        ops.append(dict(kind=int(kind), qs=qs, cqs=cqs,
                        cvals=int(d["cvals"][i]), m=m))
    return ops


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _gate_list_cases():
    out = []
    for p in glob.glob(os.path.join(GOLDEN, "*.npz")):
        with np.load(p) as z:
            if ("kinds" in z.files and "op_channel" not in z.files
                    and "u64" not in z.files):
                out.append(os.path.basename(p)[:-4])
    return sorted(out)


# Golden cases that hold a gate list (no channels) and the reference's
# state-vector outputs for it (the unitary cases hold a unitary instead).
GOLDEN_CASES = _gate_list_cases()
UNITARY_CASES = sorted(os.path.basename(p)[:-4]
                       for p in glob.glob(os.path.join(GOLDEN, "unitary*.npz")))


PAULI = {
    "I": np.eye(2, dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def pauli_matrix(ops: str) -> np.ndarray:
    """Pauli string on sorted qubits: ops[j] acts on qs[j], bit j of the
    matrix index is qs[j]."""
    m = np.array([[1.0 + 0j]])
    for p in ops:
        m = np.kron(PAULI[p], m)
    return m


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ---------------------------------------------------------------- engine --
@pytest.fixture(scope="session")
def qsg():
    import qsim_gb300
    return qsim_gb300
