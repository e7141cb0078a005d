"""Generates the golden fixtures in tests/golden/ by running the reference
implementation (quantumlib/qsim) through oracle/_ref/ref_driver.

Run in a container where the reference checkout exists:

    make -C oracle ref REF=<qsim checkout>
    python tests/golden/make_golden.py

Each case is a seeded gate list (written in the driver's text format) plus
the reference's outputs: the FP64 final state of SimulatorBasic<double>
(unfused), the FP32 final state of QSimRunner + MultiQubitGateFuser + the
SIMD simulator, samples, expectation values and measurement outcomes.
Everything is saved to one compressed .npz per case.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
# The reference checkout whose test files hold known answers.
REF_ROOT = os.environ.get("QSIM_REF",
                          os.path.join(os.path.dirname(ROOT), "reference"))

PAULI = {
    "I": np.eye(2, dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def random_unitary(rng: np.random.Generator, k: int) -> np.ndarray:
    d = 1 << k
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def interleave(m: np.ndarray) -> np.ndarray:
    """Row-major interleaved float32 (re, im) of a complex matrix."""
    return np.ascontiguousarray(m.astype(np.complex64)).view(np.float32).ravel()


def hexf(xs) -> str:
    return " ".join(float(x).hex() for x in np.asarray(xs, dtype=np.float32))


def pauli_matrix(ops: str) -> np.ndarray:
    """Matrix of a Pauli string on sorted qubits; ops[j] acts on qs[j], and
    bit j of the matrix index is qs[j] (so qs[0] is the least significant
    factor of the Kronecker product)."""
    m = np.array([[1.0 + 0j]])
    for p in ops:
        m = np.kron(PAULI[p], m)
    return m


def random_gate_list(rng, n, ngates, kmax, ctrl_frac=0.0, meas_at=None):
    """Returns list of dicts: kind g/c/m, qs, cqs, cvals, matrix (complex)."""
    ops = []
    for t in range(ngates):
        if meas_at is not None and t in meas_at:
            k = int(rng.integers(1, 4))
            qs = sorted(rng.choice(n, size=k, replace=False).tolist())
            ops.append(dict(kind="m", time=t, qs=qs))
            continue
        k = int(rng.integers(1, kmax + 1))
        if ctrl_frac > 0 and rng.random() < ctrl_frac:
            k = min(k, 3)
            c = int(rng.integers(1, 4))
            picks = rng.choice(n, size=k + c, replace=False).tolist()
            qs, cqs = sorted(picks[:k]), sorted(picks[k:])
            cvals = int(rng.integers(0, 1 << c))
            ops.append(dict(kind="c", time=t, qs=qs, cqs=cqs, cvals=cvals,
                            m=random_unitary(rng, k)))
        else:
            qs = sorted(rng.choice(n, size=k, replace=False).tolist())
            ops.append(dict(kind="g", time=t, qs=qs, m=random_unitary(rng, k)))
    return ops


def write_gate_list(path, n, ops):
    with open(path, "w") as f:
        f.write(f"n {n}\n")
        for o in ops:
            k = len(o["qs"])
            q = " ".join(map(str, o["qs"]))
            if o["kind"] == "g":
                f.write(f"g {o['time']} {k} {q} {hexf(interleave(o['m']))}\n")
            elif o["kind"] == "c":
                cq = " ".join(map(str, o["cqs"]))
                f.write(f"c {o['time']} {k} {q} {len(o['cqs'])} {cq} "
                        f"{o['cvals']} {hexf(interleave(o['m']))}\n")
            elif o["kind"] == "m":
                f.write(f"m {o['time']} {k} {q}\n")
            elif o["kind"] == "R":
                f.write(f"R {o['time']} {q}\n")
            elif o["kind"] == "Q":
                f.write(f"Q {o['time']} {k} {q} {float(o['p']).hex()}\n")
            else:  # one-qubit channel with one parameter
                f.write(f"{o['kind']} {o['time']} {q} {float(o['p']).hex()}\n")


def pack_ops(ops):
    """Flat arrays for the fixture: kinds, offsets into qubit/matrix pools."""
    kinds, qoff, qpool, coff, cpool, cvals, moff, mpool = [], [0], [], [0], [], [], [0], []
    for o in ops:
        kinds.append({"g": 0, "c": 1, "m": 2}[o["kind"]])
        qpool += o["qs"]
        qoff.append(len(qpool))
        cpool += o.get("cqs", [])
        coff.append(len(cpool))
        cvals.append(o.get("cvals", 0))
        if "m" in o:
            mpool += interleave(o["m"]).tolist()
        moff.append(len(mpool))
    return dict(kinds=np.array(kinds, np.int32), qoff=np.array(qoff, np.int64),
                qpool=np.array(qpool, np.int32), coff=np.array(coff, np.int64),
                cpool=np.array(cpool, np.int32), cvals=np.array(cvals, np.uint64),
                moff=np.array(moff, np.int64), mpool=np.array(mpool, np.float32))


def random_pauli_evs(rng, n, count, wmax):
    evs = []
    for _ in range(count):
        w = int(rng.integers(1, wmax + 1))
        qs = sorted(rng.choice(n, size=w, replace=False).tolist())
        ops = "".join(rng.choice(list("XYZ"), size=w).tolist())
        evs.append((qs, ops, pauli_matrix(ops)))
    return evs


def run_case(name, n, ops, fsize, nsamples, sseed, evs=None, measure=None):
    with tempfile.TemporaryDirectory() as td:
        gl = os.path.join(td, "gates.txt")
        write_gate_list(gl, n, ops)
        out = os.path.join(td, "out")
        cmd = [DRIVER, "run", gl, out, str(fsize), str(nsamples), str(sseed)]
        if evs:
            evf = os.path.join(td, "ev.txt")
            with open(evf, "w") as f:
                for qs, _, m in evs:
                    f.write(f"{len(qs)} {' '.join(map(str, qs))} "
                            f"{hexf(interleave(m))}\n")
            cmd.append(evf)
        subprocess.run(cmd, check=True)
        rd = lambda ext, dt: np.fromfile(out + ext, dtype=dt)
        data = dict(n=np.int32(n), fsize=np.int32(fsize),
                    sample_seed=np.uint32(sseed),
                    f64=rd(".f64", np.float64)[: 2 << n].view(np.complex128),
                    f32=rd(".f32", np.float32).view(np.complex64),
                    meta=rd(".meta", np.float64))
        if nsamples:
            data["s32"] = rd(".s32", np.uint64)
            data["s64"] = rd(".s64", np.uint64)
        if evs:
            ev = rd(".ev", np.float64).reshape(-1, 4)
            data["ev32"] = ev[:, 0] + 1j * ev[:, 1]
            data["ev64"] = ev[:, 2] + 1j * ev[:, 3]
            data["ev_qoff"] = np.cumsum([0] + [len(q) for q, _, _ in evs])
            data["ev_qpool"] = np.array(sum([q for q, _, _ in evs], []), np.int32)
            data["ev_ops"] = np.array([o for _, o, _ in evs])
        if measure:
            mseed, reps, mqs = measure
            mo = os.path.join(td, "meas")
            subprocess.run([DRIVER, "measure", gl, mo, str(mseed), str(reps),
                            str(len(mqs))] + [str(q) for q in mqs], check=True)
            data["meas_seed"] = np.uint32(mseed)
            data["meas_qs"] = np.array(mqs, np.int32)
            data["meas_bits"] = np.fromfile(mo + ".bits", dtype=np.uint64)
            data["meas_state"] = np.fromfile(mo + ".f64", np.float64)[: 2 << n].view(np.complex128)
        data.update(pack_ops(ops))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, "written")


GATES_1Q = ["id1", "h", "t", "x", "y", "z", "x_1_2", "y_1_2", "hz_1_2", "s"]
GATES_1Q_P = [("rx", 1), ("ry", 1), ("rz", 1), ("rxy", 2)]
GATES_2Q = ["id2", "cz", "cnot", "cx", "sw", "is"]
GATES_2Q_P = [("fs", 2), ("cp", 1)]


def random_text_circuit(rng, n, layers):
    """Every gate of the text format (docs/input_format.md), random qubits in
    both orders, angles that are exact in float (multiples of 1/64, some
    negative), controlled gates and a final measurement."""
    lines = [str(n)]
    for t in range(layers):
        perm = rng.permutation(n).tolist()
        i = 0
        while i < n:
            r = rng.random()
            ang = lambda: f"{int(rng.integers(-400, 400)) / 64}"
            if r < 0.35 or i == n - 1:
                g = GATES_1Q[int(rng.integers(len(GATES_1Q)))]
                lines.append(f"{t} {g} {perm[i]}")
                i += 1
            elif r < 0.5:
                g, npar = GATES_1Q_P[int(rng.integers(len(GATES_1Q_P)))]
                lines.append(f"{t} {g} {perm[i]} " + " ".join(ang() for _ in range(npar)))
                i += 1
            elif r < 0.8:
                g = GATES_2Q[int(rng.integers(len(GATES_2Q)))]
                lines.append(f"{t} {g} {perm[i]} {perm[i + 1]}")
                i += 2
            elif r < 0.93 or i + 2 >= n:
                g, npar = GATES_2Q_P[int(rng.integers(len(GATES_2Q_P)))]
                lines.append(f"{t} {g} {perm[i]} {perm[i + 1]} " + " ".join(ang() for _ in range(npar)))
                i += 2
            else:
                lines.append(f"{t} c {perm[i]} {perm[i + 1]} rx {perm[i + 2]} {ang()}")
                i += 3
    lines.append(f"{layers} m " + " ".join(str(q) for q in range(n)))
    return "\n".join(lines) + "\n"


def text_case(name, n, layers, seed):
    rng = np.random.default_rng(seed)
    text = random_text_circuit(rng, n, layers)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "c.txt")
        with open(p, "w") as f:
            f.write(text)
        subprocess.run([DRIVER, "text", p, os.path.join(td, "out")], check=True)
        f64 = np.fromfile(os.path.join(td, "out.f64"), np.float64)[: 2 << n]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), n=np.int32(n),
                        text=np.array(text), f64=f64.view(np.complex128))
    print(name, "written")


def fuse_counts_case():
    """Pass counts of the reference's MultiQubitGateFuser on the seeded grid
    circuits, for comparison with this engine's planner."""
    sys.path.insert(0, ROOT)
    from qsim_gb300 import engine as E
    out = {}
    for name, args in [("grid5x6d20", (5, 6, 0, 20, 1)),
                       ("grid4x5d14", (4, 5, 0, 14, 1)),
                       ("grid5x6p2d24", (5, 6, 2, 24, 1))]:
        c = E.Circuit.grid(*args)
        ops = []
        for o in c.ops():
            ops.append(dict(kind="g", time=o["time"], qs=o["qs"], m=o["m"]))
        with tempfile.TemporaryDirectory() as td:
            gl = os.path.join(td, "g.txt")
            write_gate_list(gl, c.num_qubits, ops)
            counts = []
            for f in (2, 3, 4, 5, 6):
                r = subprocess.run([DRIVER, "fuse", gl, str(f)], check=True,
                                   capture_output=True, text=True).stdout.split()
                counts.append(int(r[0]))
        out[name] = np.array(counts, np.int32)
        out[name + "_args"] = np.array(args, np.int64)
    np.savez_compressed(os.path.join(HERE, "fuser_mqubit_counts.npz"), **out)
    print("fuser_mqubit_counts written")


def config1_case():
    """The 20-qubit 4x5 grid workload (depth 14, seed 1) through the
    reference at max_fused_size 2 with 1000 samples (seed 1).  The full
    state is too large to commit; the fixture keeps the reference's FP64
    amplitudes at 4096 fixed indices, its norm, its samples from the FP32
    (SIMD, fused) and FP64 states, and its fused-op count."""
    sys.path.insert(0, ROOT)
    from qsim_gb300 import engine as E
    c = E.Circuit.grid(4, 5, 0, 14, 1)
    n = c.num_qubits
    ops = [dict(kind="g", time=o["time"], qs=o["qs"], m=o["m"]) for o in c.ops()]
    with tempfile.TemporaryDirectory() as td:
        gl = os.path.join(td, "g.txt")
        write_gate_list(gl, n, ops)
        out = os.path.join(td, "out")
        subprocess.run([DRIVER, "run", gl, out, "2", "1000", "1"], check=True)
        f64 = np.fromfile(out + ".f64", np.float64)[: 2 << n].view(np.complex128)
        f32 = np.fromfile(out + ".f32", np.float32).view(np.complex64)
        idx = np.sort(np.random.default_rng(4).choice(1 << n, 4096, replace=False))
        meta = np.fromfile(out + ".meta", np.float64)
        np.savez_compressed(
            os.path.join(HERE, "config1_grid4x5d14.npz"), n=np.int32(n),
            idx=idx.astype(np.int64), amp64=f64[idx],
            ref_f32_rel_l2=np.float64(np.linalg.norm(f32 - f64) / np.linalg.norm(f64)),
            s32=np.fromfile(out + ".s32", np.uint64),
            s64=np.fromfile(out + ".s64", np.uint64), meta=meta)
    print("config1_grid4x5d14 written")


def read_ref_plan(path):
    """Fused gates written by `ref_driver plan`: per gate k, k qubits and
    the 2*4^k floats of its matrix."""
    import struct
    raw = open(path, "rb").read()
    pos, ks, qs, ms = 0, [], [], []
    while pos < len(raw):
        k = struct.unpack_from("<I", raw, pos)[0]
        pos += 4
        qs.extend(struct.unpack_from(f"<{k}I", raw, pos))
        pos += 4 * k
        cnt = 2 * 4 ** k
        ms.append(np.frombuffer(raw, np.float32, cnt, pos).copy())
        pos += 4 * cnt
        ks.append(k)
    return (np.array(ks, np.int32), np.array(qs, np.int32),
            np.concatenate(ms).astype(np.float32))


def ref_plan_case():
    """The reference's own fused plan (MultiQubitGateFuser, max_fused_size
    4, matrices from CalculateFusedMatrix) of the 30-qubit 5x6 grid depth-20
    circuit (seed 1): the gate passes the CPU baseline times, with no part
    of this repository's engine in the loop."""
    sys.path.insert(0, ROOT)
    from qsim_gb300 import engine as E
    c = E.Circuit.grid(5, 6, 0, 20, 1)
    n = c.num_qubits
    ops = [dict(kind="g", time=o["time"], qs=o["qs"], m=o["m"]) for o in c.ops()]
    with tempfile.TemporaryDirectory() as td:
        gl = os.path.join(td, "g.txt")
        write_gate_list(gl, n, ops)
        out = os.path.join(td, "plan.bin")
        subprocess.run([DRIVER, "plan", gl, "4", out], check=True)
        ks, qs, ms = read_ref_plan(out)
    np.savez_compressed(os.path.join(HERE, "ref_plan_grid5x6d20_f4.npz"),
                        n=np.int32(n), max_fused_size=np.int32(4), k=ks,
                        qubits=qs, matrices=ms)
    print(f"ref_plan_grid5x6d20_f4 written ({len(ks)} fused gates)")


def mt_case():
    with tempfile.TemporaryDirectory() as td:
        out = {}
        for seed in (0, 1, 5489, 123456789, 4294967295):
            p = os.path.join(td, f"mt{seed}")
            subprocess.run([DRIVER, "mt", str(seed), "2000", p], check=True)
            out[f"raw_{seed}"] = np.fromfile(p + ".raw", np.uint32)
            out[f"u01_{seed}"] = np.fromfile(p + ".u01", np.float64)
            out[f"f073_{seed}"] = np.fromfile(p + ".f073", np.float32)
        np.savez_compressed(os.path.join(HERE, "mt19937.npz"), **out)
        print("mt19937 written")


CHANNEL_CODES = {"D": 0, "A": 1, "P": 2, "B": 3, "F": 4, "R": 5, "Q": 6}


def noisy_chain_ops(n, cycles, seed, p_depol, gamma, cycle_len=2):
    """The chain workload with noise inserted by the rule of the engine's
    make_noisy (lib/circuit_noisy.h:33-64 plus amplitude damping on every
    qubit after each cycle), written out op by op."""
    sys.path.insert(0, ROOT)
    from qsim_gb300 import engine as E
    c = E.Circuit.chain(n, cycles, seed)
    clean = c.ops()
    ops = []
    for i, o in enumerate(clean):
        t = o["time"]
        t2 = 2 * (t + t // cycle_len) if gamma > 0 else 2 * t
        kind = {0: "g", 1: "c", 2: "m"}[o["kind"]]
        d = dict(kind=kind, time=t2, qs=o["qs"])
        if kind != "m":
            d["m"] = o["m"]
        if kind == "c":
            d["cqs"], d["cvals"] = o["cqs"], o["cvals"]
        ops.append(d)
        if p_depol > 0:
            for q in o["qs"] + o["cqs"]:
                ops.append(dict(kind="D", time=t2 + 1, qs=[q], p=p_depol))
        last = i + 1 == len(clean) or clean[i + 1]["time"] // cycle_len != t // cycle_len
        if gamma > 0 and last:
            for q in range(n):
                ops.append(dict(kind="A", time=t2 + 2, qs=[q], p=gamma))
    return ops


def mixed_noisy_ops(rng, n, layers):
    """Random one- and two-qubit gates with every one-qubit channel kind of
    lib/channels_cirq.h and measurements."""
    ops = []
    t = 0
    for layer in range(layers):
        for q in range(n):
            ops.append(dict(kind="g", time=t, qs=[q], m=random_unitary(rng, 1)))
        for q in range(layer % 2, n - 1, 2):
            ops.append(dict(kind="g", time=t + 1, qs=[q, q + 1],
                            m=random_unitary(rng, 2)))
        for q in range(n):
            kind = "DAPBFR"[int(rng.integers(6))] if rng.random() < 0.5 else None
            if kind is None:
                continue
            p = {"D": 0.2, "A": 0.3, "P": 0.25, "B": 0.15, "F": 0.15, "R": 0}[kind]
            ops.append(dict(kind=kind, time=t + 2, qs=[q], p=p))
        if layer in (1, layers - 1):
            qs = sorted(rng.choice(n, size=2, replace=False).tolist())
            ops.append(dict(kind="m", time=t + 3, qs=qs))
        t += 4
    return ops


def pack_noisy(ops):
    """Fixture arrays: gates packed as pack_ops does, plus per op a channel
    code (-1 for gates and measurements) and parameter."""
    gate_ops = [o for o in ops if o["kind"] in "gcm"]
    data = pack_ops(gate_ops)
    data["op_channel"] = np.array([CHANNEL_CODES.get(o["kind"], -1) for o in ops],
                                  np.int32)
    data["op_time"] = np.array([o["time"] for o in ops], np.int64)
    data["op_q"] = np.array([o["qs"][0] if o["kind"] in CHANNEL_CODES else -1
                             for o in ops], np.int32)
    data["op_p"] = np.array([o.get("p", 0.0) for o in ops], np.float64)
    data["op_qmask"] = np.array(
        [sum(1 << q for q in o["qs"]) if o["kind"] in CHANNEL_CODES else 0
         for o in ops], np.int64)
    return data


def traj_case(name, n, ops, fsize, r0, r1, states_c64=False):
    """QuantumTrajectorySimulator::RunBatch of the reference over [r0, r1):
    stat.samples per repetition and the final states, in float (SIMD
    simulator) and double (SimulatorBasic)."""
    with tempfile.TemporaryDirectory() as td:
        gl = os.path.join(td, "noisy.txt")
        write_gate_list(gl, n, ops)
        out = os.path.join(td, "out")
        subprocess.run([DRIVER, "traj", gl, out, str(fsize), str(r0), str(r1)],
                       check=True)
        data = dict(n=np.int32(n), fsize=np.int32(fsize), r0=np.int64(r0),
                    r1=np.int64(r1))
        for suf in ("32", "64"):
            st = np.fromfile(out + ".stat" + suf, np.uint64)
            counts, flat, i = [], [], 0
            while i < len(st):
                c = int(st[i])
                counts.append(c)
                flat.extend(st[i + 1:i + 1 + c].tolist())
                i += 1 + c
            data["stat_count" + suf] = np.array(counts, np.int64)
            data["stat" + suf] = np.array(flat, np.uint64)
        f32 = np.fromfile(out + ".f32", np.float32).view(np.complex64)
        f64 = np.fromfile(out + ".f64", np.float64).view(np.complex128)
        data["f32"] = f32.reshape(r1 - r0, -1)
        data["f64"] = (f64.astype(np.complex64) if states_c64 else f64).reshape(r1 - r0, -1)
        data.update(pack_noisy(ops))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, "written")


def depol_register_ops(rng, n, layers):
    """Random one- and two-qubit gates with two-qubit depolarizing channels
    (p = 0.3) on qubit pairs away from qubits 0 and 1, through the
    reference's multi-qubit factory, whose Pauli of digit j acts on
    register qubit j (lib/channels_cirq.h:147-189)."""
    ops, t = [], 0
    for layer in range(layers):
        for q in range(n):
            ops.append(dict(kind="g", time=t, qs=[q], m=random_unitary(rng, 1)))
        for q in range(layer % 2, n - 1, 2):
            ops.append(dict(kind="g", time=t + 1, qs=[q, q + 1],
                            m=random_unitary(rng, 2)))
        qs = sorted(rng.choice(np.arange(2, n), size=2, replace=False).tolist())
        ops.append(dict(kind="Q", time=t + 2, qs=qs, p=0.3))
        t += 3
    return ops


def traj_cases():
    traj_case("traj_depol8", 8, noisy_chain_ops(8, 4, 3, 0.05, 0.0), 2, 0, 48)
    traj_case("traj_ad8", 8, noisy_chain_ops(8, 4, 4, 0.02, 0.1), 3, 0, 48)
    rng = np.random.default_rng(99)
    traj_case("traj_mixed6", 6, mixed_noisy_ops(rng, 6, 5), 2, 0, 40)
    # The batched-trajectory workload's noise model at n = 12, depth 12.
    traj_case("traj_chain12", 12, noisy_chain_ops(12, 12, 5, 1e-3, 5e-3), 4,
              0, 8, states_c64=True)
    traj_depol_register_case()


def traj_depol_register_case():
    rng = np.random.default_rng(123)
    traj_case("traj_depol2q_reg", 6, depol_register_ops(rng, 6, 5), 2, 0, 40)


def unitary_case(name, n, ops):
    """The reference's UnitaryCalculatorBasic<double> from the identity:
    4^n complex entries, entry (i, j) at i * 2^n + j."""
    with tempfile.TemporaryDirectory() as td:
        gl = os.path.join(td, "gates.txt")
        write_gate_list(gl, n, ops)
        out = os.path.join(td, "u.f64")
        subprocess.run([DRIVER, "unitary", gl, out], check=True)
        u = np.fromfile(out, dtype=np.float64).view(np.complex128)
        data = dict(n=np.int32(n), u64=u, **pack_ops(ops))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)


def small_gate_list(rng, n, ngates, kmax, ctrl_frac):
    """Gates of 1..kmax targets; with probability ctrl_frac 1..2 controls
    (targets + controls <= n)."""
    ops = []
    for t in range(ngates):
        k = int(rng.integers(1, kmax + 1))
        if n - k >= 1 and rng.random() < ctrl_frac:
            c = int(rng.integers(1, min(2, n - k) + 1))
            picks = rng.choice(n, size=k + c, replace=False).tolist()
            ops.append(dict(kind="c", time=t, qs=sorted(picks[:k]),
                            cqs=sorted(picks[k:]),
                            cvals=int(rng.integers(0, 1 << c)),
                            m=random_unitary(rng, k)))
        else:
            qs = sorted(rng.choice(n, size=k, replace=False).tolist())
            ops.append(dict(kind="g", time=t, qs=qs, m=random_unitary(rng, k)))
    return ops


def unitary_cases():
    rng = np.random.default_rng(7070)
    unitary_case("unitary3", 3, small_gate_list(rng, 3, 10, 2, 0.3))
    unitary_case("unitary5", 5, small_gate_list(rng, 5, 24, 3, 0.3))
    unitary_case("unitary7", 7, small_gate_list(rng, 7, 30, 4, 0.2))


def random_hybrid_text(rng, n, layers, parts, max_cut):
    """One- and two-qubit named gates only (the hybrid simulator's gate set),
    two-qubit gates on random pairs in random order, at most `max_cut` of
    them across the cut (each cut gate adds up to two path bits), angles
    exact in float."""
    lines = [str(n)]
    cut = 0
    for t in range(layers):
        perm = rng.permutation(n).tolist()
        used = set()
        for i, q in enumerate(perm):
            if q in used:
                continue
            used.add(q)
            free = [p for p in perm[i + 1:] if p not in used]
            same = [p for p in free if parts[p] == parts[q]]
            other = [p for p in free if parts[p] != parts[q]]
            r = rng.random()
            ang = lambda: f"{int(rng.integers(-400, 400)) / 64}"
            two = r >= 0.45 and (same or (other and cut < max_cut))
            if not two:
                if r < 0.3:
                    g = GATES_1Q[int(rng.integers(len(GATES_1Q)))]
                    lines.append(f"{t} {g} {q}")
                else:
                    g, npar = GATES_1Q_P[int(rng.integers(len(GATES_1Q_P)))]
                    lines.append(f"{t} {g} {q} " + " ".join(ang() for _ in range(npar)))
                continue
            pool = other if (other and cut < max_cut and rng.random() < 0.5) or not same else same
            p2 = pool[int(rng.integers(len(pool)))]
            used.add(p2)
            if parts[p2] != parts[q]:
                cut += 1
            a, b = (q, p2) if rng.random() < 0.5 else (p2, q)
            if rng.random() < 0.6:
                g = GATES_2Q[int(rng.integers(len(GATES_2Q)))]
                lines.append(f"{t} {g} {a} {b}")
            else:
                g, npar = GATES_2Q_P[int(rng.integers(len(GATES_2Q_P)))]
                # fs angles with sin(theta) >= 0 (the reference's fs
                # decomposition takes sqrt(sin(theta))).
                ps = [f"{int(rng.integers(0, 200)) / 64}"] if g == "fs" else []
                ps += [ang() for _ in range(npar - len(ps))]
                lines.append(f"{t} {g} {a} {b} " + " ".join(ps))
    return "\n".join(lines) + "\n"


def hybrid_run(text, parts, np_, nr, prefix, bitstrings):
    with tempfile.TemporaryDirectory() as td:
        cp = os.path.join(td, "c.txt")
        bp = os.path.join(td, "b.u64")
        op = os.path.join(td, "out")
        with open(cp, "w") as f:
            f.write(text)
        np.asarray(bitstrings, np.uint64).tofile(bp)
        subprocess.run([DRIVER, "hybrid", cp, op, str(np_), str(nr), str(prefix),
                        ",".join(str(int(x)) for x in parts), bp], check=True)
        return np.fromfile(op, np.complex128)


def hybrid_known_case():
    """The reference's own hybrid known-answer tests
    (tests/hybrid_testfixture.h: circuits, parts, runs and EXPECT_NEAR
    values), read from the reference's test file, checked against the
    reference driver here and stored as a fixture."""
    import re
    src = open(os.path.join(REF_ROOT, "tests", "hybrid_testfixture.h")).read()
    bodies = src.split("void TestHybrid")[1:]
    cases = []
    for body in bodies:
        text = re.search(r'R"\((.*?)\)"', body, re.S).group(1)
        text = text.lstrip("\n")
        parts = [int(x) for x in re.search(
            r"std::vector<unsigned> parts = \{([^}]*)\};", body).group(1).split(",")]
        nres = int(re.search(r"results\((\d+), 0\)", body).group(1))
        counts = [int(re.search(r"EXPECT_EQ\(hd\.%s(?:\.size\(\))?, (\d+)\);" % k,
                                body).group(1))
                  for k in ("ops0", "ops1", "gatexs", "num_qubits0", "num_qubits1")]
        runs, cur = [], {}
        for line in body.splitlines():
            m = re.search(r"param\.(prefix|num_prefix_gatexs|num_root_gatexs) = (\d+);", line)
            if m:
                cur[m.group(1)] = int(m.group(2))
            if "HybridSimulator(1).Run(" in line:
                runs.append(dict(cur, want=np.zeros(nres, np.complex128),
                                 seen=np.zeros((nres, 2), bool)))
            m = re.search(r"EXPECT_NEAR\(std::(real|imag)\(results\[(\d+)\]\), "
                          r"([-0-9.e]+), ", line)
            if m and runs:
                i, v = int(m.group(2)), float(m.group(3))
                if m.group(1) == "real":
                    runs[-1]["want"][i] += v
                    runs[-1]["seen"][i, 0] = True
                else:
                    runs[-1]["want"][i] += 1j * v
                    runs[-1]["seen"][i, 1] = True
        for r in runs:
            k = int(r["seen"].all(axis=1).sum())   # results with expectations
            got = hybrid_run(text, parts, r["num_prefix_gatexs"],
                             r["num_root_gatexs"], r["prefix"], range(k))
            assert np.abs(got - r["want"][:k]).max() < 1e-6, (got, r["want"])
            cases.append(dict(text=text, parts=parts, counts=counts,
                              prefix=r["prefix"],
                              np=r["num_prefix_gatexs"], nr=r["num_root_gatexs"],
                              want=r["want"][:k]))
    out = {}
    for i, c in enumerate(cases):
        for key, v in c.items():
            out[f"{key}{i}"] = np.array(v)
    np.savez_compressed(os.path.join(HERE, "hybrid_known.npz"),
                        count=np.int32(len(cases)), **out)
    print("hybrid_known written:", len(cases), "runs")


def hybrid_random_cases():
    """Seeded circuits of 6..10 qubits: parts contiguous or interleaved,
    prefix / root / suffix splits including a nonzero prefix; amplitudes of
    every bitstring (n <= 8) or 256 random ones, from the reference."""
    rng = np.random.default_rng(4242)
    specs = [("hybrid6", 6, 10, [0, 0, 0, 1, 1, 1], [(0, 0, 0), (0, 2, 0), (2, 1, 1)]),
             ("hybrid8", 8, 12, [0, 1, 0, 1, 1, 0, 0, 1], [(0, 0, 0), (1, 2, 0), (3, 0, 2)]),
             ("hybrid10", 10, 14, [0] * 5 + [1] * 5, [(0, 0, 0), (0, 3, 0), (2, 2, 2)])]
    for name, n, layers, parts, runs in specs:
        text = random_hybrid_text(rng, n, layers, parts, 7)
        if n <= 8:
            bits = np.arange(1 << n, dtype=np.uint64)
        else:
            bits = rng.choice(1 << n, 256, replace=False).astype(np.uint64)
        res = []
        for np_, nr, prefix in runs:
            res.append(hybrid_run(text, parts, np_, nr, prefix, bits))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), n=np.int32(n),
                            text=np.array(text), parts=np.array(parts, np.uint32),
                            runs=np.array(runs, np.uint64), bits=bits,
                            amps=np.array(res))
        print(name, "written")


# ---- qsim_cuda-compatible module (pybind_interface) ----------------------
# Circuits are described as data (JSON) and built through the module API, so
# the same description drives the reference's module (built from its
# sources by `make -C oracle pybind`) here and qsim_gb300.qsim_cuda in the
# tests.

_EXP = ("exponent", "global_shift")
PARAM_KINDS = {
    "kXPowGate": _EXP, "kYPowGate": _EXP, "kZPowGate": _EXP, "kHPowGate": _EXP,
    "kCZPowGate": _EXP, "kCXPowGate": _EXP, "krx": ("phi",), "kry": ("phi",),
    "krz": ("phi",), "kPhasedXPowGate": ("phase_exponent",) + _EXP,
    "kPhasedXZGate": ("x_exponent", "z_exponent", "axis_phase_exponent"),
    "kXXPowGate": _EXP, "kYYPowGate": _EXP, "kZZPowGate": _EXP,
    "kSwapPowGate": _EXP, "kISwapPowGate": _EXP, "kriswap": ("phi",),
    "kPhasedISwapPowGate": ("phase_exponent", "exponent"), "kgivens": ("phi",),
    "kFSimGate": ("theta", "phi"), "kCCZPowGate": _EXP, "kCCXPowGate": _EXP,
}
KIND_QUBITS = {
    "kI1": 1, "kI2": 2, "kXPowGate": 1, "kYPowGate": 1, "kZPowGate": 1,
    "kHPowGate": 1, "kCZPowGate": 2, "kCXPowGate": 2, "krx": 1, "kry": 1,
    "krz": 1, "kH": 1, "kS": 1, "kCZ": 2, "kCX": 2, "kT": 1, "kX": 1, "kY": 1,
    "kZ": 1, "kPhasedXPowGate": 1, "kPhasedXZGate": 1, "kXXPowGate": 2,
    "kYYPowGate": 2, "kZZPowGate": 2, "kXX": 2, "kYY": 2, "kZZ": 2,
    "kSwapPowGate": 2, "kISwapPowGate": 2, "kriswap": 2, "kSWAP": 2,
    "kISWAP": 2, "kPhasedISwapPowGate": 2, "kgivens": 2, "kFSimGate": 2,
    "kCCZPowGate": 3, "kCCXPowGate": 3, "kCSwapGate": 3, "kCCZ": 3, "kCCX": 3,
}


def build_module_circuit(mod, n, desc):
    c = mod.Circuit()
    c.num_qubits = n
    for d in desc:
        if d["t"] == "gate":
            mod.add_gate(getattr(mod, d["kind"]), d["time"], d["qubits"], d["params"], c)
        elif d["t"] == "diag":
            mod.add_diagonal_gate(d["time"], d["qubits"], d["angles"], c)
        elif d["t"] == "matrix":
            mod.add_matrix_gate(d["time"], d["qubits"], d["matrix"], c)
        elif d["t"] == "ctrl":
            mod.control_last_gate(d["qubits"], d["values"], c)
        elif d["t"] == "meas":
            mod.add_measurement(d["time"], d["qubits"], c)
        elif d["t"] == "chan":
            mod.add_channel(d["time"], d["qubits"],
                            [(p, m, u) for p, m, u in d["kops"]], c)
    return c


def build_module_opsums(mod, spec):
    out = []
    for strings, count in spec:
        ops = []
        for weight, terms in strings:
            s = mod.OpString()
            s.weight = complex(*weight)
            for kind, qs in terms:
                mod.add_gate_to_opstring(getattr(mod, kind), qs, s)
            ops.append(s)
        out.append((ops, count))
    return out


def random_module_gate(rng, n, time, kinds=None):
    kinds = kinds or list(KIND_QUBITS)
    kind = kinds[int(rng.integers(len(kinds)))]
    qs = rng.permutation(n)[:KIND_QUBITS[kind]].tolist()
    ps = {p: float(np.float32(rng.uniform(-1.5, 1.5))) for p in PARAM_KINDS.get(kind, ())}
    return dict(t="gate", kind=kind, time=time, qubits=qs, params=ps)


def random_module_circuit(rng, n, layers, measure_at=()):
    """Every op at its own time step (the reference's fuser needs the gates
    of each qubit in time order)."""
    desc = [dict(t="gate", kind="kH", time=0, qubits=[q], params={}) for q in range(n)]
    t = 1
    for layer in range(layers):
        for _ in range(max(1, n // 2)):
            desc.append(random_module_gate(rng, n, t))
            t += 1
            r = rng.random()
            if r < 0.1 and KIND_QUBITS[desc[-1]["kind"]] < n - 1:
                free = [q for q in range(n) if q not in desc[-1]["qubits"]]
                cq = rng.permutation(free)[:1 + int(rng.integers(2))].tolist()
                desc.append(dict(t="ctrl", qubits=cq,
                                 values=rng.integers(0, 2, len(cq)).tolist()))
            elif r < 0.2:
                k = 2 + int(rng.integers(2))
                qs = rng.permutation(n)[:k].tolist()
                na = int(rng.integers(1, (1 << k) + 1))
                desc.append(dict(t="diag", time=t, qubits=qs,
                                 angles=rng.uniform(-3, 3, na).tolist()))
                t += 1
            elif r < 0.3:
                k = 1 + int(rng.integers(3))
                qs = rng.permutation(n)[:k].tolist()
                m = interleave(random_unitary(rng, k)).astype(np.float32)
                desc.append(dict(t="matrix", time=t, qubits=qs, matrix=m.tolist()))
                t += 1
        if layer in measure_at:
            desc.append(dict(t="meas", time=t, qubits=rng.permutation(n)[:3].tolist()))
            t += 1
    return desc


def random_pauli_opsums(rng, n, count, wmax, big=None):
    spec = []
    for _ in range(count):
        strings = []
        for _ in range(1 + int(rng.integers(3))):
            w = 1 + int(rng.integers(wmax))
            qs = rng.permutation(n)[:w].tolist()
            terms = [[["kX", "kY", "kZ"][int(rng.integers(3))], [q]] for q in qs]
            strings.append([[float(rng.uniform(-1, 1)), float(rng.uniform(-1, 1))], terms])
        cnt = len({q for _, ts in strings for _, qq in ts for q in qq})
        spec.append([strings, cnt])
    if big:
        qs = rng.permutation(n)[:big].tolist()
        terms = [[["kX", "kY", "kZ"][int(rng.integers(3))], [q]] for q in qs]
        spec.append([[[[0.5, 0.25], terms]], big])
    spec.append([[[[0.75, 0.0], []]], 0])          # identity: EV = weight
    return spec


def _flat(m):
    return interleave(np.asarray(m, np.complex128)).astype(np.float32).tolist()


def random_noisy_module_circuit(rng, n, layers, measure=False):
    """Every op at its own time step; after each gate a channel on one of
    its qubits: a Pauli mixture (unitary), amplitude damping (non-unitary,
    lower bounds 1 - gamma and 0) or, for two-qubit gates, a mixture of the
    identity and CZ."""
    px = np.array([[0, 1], [1, 0]])
    py = np.array([[0, -1j], [1j, 0]])
    pz = np.diag([1, -1])
    desc = [dict(t="gate", kind="kH", time=0, qubits=[q], params={}) for q in range(n)]
    t = 1
    for layer in range(layers):
        for _ in range(max(1, n // 2)):
            g = random_module_gate(rng, n, t, [k for k in KIND_QUBITS
                                               if KIND_QUBITS[k] <= 2])
            desc.append(g)
            t += 1
            q = g["qubits"][0]
            r = rng.random()
            if r < 0.4:
                p = float(np.float32(0.02 + 0.1 * rng.random()))
                kops = [[1 - 3 * p, _flat(np.eye(2)), True]]
                kops += [[p, _flat(m), True] for m in (px, py, pz)]
            elif r < 0.8:
                gam = float(np.float32(0.05 + 0.2 * rng.random()))
                kops = [[1 - gam, _flat(np.diag([1, np.sqrt(1 - gam)])), False],
                        [0.0, _flat(np.array([[0, np.sqrt(gam)], [0, 0]])), False]]
            else:
                if len(g["qubits"]) < 2:
                    continue
                cz = np.diag([1, 1, 1, -1])
                p = float(np.float32(0.1 + 0.2 * rng.random()))
                desc.append(dict(t="chan", time=t, qubits=g["qubits"],
                                 kops=[[1 - p, _flat(np.eye(4)), True],
                                       [p, _flat(cz), True]]))
                t += 1
                continue
            desc.append(dict(t="chan", time=t, qubits=[q], kops=kops))
            t += 1
        if measure and layer in (1, layers - 1):
            desc.append(dict(t="meas", time=t, qubits=rng.permutation(n)[:3].tolist()))
            t += 1
    return desc


def noisy_module_case(ref, rng, opts):
    n = 6
    desc = random_noisy_module_circuit(rng, n, 5)
    c = build_module_circuit(ref, n, desc)
    vec = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    vec = (vec / np.linalg.norm(vec)).astype(np.complex64).view(np.float32)
    out = dict(n=n, desc=desc, vec=vec.tolist(), fs={}, fs_vec={}, amps={},
               samples={})
    bits = rng.choice(1 << n, 8, replace=False)
    btxt = "\n".join("".join(str((int(b) >> q) & 1) for q in range(n)) for b in bits)
    out["btxt"] = btxt
    for seed in (1, 2, 3, 4, 5, 6):
        out["fs"][str(seed)] = np.array(
            ref.qtrajectory_simulate_fullstate(opts(c, s=seed, r=1), 0)).tolist()
        out["fs_vec"][str(seed)] = np.array(
            ref.qtrajectory_simulate_fullstate(opts(c, s=seed, r=1), vec)).tolist()
        out["amps"][str(seed)] = [[a.real, a.imag] for a in
                                  ref.qtrajectory_simulate(opts(c, s=seed, i=btxt))]
        out["samples"][str(seed)] = [int(x) for x in
                                     ref.qtrajectory_sample_final(opts(c, s=seed, r=1), 200)]
    spec = random_pauli_opsums(rng, n, 4, 3)
    out["opsums"] = spec
    evs = ref.qtrajectory_simulate_expectation_values(
        opts(c, r=8), build_module_opsums(ref, spec), 0)
    out["evs"] = [[e.real, e.imag] for e in evs]
    nops = sum(1 for d in desc if d["t"] != "ctrl")
    moments = [[nops // 2, random_pauli_opsums(rng, n, 2, 2)],
               [nops, random_pauli_opsums(rng, n, 2, 2)]]
    out["moments"] = moments
    mevs = ref.qtrajectory_simulate_moment_expectation_values(
        opts(c, r=4), [(end, build_module_opsums(ref, sp)) for end, sp in moments], 0)
    out["mevs"] = [[[e.real, e.imag] for e in row] for row in mevs]
    mdesc = random_noisy_module_circuit(rng, n, 4, measure=True)
    mc = build_module_circuit(ref, n, mdesc)
    out["mdesc"] = mdesc
    out["mbits"] = {str(seed): [int(b) for b in ref.qtrajectory_sample(opts(mc, s=seed))]
                    for seed in (1, 2, 3, 4)}
    assert all(out["mbits"].values()) and out["evs"] and out["mevs"]
    assert all(out["samples"].values()) and all(out["fs"].values())
    return out


# Cirq two-qubit gates with a Schmidt decomposition in the reference
# (lib/gates_cirq.h GetSchmidtDecomp), the ones qsimh accepts on the cut.
SCHMIDT_KINDS = ["kI2", "kCZPowGate", "kCXPowGate", "kCZ", "kCX", "kXXPowGate",
                 "kYYPowGate", "kZZPowGate", "kXX", "kYY", "kZZ", "kSwapPowGate",
                 "kISwapPowGate", "kriswap", "kSWAP", "kISWAP",
                 "kPhasedISwapPowGate", "kgivens", "kFSimGate"]


def hybrid_module_case(ref, rng, opts):
    n = 8
    parts = [0, 0, 0, 0, 1, 1, 1, 1]
    ones = [k for k, v in KIND_QUBITS.items() if v == 1]
    desc = [dict(t="gate", kind="kH", time=0, qubits=[q], params={}) for q in range(n)]
    t, cut = 1, 0
    for _ in range(10):
        for _ in range(4):
            if rng.random() < 0.4:
                g = random_module_gate(rng, n, t, ones)
            else:
                g = random_module_gate(rng, n, t, SCHMIDT_KINDS)
                a, b = g["qubits"]
                if parts[a] != parts[b]:
                    if cut >= 6:
                        continue
                    cut += 1
                if g["kind"] == "kFSimGate":
                    g["params"]["theta"] = float(np.float32(rng.uniform(0, 3)))
            desc.append(g)
            t += 1
    c = build_module_circuit(ref, n, desc)
    bits = rng.choice(1 << n, 32, replace=False)
    btxt = "\n".join("".join(str((int(b) >> q) & 1) for q in range(n)) for b in bits)
    runs = []
    for p, r, w in ((0, 0, 0), (0, 2, 0), (2, 1, 1), (3, 0, 2), (1, 1, 3)):
        amps = ref.qsimh_simulate(opts(c, i=btxt, k=[4, 5, 6, 7], w=w, p=p, r=r))
        assert amps, (p, r, w)
        runs.append(dict(p=p, r=r, w=w, amps=[[a.real, a.imag] for a in amps]))
    return dict(n=n, desc=desc, btxt=btxt, k=[4, 5, 6, 7], cut=cut, runs=runs)


def pybind_cases():
    import json
    sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
    import qsim_basic as ref  # the reference's module, built from its sources

    def opts(c, **kw):
        return dict(dict(c=c, f=2, s=1, t=1, v=0, z=0), **kw)

    rng = np.random.default_rng(9090)
    out = {}
    # One circuit per gate kind: a generic 4-qubit state, then the gate.
    kinds = []
    for kind in KIND_QUBITS:
        desc = [dict(t="gate", kind="kH", time=0, qubits=[q], params={}) for q in range(4)]
        desc += [dict(t="gate", kind="krx", time=1, qubits=[q],
                      params={"phi": 0.3 + 0.4 * q}) for q in range(4)]
        desc += [dict(t="gate", kind="kCZ", time=2, qubits=[0, 1], params={}),
                 dict(t="gate", kind="kCZ", time=2, qubits=[2, 3], params={})]
        desc.append(random_module_gate(rng, 4, 3, [kind]))
        fs = np.array(ref.qsim_simulate_fullstate(opts(build_module_circuit(ref, 4, desc)), 0))
        kinds.append(dict(desc=desc, fs=fs.tolist()))
    out["gate_kinds"] = json.dumps(kinds)
    # A 10-qubit circuit of every builder.
    n = 10
    desc = random_module_circuit(rng, n, 12)
    c = build_module_circuit(ref, n, desc)
    vec = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    vec = (vec / np.linalg.norm(vec)).astype(np.complex64).view(np.float32)
    bits = rng.choice(1 << n, 16, replace=False)
    btxt = "\n".join("".join(str((int(b) >> q) & 1) for q in range(n)) for b in bits)
    ops_spec = random_pauli_opsums(rng, n, 6, 4, big=8)
    nops = sum(1 for d in desc if d["t"] != "ctrl")   # control_last_gate adds none
    moments = [[nops // 2, random_pauli_opsums(rng, n, 2, 3)],
               [nops, random_pauli_opsums(rng, n, 2, 3)]]
    mix = dict(n=n, desc=desc, bits=[int(b) for b in bits], btxt=btxt,
               vec=vec.tolist(), opsums=ops_spec, moments=moments)
    mix["fs0"] = np.array(ref.qsim_simulate_fullstate(opts(c), 0)).tolist()
    mix["fs_vec"] = np.array(ref.qsim_simulate_fullstate(opts(c), vec)).tolist()
    mix["fs_basis"] = np.array(ref.qsim_simulate_fullstate(opts(c), 37)).tolist()
    mix["amps"] = [[a.real, a.imag] for a in ref.qsim_simulate(opts(c, i=btxt))]
    mix["samples"] = [int(x) for x in ref.qsim_sample_final(opts(c, s=5), 500)]
    evs = ref.qsim_simulate_expectation_values(opts(c), build_module_opsums(ref, ops_spec), 0)
    mix["evs"] = [[e.real, e.imag] for e in evs]
    mevs = ref.qsim_simulate_moment_expectation_values(
        opts(c), [(end, build_module_opsums(ref, sp)) for end, sp in moments], 0)
    mix["mevs"] = [[[e.real, e.imag] for e in row] for row in mevs]
    assert mix["amps"] and mix["samples"] and mix["evs"] and mix["mevs"]
    out["mixed"] = json.dumps(mix)
    # Measurements inside the circuit: qsim_sample's bits.
    n = 6
    desc = random_module_circuit(rng, n, 6, measure_at=(2, 5))
    c = build_module_circuit(ref, n, desc)
    meas = dict(n=n, desc=desc, seeds={})
    for seed in (1, 2, 3):
        meas["seeds"][str(seed)] = [int(b) for b in ref.qsim_sample(opts(c, s=seed))]
        assert meas["seeds"][str(seed)]
    out["measure"] = json.dumps(meas)
    # Noisy circuits: gates, Pauli-mixture and amplitude-damping channels on
    # one qubit, a two-qubit unitary mixture, measurements.
    out["noisy"] = json.dumps(noisy_module_case(ref, rng, opts))
    out["hybrid"] = json.dumps(hybrid_module_case(ref, rng, opts))
    out["names"] = json.dumps(sorted(x for x in dir(ref) if not x.startswith("_")))
    out["kind_values"] = json.dumps({x: int(getattr(ref, x)) for x in dir(ref)
                                     if x.startswith("k")})
    np.savez_compressed(os.path.join(HERE, "pybind_module.npz"),
                        **{k: np.array(v) for k, v in out.items()})
    print("pybind_module written")


def main():
    if not os.path.exists(DRIVER):
        sys.exit(f"{DRIVER} missing: run `make -C oracle ref` first")
    if sys.argv[1:] == ["traj"]:
        traj_cases()
        return
    if sys.argv[1:] == ["traj_depol_register"]:
        traj_depol_register_case()
        return
    if sys.argv[1:] == ["unitary"]:
        unitary_cases()
        return
    if sys.argv[1:] == ["pybind"]:
        pybind_cases()
        return
    if sys.argv[1:] == ["mt"]:
        mt_case()
        return
    if sys.argv[1:] == ["refplan"]:
        ref_plan_case()
        return
    if sys.argv[1:] == ["hybrid"]:
        hybrid_known_case()
        hybrid_random_cases()
        return
    mt_case()
    text_case("text_gates9", 9, 30, 5)
    fuse_counts_case()
    config1_case()
    rng = np.random.default_rng(20261204)
    # k = 1..6 gates at random positions (covers low/high targets, pair and
    # non-pair layouts), FP32 fused at f=4, EVs of Pauli strings up to 6.
    ops = random_gate_list(rng, 12, 48, 6)
    run_case("rand12_k6", 12, ops, 4, 2000, 7,
             evs=random_pauli_evs(rng, 12, 24, 6))
    # Controlled gates with 1..3 controls and 1..3 targets.
    ops = random_gate_list(rng, 11, 40, 3, ctrl_frac=0.5)
    run_case("ctrl11", 11, ops, 3, 1000, 11)
    # Small states (n = 1..6) with gates up to k = n.
    for n in (1, 3, 6):
        ops = random_gate_list(rng, n, 12, min(n, 4))
        run_case(f"small{n}", n, ops, 2, 500, 3,
                 evs=random_pauli_evs(rng, n, 4, min(n, 3)))
    # Larger state, depth typical of the configs, measurement golden.
    ops = random_gate_list(rng, 14, 60, 2)
    run_case("rand14_k2", 14, ops, 2, 4000, 1,
             measure=(17, 6, [0, 5, 13]))
    traj_cases()
    unitary_cases()
    hybrid_known_case()
    hybrid_random_cases()
    pybind_cases()
    ref_plan_case()


if __name__ == "__main__":
    main()
