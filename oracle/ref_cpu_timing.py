"""Times the reference's own CPU path for the 30-qubit 5x6 grid depth-20
circuit (seed 1) where the reference checkout is present, beside the
oracle's FP32 port on the same cores.  TEST INFRASTRUCTURE: the numbers are
recorded as the CPU baselines of this path; nothing here is product code.

  make -C oracle ref refbench
  python oracle/ref_cpu_timing.py [--reps 3] [--threads N] [--rows 5 --cols 6]
  python oracle/ref_cpu_timing.py --traj [--reps 3] [--threads N]

Arms (one JSON line each):
  reference_avx512  QSimRunner + MultiQubitGateFuser(max_fused_size 4) +
                    SimulatorAVX512 (lib/simmux.h on this x86 host), the
                    reference's release flags (-O3 -fopenmp), ParallelFor
                    over all threads; seconds of Run (fusion + every fused
                    gate), median of the reps (lib/run_qsim.h:225-289).
  reference_sse     the same with SimulatorSSE (128-bit vectors, the x86
                    counterpart of the NEON simulator an Arm host selects).
  port              the oracle's lane-batched FP32 gate application
                    (orc_port_apply_gate_f32) over the reference's fused
                    gates (ref_driver plan), the CPU baseline that also
                    runs where the reference is absent.

With --traj, the batched noisy-trajectory workload instead (4096
trajectories: 128 chain circuits of 12..24 qubits, depth 12, depolarizing
after every gate qubit, amplitude damping on every qubit per cycle): for
each qubit count the first circuit of that size, `--reps` repetitions
through the reference's QuantumTrajectorySimulator::RunBatch on
SimulatorAVX512 (ref_driver trajbench, max_fused_size 2 as its Parameter
defaults), and through the oracle's port of RunIteration on the same
cores; the batch time is estimated as the sum over the 128 circuits of 32
x the mean time at the circuit's qubit count.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--rows", type=int, default=5)
    ap.add_argument("--cols", type=int, default=6)
    ap.add_argument("--cycles", type=int, default=20)
    ap.add_argument("--fsize", type=int, default=4)
    ap.add_argument("--traj", action="store_true")
    args = ap.parse_args()
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import read_ref_plan, write_gate_list
    from qsim_gb300 import engine as E
    if args.traj:
        traj(args, E, write_gate_list)
        return
    c = E.Circuit.grid(args.rows, args.cols, 0, args.cycles, 1)
    n = c.num_qubits
    ops = [dict(kind="g", time=o["time"], qs=o["qs"], m=o["m"]) for o in c.ops()]
    common = {"workload": f"grid{args.rows}x{args.cols} ({n} qubits) depth "
                          f"{args.cycles}, seed 1, max_fused_size {args.fsize}",
              "threads": args.threads, "host": os.uname().machine,
              "cpu": _cpu_name()}
    with tempfile.TemporaryDirectory() as td:
        gl = os.path.join(td, "g.txt")
        write_gate_list(gl, n, ops)
        for arm, exe in (("reference_avx512", "ref_bench_avx512"),
                         ("reference_sse", "ref_bench_sse")):
            path = os.path.join(HERE, "_ref", exe)
            r = subprocess.run([path, "bench", gl, str(args.fsize),
                                str(args.reps), str(args.threads)],
                               check=True, capture_output=True, text=True)
            rows = [list(map(float, ln.split())) for ln in r.stdout.split("\n")
                    if ln.strip()]
            print(json.dumps(dict(common, arm=arm,
                                  run_s=[x[0] for x in rows],
                                  median_s=statistics.median(x[0] for x in rows),
                                  fuse_s=statistics.median(x[1] for x in rows),
                                  fused_gates=int(rows[0][2]))), flush=True)
        planf = os.path.join(td, "plan.bin")
        subprocess.run([os.path.join(HERE, "_ref", "ref_driver"), "plan", gl,
                        str(args.fsize), planf], check=True)
        ks, qs, ms = read_ref_plan(planf)
    L = C.CDLL(os.path.join(HERE, "_build", "liboracle.so"))
    P = C.POINTER
    L.orc_port_apply_gate_f32.argtypes = [P(C.c_float), C.c_uint, P(C.c_uint),
                                          C.c_uint, P(C.c_float)]
    L.orc_set_num_threads(args.threads)
    gates, qo, mo = [], 0, 0
    for k in ks:
        q = (C.c_uint * max(1, k))(*qs[qo:qo + k])
        m = np.ascontiguousarray(ms[mo:mo + 2 * 4 ** k])
        gates.append((int(k), q, m))
        qo += k
        mo += 2 * 4 ** k
    st = np.zeros(2 << n, np.float32)
    times = []
    for _ in range(args.reps):
        st[:] = 0
        st[0] = 1
        t0 = time.perf_counter()
        for k, q, m in gates:
            L.orc_port_apply_gate_f32(st.ctypes.data_as(P(C.c_float)), n, q, k,
                                      m.ctypes.data_as(P(C.c_float)))
        times.append(time.perf_counter() - t0)
    print(json.dumps(dict(common, arm="port", run_s=times,
                          median_s=statistics.median(times),
                          fused_gates=len(ks))), flush=True)


def noisy_gate_list(clean, n, p_depol, gamma, cycle_len=2):
    """The trajectory workload's noisy circuit as ref_driver gate-list
    entries: each gate at time 3t, then a depolarizing channel on each of
    its qubits at 3t + 1 (lib/circuit_noisy.h:33-64 with its times spread
    to leave room for a second channel), and after the last gate of each
    cycle of `cycle_len` time steps amplitude damping on every qubit at
    3t + 2 (the rule of oracle/traj_port.py noisy_ops).  The reference's
    fuser rejects two deferred operators on one qubit at one time, which a
    depolarizing and a damping channel at the same time would give."""
    ops = []
    for i, o in enumerate(clean):
        t = int(o["time"])
        ops.append(dict(kind="g", time=3 * t, qs=list(o["qs"]), m=o["m"]))
        for q in o["qs"]:
            ops.append(dict(kind="D", time=3 * t + 1, qs=[int(q)], p=p_depol))
        last = (i + 1 == len(clean)
                or clean[i + 1]["time"] // cycle_len != t // cycle_len)
        if gamma > 0 and last:
            for q in range(n):
                ops.append(dict(kind="A", time=3 * t + 2, qs=[q], p=gamma))
    return ops


def traj(args, E, write_gate_list):
    sys.path.insert(0, HERE)
    import bench
    import traj_port
    T = bench.TRAJ
    rng = np.random.default_rng(T["seed"])
    ns = rng.integers(T["n_min"], T["n_max"] + 1, size=T["circuits"])
    circuits = [(int(n), E.Circuit.chain(int(n), T["cycles"], 1000 + i).ops())
                for i, n in enumerate(ns)]
    first = {}
    for n, clean in circuits:
        first.setdefault(n, clean)
    ref_mean = {}
    with tempfile.TemporaryDirectory() as td:
        for n, clean in sorted(first.items()):
            gl = os.path.join(td, f"traj{n}.txt")
            write_gate_list(gl, n, noisy_gate_list(clean, n, T["p_depol"],
                                                   T["gamma"]))
            r = subprocess.run([os.path.join(HERE, "_ref", "ref_bench_avx512"),
                                "trajbench", gl, "2", str(args.reps),
                                str(args.threads)],
                               check=True, capture_output=True, text=True)
            ts = [float(x) for x in r.stdout.split()]
            ref_mean[n] = float(np.mean(ts))
    L = C.CDLL(os.path.join(HERE, "_build", "liboracle.so"))
    L.orc_set_num_threads(args.threads)
    L.orc_num_threads.restype = C.c_int
    port_total, _, port_mean = traj_port.time_batch(
        L, circuits, T["reps"], args.reps, T["p_depol"], T["gamma"], 2)
    ref_total = sum(T["reps"] * ref_mean[n] for n, _ in circuits)
    batch = T["circuits"] * T["reps"]
    common = {"workload": f"{batch} noisy trajectories: {T['circuits']} chain "
                          f"circuits of {T['n_min']}..{T['n_max']} qubits, "
                          f"depth {T['cycles']}",
              "threads": args.threads, "host": os.uname().machine,
              "cpu": _cpu_name(), "reps_per_qubit_count": args.reps}
    print(json.dumps(dict(common, arm="reference_avx512",
                          traj_per_s=batch / ref_total,
                          mean_s_by_n={str(k): v for k, v in ref_mean.items()})),
          flush=True)
    print(json.dumps(dict(common, arm="port", traj_per_s=batch / port_total,
                          mean_s_by_n={str(k): v for k, v in port_mean.items()})),
          flush=True)


def _cpu_name():
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


if __name__ == "__main__":
    main()
