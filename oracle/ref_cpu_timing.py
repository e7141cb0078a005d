"""Times the reference's own CPU path for the 30-qubit 5x6 grid depth-20
circuit (seed 1) where the reference checkout is present, beside the
oracle's FP32 port on the same cores.  TEST INFRASTRUCTURE: the numbers are
recorded as the CPU baselines of this path; nothing here is product code.

  make -C oracle ref refbench
  python oracle/ref_cpu_timing.py [--reps 3] [--threads N] [--rows 5 --cols 6]

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
    args = ap.parse_args()
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import read_ref_plan, write_gate_list
    from qsim_gb300 import engine as E
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
