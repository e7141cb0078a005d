#!/usr/bin/env python3
"""Headline benchmark: seconds per run of the 30-qubit depth-20 random grid
circuit (5x6 grid, sqrt(X)/sqrt(Y)/sqrt(W) + fSim(pi/2, pi/6), coupler
sequence A,B,C,D,C,D,A,B, seed 1) on one GB300, complex64 state (8 GiB)
from |0...0>.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One step = SetStateZero + every fused op of the plan, replayed from a CUDA
graph on a resident state (8 GiB > 129 MB L2, so no L2 flush is needed).
The headline form is the fastest engine form (tensor-core path and learned
planner when available); the plain CUDA-core f=4 form is timed beside it.
`e2e` is the same run through the public API with host buffers, as a user
runs QSimRunner::Run: fusion of the circuit, the plan applied through the C
ABI (matrices uploaded per launch), 1000 samples and the full final state
copied to pinned host memory on the GPU's NUMA node, inside each timed step.
`precision` states the error of the benched forms against the FP64 oracle.

Multi-GPU: the path does not shard (one state per GPU), so N > 1 runs N
independent replicas (one rank per GPU; `--gpus N` starts them itself when
no launcher did); value = whole-job seconds per run = slowest rank's time /
(N runs).

--impl reference times the reference's CPU path on the host cores: the
reference's own fused plan of the circuit (its MultiQubitGateFuser at f=4,
a fixture written by the reference compiled from its sources) applied by the
oracle's port of its SIMD gate kernels (the reference's code is not present
on the GPU host).  Each step is a bounded sample (the next gates of the
plan); the K steps time every gate, and value is the sum of the per-gate
times.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "30q d20 circuit s/run: tensor-core+learned fusion vs plain, F>=1-1e-6; traj/s"
UNIT = "s/run"
GRID = dict(rows=5, cols=6, extra=0, cycles=20, seed=1)
# Two-gate tensor-core passes for consecutive blocks whose 12-qubit tile has
# >= 2 run bits (measured 0.78-0.95 of two one-gate passes at 30 qubits; the
# planner pairs by the measured saving per run-bit count).
TC_PAIR_BITS = 2
WORKLOAD = "grid5x6 (30 qubits) random circuit depth 20, seed 1, complex64, from |0>"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed
    region (the process started here is the only one stopped)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or not f[0].isdigit() or int(f[0]) != self.gpu:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [s for s, p in zip(sm, power) if p > 0.3 * max(power)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(dist, world: int, units_per_rank: float, seconds: float):
    """Whole-job rate of `world` independent replicas that each process
    `units_per_rank` units: all units over the slowest rank's time."""
    return world * units_per_rank / max_over_ranks(dist, seconds)


def replica_seconds_per_unit(dist, world: int, units_per_rank: float,
                             seconds: float):
    """Whole-job seconds per unit of `world` independent replicas (the
    inverse of replica_rate)."""
    return max_over_ranks(dist, seconds) / (world * units_per_rank)


def self_launch(args) -> int | None:
    """--gpus N without a launcher: start N ranks with torch's launcher on
    this node (rendezvous on 127.0.0.1) and return its exit status.  Under
    a launcher, WORLD_SIZE must equal N."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if "WORLD_SIZE" in os.environ:
        if world != args.gpus:
            raise SystemExit(f"--gpus {args.gpus} but WORLD_SIZE={world}: "
                             "launch one rank per GPU")
        return None
    if args.gpus <= 1:
        return None
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={args.gpus}", "--master-addr=127.0.0.1",
           f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def traffic_from_profiles(n: int, kernel: str):
    """dram read+write bytes per launch of `kernel`, from its committed ncu
    summary (scaled from the capture's qubit count to n: traffic grows in
    proportion to the state)."""
    name = {"gate_tile_kernel": "gate_tile_k4_plain_pass.md",
            "tc_gate_kernel": "tc_gate_k6_pass.md",
            "tc_gate2_kernel": "tc_gate2_pair_pass.md"}.get(kernel)
    if name is None:
        return None
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    nq, tb = None, None
    for line in open(p):
        if line.startswith("capture_qubits:"):
            nq = int(line.split(":")[1])
        if line.startswith("dram_bytes_per_launch:"):
            tb = float(line.split(":")[1])
    if nq is None or tb is None:
        return None
    return tb * (2 ** (n - nq))


# --------------------------------------------------------------------------
REF_PLAN = os.path.join(ROOT, "tests", "golden", "ref_plan_grid5x6d20_f4.npz")


def load_ref_plan():
    """The reference's own fused plan of the headline circuit: its
    MultiQubitGateFuser at max_fused_size 4 with CalculateFusedMatrix
    matrices, written by the reference compiled from its sources
    (tests/golden/make_golden.py refplan).  Returns (n, [(k, qubits,
    float32 matrix)])."""
    import numpy as np
    d = np.load(REF_PLAN)
    gates, qo, mo = [], 0, 0
    for k in d["k"]:
        k = int(k)
        gates.append((k, [int(q) for q in d["qubits"][qo:qo + k]],
                      np.ascontiguousarray(d["matrices"][mo:mo + 2 * 4 ** k])))
        qo += k
        mo += 2 * 4 ** k
    return int(d["n"]), gates


def oracle_lib():
    """The oracle's shared library (CPU restatement; the timed CPU baseline
    and the FP64 checker)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import Oracle
    orc = Oracle()
    return orc, orc.L


class CpuPort:
    """The oracle's lane-batched FP32 port of the reference's SIMD gate
    application (orc_port_apply_gate_f32) on an n-qubit host state, every
    host core (OpenMP), |0...0> at the start."""

    def __init__(self, n: int, threads: int | None = None):
        import numpy as np
        _, self.L = oracle_lib()
        if threads:
            self.L.orc_set_num_threads(threads)
        self.threads = self.L.orc_num_threads()
        self.n = n
        self.st = np.zeros(2 << n, dtype=np.float32)
        self.st[0] = 1.0
        self.sp = self.st.ctypes.data_as(C.POINTER(C.c_float))

    def apply(self, gate) -> float:
        k, qs, m = gate
        qa = (C.c_uint * max(1, k))(*qs)
        t0 = time.perf_counter()
        self.L.orc_port_apply_gate_f32(self.sp, self.n, qa, k,
                                       m.ctypes.data_as(C.POINTER(C.c_float)))
        return time.perf_counter() - t0


def cpu_full_run(max_seconds: float = 240.0):
    """Every fused gate of the reference's plan applied once, in order, on
    an 8 GiB FP32 host state: seconds per run (stops early, and says so,
    beyond `max_seconds`)."""
    n, gates = load_ref_plan()
    port = CpuPort(n)
    port.apply(gates[0])          # page faults of the state, untimed
    port.st[:] = 0
    port.st[0] = 1.0
    total, done = 0.0, 0
    for g in gates:
        total += port.apply(g)
        done += 1
        if total > max_seconds:
            break
    value = total * len(gates) / done
    sample = (f"every one of the reference's {len(gates)} fused gates "
              f"(MultiQubitGateFuser, max_fused_size 4, "
              f"tests/golden/ref_plan_grid5x6d20_f4.npz) applied once, in "
              f"order, on an 8 GiB FP32 host state by the oracle's "
              f"lane-batched port of the reference's SIMD gate kernels")
    if done < len(gates):
        sample += f"; stopped after {done} gates, extrapolated by gate count"
    return {"value": value, "unit": UNIT, "cores": port.threads,
            "kind": "port", "sample": sample, "gates_timed": done}


def fp64_precision(ctx, ss, c, plans):
    """The checker of the benched forms: relative L2 and fidelity of each
    plan's final state (run once on a fresh state) against the FP64 oracle
    (SimulatorBasic<double> restated, one-qubit gates folded into the
    two-qubit gates in FP64; 16 GiB on the host for 30 qubits)."""
    import numpy as np
    orc, _ = oracle_lib()
    n = c.num_qubits
    t0 = time.perf_counter()
    want = orc.run_ops_fp64_fused(n, c.ops())
    out = {"oracle": "FP64 state-vector oracle (SimulatorBasic<double> "
                     "restated), one-qubit gates folded into two-qubit "
                     "gates in FP64",
           "oracle_s": time.perf_counter() - t0,
           "bar": {"rel_l2": 1e-5, "fidelity": 1 - 1e-6}}
    st = ss.Create(n)
    buf = np.empty(ss.MinSize(n), dtype=np.float32)
    chunk = 1 << 24
    for name, plan in plans.items():
        ss.SetStateZero(st)
        plan.run(ctx, st)
        ss.Copy(st, buf)
        got = buf[: 2 << n].view(np.complex64)
        d2 = w2 = g2 = 0.0
        ip = 0j
        for i in range(0, want.size, chunk):
            g = got[i:i + chunk].astype(np.complex128)
            w = want[i:i + chunk]
            d2 += float(np.vdot(g - w, g - w).real)
            w2 += float(np.vdot(w, w).real)
            g2 += float(np.vdot(g, g).real)
            ip += complex(np.vdot(w, g))
        out[name] = {"rel_l2": float(np.sqrt(d2 / w2)),
                     "fidelity": float(abs(ip) ** 2 / (w2 * g2)),
                     "passes": len(plan)}
    del st, want, buf
    return out


def run_reference(args, world, rank, dist):
    """The reference arm: the reference's CPU path for the headline
    circuit on the host cores.  The reference checkout is not present on
    the GPU host, so its fused plan comes from the committed fixture and the
    gate passes from the oracle's port of its SIMD simulator (within 1.1-1.2x
    of the reference's own 128-bit SSE simulator on the same cores where
    both run).  Nothing of the engine is imported.  Each step is a bounded
    sample: the next ceil(G/K) fused gates of the plan, in order (the state
    carries over, as in a run), so that the K timed steps time every one of
    the G gates at least once; value = the sum over the G gates of each
    gate's mean time (seconds per run)."""
    if rank != 0:
        return
    import numpy as np
    n, gates = load_ref_plan()
    port = CpuPort(n)
    G = len(gates)
    per_step = -(-G // max(1, args.steps))
    pos = 0
    for _ in range(args.warmup):
        for _ in range(per_step):
            port.apply(gates[pos % G])
            pos += 1
    pos = 0
    op_times = [[] for _ in gates]
    step_s = []
    for _ in range(args.steps):
        t_step = 0.0
        for _ in range(per_step):
            t = port.apply(gates[pos % G])
            op_times[pos % G].append(t)
            t_step += t
            pos += 1
        step_s.append(t_step)
    timed = [t for t in op_times if t]
    v = float(sum(np.mean(t) for t in timed)) * G / len(timed)
    sample = (f"the reference's own f=4 plan of the 30-qubit circuit "
              f"({G} fused gates, MultiQubitGateFuser + CalculateFusedMatrix, "
              f"tests/golden/ref_plan_grid5x6d20_f4.npz) on an 8 GiB FP32 "
              f"host state; each step applies the next {per_step} gates; "
              f"{len(timed)} of {G} gates timed; value = sum of per-gate "
              f"mean times")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(step_s) * 1e3,
        "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "max_fused_size": 4,
                   "fused_ops": G, "gates_per_step": per_step,
                   "step": "a bounded sample of the run: the next "
                           f"{per_step} fused gates"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": port.threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
def run_engine(args, world, rank, local, dist):
    import numpy as np
    import qsim_gb300 as q
    from qsim_gb300 import engine as E
    from qsim_gb300 import _native as N
    from qsim_gb300 import learned as L

    hbm_peak, _, peak_kind = peaks()
    ctx = q.Context(local)       # one replica per GPU: LOCAL_RANK's device
    ss = q.StateSpace(ctx=ctx)
    c = E.Circuit.grid(GRID["rows"], GRID["cols"], GRID["extra"],
                       GRID["cycles"], GRID["seed"] + (rank if args.distinct_replicas else 0))
    n = c.num_qubits
    nbytes_state = 8 << n
    st = ss.Create(n)
    if ss.IsNull(st):
        raise RuntimeError("not enough device memory for the 30-qubit state")

    # Tensor-core forms: blocks of >= tc_min_k qubits on tcgen05.  Learned
    # planner: block boundaries, sizes and paths from the cost model trained
    # on this engine's GB300 launch times.
    model = L.CostMLP.load()
    head_options = {
        "plain_f4": dict(max_fused_size=4),
        "plain_f5": dict(max_fused_size=5),
        "plain_f6": dict(max_fused_size=6),
        "tc_f6": dict(max_fused_size=6, tensor_path=True, tc_min_k=5),
        "learned_tc_f6": dict(max_fused_size=6, tensor_path=True, tc_min_k=2,
                              cost_model=model),
        "tc_f6_pairs": dict(max_fused_size=6, tensor_path=True, tc_min_k=5,
                            tc_pairs=TC_PAIR_BITS),
        "learned_tc_f6_pairs": dict(max_fused_size=6, tensor_path=True,
                                    tc_min_k=2, cost_model=model,
                                    tc_pairs=TC_PAIR_BITS),
        "tc_f6_all": dict(max_fused_size=6, tensor_path=True, tc_min_k=1),
        "tc_f5_all": dict(max_fused_size=5, tensor_path=True, tc_min_k=1),
    }
    forms = {k: E.Plan(c, **o) for k, o in head_options.items()}

    def time_form(plan, steps, warmup):
        plan.capture(ctx, st)
        for _ in range(warmup):
            ss.SetStateZero(st)
            plan.replay(ctx)
        ctx.sync()
        barrier(dist)
        ctx.timer_start()
        for _ in range(steps):
            ss.SetStateZero(st)
            plan.replay(ctx)
        return ctx.timer_stop() / steps

    def kernels_per_run(plan):
        # Kernels of one run of the plan (its fused ops plus, for unitary
        # tensor-core plans, the norm-restoration kernels), counted by the
        # library; the run itself precedes the timed region.
        before = ctx.launches()
        plan.run(ctx, st)
        ctx.sync()
        return ctx.launches() - before

    results = {}
    # Kernels launched before the headline's timed region (for the ncu
    # launch-list window): SetStateZero is two kernels.
    launches_before = 0
    kernels = {}
    form_steps = max(1, args.steps // 2)
    for name, plan in forms.items():
        kernels[name] = kernels_per_run(plan)
        results[name] = time_form(plan, form_steps, 1)
        launches_before += kernels[name] + (1 + form_steps) * (kernels[name] + 2)
    # The headline form is the metric's "tensor-core + learned fusion" plan
    # with two-gate tensor-core passes; every form's time is in forms_s and
    # the fastest is named beside it.
    fastest = min(results, key=results.get)
    best = "learned_tc_f6_pairs"
    head = forms[best]
    launches_before += args.warmup * (kernels[best] + 2)

    # Headline timed region: K steps of the headline form.
    head.capture(ctx, st)
    for _ in range(args.warmup):
        ss.SetStateZero(st)
        head.replay(ctx)
    ctx.sync()
    launches_per_step = kernels[best] + 2  # plan + fill + set-one kernels
    barrier(dist)
    clk = ClockSampler(local)
    ctx.timer_start()
    for _ in range(args.steps):
        ss.SetStateZero(st)
        head.replay(ctx)
    ms = ctx.timer_stop() / args.steps
    clocks = clk.stop()
    # N replicas each run one circuit per step: whole-job seconds per run.
    value = replica_seconds_per_unit(dist, world, 1.0, ms / 1e3)
    ms = max_over_ranks(dist, ms)

    # Roofline of the dominant kernel of the headline plan: per-op CUDA-event
    # times; algorithmic bytes per launch = 16 * 2^n (one read + one write
    # of the state).
    # Three profiled runs (CUDA events around every launch); per launch the
    # median of the three.
    runs = []
    for _ in range(3):
        ss.SetStateZero(st)
        runs.append(np.asarray(head.profile(ctx, st), dtype=np.float64))
    prof = np.median(np.stack(runs), axis=0)
    hops = head.ops()
    pair_next = head.tc_pair_next()
    # Per kernel: launches, time, and fused-gate units per launch (a
    # two-gate pass applies two fused gates; the profile gives its time to
    # its first op and 0 to the second).  Algorithmic bytes of a unit:
    # 16 * 2^n (one read + one write of the state per fused gate); the
    # physical DRAM traffic of a two-gate pass is one read + one write.
    per_kernel = {}
    i = 0
    while i < len(hops):
        o = hops[i]
        if o["path"] == 1 and pair_next[i]:
            kname, units = "tc_gate2_kernel", 2
        elif o["path"] == 1:
            kname, units = "tc_gate_kernel", 1
        else:
            kname, units = "gate_tile_kernel", 1
        d = per_kernel.setdefault(kname, {"launches": 0, "total_ms": 0.0,
                                          "units_per_launch": units})
        d["launches"] += 1
        d["total_ms"] += float(prof[i])
        i += units
    dom = max(per_kernel, key=lambda kname: per_kernel[kname]["total_ms"])
    for kname, d in per_kernel.items():
        d["avg_ms"] = d["total_ms"] / d["launches"]
        d["gbs"] = (d["units_per_launch"] * 16.0 * (1 << n)
                    / (d["avg_ms"] * 1e-3) / 1e9)
        d["dram_gbs"] = 16.0 * (1 << n) / (d["avg_ms"] * 1e-3) / 1e9
        d["share"] = d["total_ms"] / float(np.sum(prof))
    achieved = per_kernel[dom]["gbs"]
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": traffic_from_profiles(n, dom),
                "kernel": dom, "peak_source": peak_kind,
                "bytes_per_launch": (per_kernel[dom]["units_per_launch"]
                                     * 16 * (1 << n)),
                "dram_frac": per_kernel[dom]["dram_gbs"] / hbm_peak,
                "per_kernel": per_kernel}
    # Plain f=4 plan breakdown by gate size (CUDA-core tile kernel).
    ss.SetStateZero(st)
    prof4 = forms["plain_f4"].profile(ctx, st)
    ops4 = forms["plain_f4"].ops()
    ks = [len(o["qs"]) for o in ops4]
    per_k = {}
    for k in sorted(set(ks)):
        ts = [t for t, kk in zip(prof4, ks) if kk == k]
        per_k[str(k)] = {"launches": len(ts), "avg_ms": float(np.mean(ts)),
                         "gbs": 16.0 * (1 << n) / (float(np.mean(ts)) * 1e-3) / 1e9}
    roofline["plain_f4_per_k"] = per_k

    # End to end through the public API with host buffers, as a user runs
    # QSimRunner::Run (lib/run_qsim.h:225-289: fusion, then every fused
    # gate, matrices uploaded per launch), then 1000 samples and the whole
    # final state copied to pinned host memory on the GPU's NUMA node.
    # Beside it, the same steps through the fused-plan cache
    # (qsg_plan_cache_run: the first call, a warm-up step, fuses, uploads
    # and captures; later calls hash the circuit and replay its graph, so
    # they copy no inputs to the device).
    hbuf = C.c_void_p()
    N.check(N.lib.qsg_host_alloc_near(local, nbytes_state, C.byref(hbuf)))
    numa = C.c_int(-1)
    N.check(N.lib.qsg_host_numa_node(local, C.byref(numa)))
    samples = np.zeros(1000, dtype=np.uint64)
    head_opts = head_options[best]
    h2d = sum(8 * (1 << (2 * len(o["qs"]))) for o in head.ops())
    pcache = E.PlanCache()

    def e2e_steps(fuse_each_call):
        times, phases = [], []
        for i in range(args.warmup + args.steps):
            ctx.sync()
            barrier(dist)
            t0 = time.perf_counter()
            ss.SetStateZero(st)
            if fuse_each_call:
                plan = E.Plan(c, **head_opts)
                tf = time.perf_counter()
                plan.run(ctx, st)
            else:
                tf = t0
                _, hit = pcache.run(ctx, c, st, **head_opts)
                assert hit or i == 0
            N.check(N.lib.qsg_sample(ctx.h, st.get(), n, 1000, 1,
                                     samples.ctypes.data_as(N.P_u64)))
            t1 = time.perf_counter()   # the samples synchronise the stream
            N.check(N.lib.qsg_copy_d2h(ctx.h, hbuf, st.get(), n))
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                times.append(dt)
                phases.append((tf - t0, t1 - tf, dt - (t1 - t0)))
        return statistics.median(times), phases

    e2e_s, phases = e2e_steps(True)
    cache_s, phases_cache = e2e_steps(False)
    N.lib.qsg_host_free(hbuf)
    e2e = replica_seconds_per_unit(dist, world, 1.0, e2e_s)
    e2e_phase = {"fuse_s": statistics.median(p[0] for p in phases),
                 "run_and_sample_s": statistics.median(p[1] for p in phases),
                 "state_d2h_s": statistics.median(p[2] for p in phases),
                 "host_numa_node": numa.value,
                 "plan_cache_hit": {
                     "value": replica_seconds_per_unit(dist, world, 1.0,
                                                       cache_s),
                     "run_and_sample_s": statistics.median(
                         p[1] for p in phases_cache),
                     "h2d_bytes_per_step": 0}}
    e2e_phase["d2h_gbs"] = nbytes_state / e2e_phase["state_d2h_s"] / 1e9

    # Learned planner on the 32-qubit 5x6+2 grid depth-24 circuit (32 GiB),
    # and batched trajectories (replicas for N > 1: every rank runs the
    # batch): the autotuned configuration, with the stream path alone at
    # f = 4 (one launch per fused block) beside it.
    del st
    if args.headline_only:
        learned = {"skipped": "--headline-only"}
        traj = {"skipped": "--headline-only"}
        expect = {"skipped": "--headline-only"}
        unitary = {"skipped": "--headline-only"}
        cache = {"skipped": "--headline-only"}
        hyb = {"skipped": "--headline-only"}
    else:
        learned = bench_learned_planner(ctx, ss, model, dist)
        learned["controlled_circuit"] = bench_learned_controlled(ctx, ss,
                                                                 model, dist)
        expect = bench_expectations(ctx, ss, dist)
        unitary = bench_unitary(ctx, dist, cpu=(rank == 0 and world == 1
                                                and not args.no_cpu))
        cache = bench_plan_cache(ctx, ss, dist)
        hyb = bench_hybrid(ctx, dist, cpu=(rank == 0 and world == 1
                                           and not args.no_cpu))
        traj = bench_trajectories(args.traj_streams, args.traj_f,
                                  mode=args.traj_mode,
                                  ctas_per_sm=args.traj_ctas_per_sm,
                                  tile_kib=args.traj_tile_kib,
                                  split=args.traj_split, device=local)
        traj["value"] = replica_rate(dist, world, traj["trajectories"],
                                     traj["wall_s"])
        traj["wall_s"] = max_over_ranks(dist, traj["wall_s"])
        alt = bench_trajectories(args.traj_streams, 4, mode="streams",
                                 device=local)
        traj["streams_only"] = {"value": alt["value"], "wall_s": alt["wall_s"],
                                "latency_ms_p50": alt["latency_ms_p50"],
                                "latency_ms_p99": alt["latency_ms_p99"],
                                "gpu_launches": alt["gpu_launches"]}
        # Every trajectory in the one persistent packed-batch kernel.
        pk = bench_trajectories(args.traj_streams, 4, mode="packed",
                                device=local)
        traj["packed_only"] = {"value": pk["value"], "wall_s": pk["wall_s"],
                               "latency_ms_p50": pk["latency_ms_p50"],
                               "latency_ms_p99": pk["latency_ms_p99"],
                               "gpu_launches": pk["gpu_launches"]}
        if rank == 0 and world == 1 and not args.no_cpu:
            traj["cpu_baseline"] = traj_cpu_baseline()
            traj["speedup_vs_cpu"] = (traj["value"]
                                      / traj["cpu_baseline"]["value"])

    cpu, precision = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        # The CPU-baseline leg: the reference's plan on the host cores, and
        # the FP64 oracle as the checker of the timed form's final state.
        cpu = cpu_full_run()
        precision = fp64_precision(ctx, ss, c, {best: head,
                                                "plain_f4": forms["plain_f4"]})
        if args.precision_all:
            # The learned plan of the layered circuit with controlled gates
            # (about 75 s of FP64 oracle on 16 host cores).
            cl = E.Circuit.layered_u3(EXPECT["n"], EXPECT["layers"],
                                      EXPECT["controlled"], EXPECT["seed"])
            precision["layered_28q"] = fp64_precision(ctx, ss, cl, {
                "learned_tc_f6": E.Plan(cl, **head_options["learned_tc_f6"]),
                "plain_f4": E.Plan(cl, max_fused_size=4)})

    if rank == 0:
        line = {
            "metric": METRIC, "value": value / 1.0, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": best,
                       "fastest_form": fastest,
                       "fused_ops": len(head), "max_k": head.info()["max_k"],
                       "state_bytes": nbytes_state,
                       "l2": "state 8 GiB > 129 MB L2, no flush needed",
                       "parallelism": f"replicas x{world}",
                       "forms_s": {k: v / 1e3 for k, v in results.items()},
                       "ncu_window": {"skip": launches_before,
                                      "count": launches_per_step * args.steps},
                       "passes": {k: len(v) for k, v in forms.items()}},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": nbytes_state + 8 * 1000,
                    "phases": e2e_phase},
            "gpu_launches": launches_per_step * args.steps,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "precision": precision,
            "clocks": clocks,
            "trajectories": traj,
            "learned_planner": learned,
            "expectations": expect,
            "unitary": unitary,
            "plan_cache": cache,
            "hybrid": hyb,
        }
        print(json.dumps(line), flush=True)


EXPECT = dict(n=28, layers=40, controlled=8, seed=3, strings=64, weight=6,
              pauli_seed=5)


def bench_expectations(ctx, ss, dist):
    """28-qubit layered circuit (U3 on every qubit, CZ/CNOT on random
    disjoint pairs, 8 gates with 1-2 controls per layer, 40 layers) and 64
    Pauli strings of weight 1..6: seconds per circuit run (the learned
    tensor-core plan with two-gate passes, and the plain f = 4 plan, from
    CUDA graphs) and per expectation value, on the one-pass monomial kernel
    and, for comparison, on the dense path (the same operator with one
    off-pattern entry of 1e-30, which the monomial test rejects: tile kernel
    for k <= 3, tensor cores for k >= 4)."""
    import numpy as np
    from qsim_gb300 import engine as E
    import qsim_gb300 as q
    sim = q.Simulator(ctx=ctx)
    paulis = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]),
              "Y": np.array([[0, -1j], [1j, 0]]), "Z": np.diag([1, -1])}

    def pauli_matrix(letters):
        # letters[j] acts on the string's j-th (sorted) qubit = index bit j.
        m = np.eye(1, dtype=np.complex128)
        for p in letters:
            m = np.kron(paulis[p], m)
        return m

    from qsim_gb300 import learned as L
    c = E.Circuit.layered_u3(EXPECT["n"], EXPECT["layers"], EXPECT["controlled"],
                             EXPECT["seed"])
    n = c.num_qubits
    st = ss.Create(n)
    # The circuit by the engine's fastest form (learned fusion on the tensor
    # cores with two-gate passes) and by the plain f = 4 plan; the Pauli sums
    # are taken on the former's state.
    circuit = {}
    for name, plan in (("plain_f4", E.Plan(c, max_fused_size=4)),
                       ("learned_tc_f6_pairs",
                        E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=2,
                               cost_model=L.CostMLP.load(),
                               tc_pairs=TC_PAIR_BITS))):
        plan.capture(ctx, st)
        ss.SetStateZero(st)
        plan.replay(ctx)
        ctx.sync()
        barrier(dist)
        ctx.timer_start()
        ss.SetStateZero(st)
        plan.replay(ctx)
        circuit[name] = max_over_ranks(dist, ctx.timer_stop() / 1e3)
        ctx.sync()
    strings = E.pauli_sum(n, EXPECT["strings"], EXPECT["weight"],
                          EXPECT["pauli_seed"])
    mats = []
    for qs, letters, coeff in strings:
        m = np.ascontiguousarray(pauli_matrix(letters).astype(np.complex64))
        md = m.copy()
        md[0, int(np.flatnonzero(m[0] == 0)[0])] += np.complex64(1e-30)
        mats.append((qs, coeff, m.view(np.float32), md.view(np.float32)))
    out = {}
    for name, idx in (("monomial", 2), ("dense", 3)):
        for qs, _, *mm in mats[:2]:
            sim.ExpectationValue(qs, mm[idx - 2], st)   # warm-up
        ctx.sync()
        t0 = time.perf_counter()
        total = 0.0
        for qs, coeff, *mm in mats:
            total += coeff * sim.ExpectationValue(qs, mm[idx - 2], st).real
        dt = time.perf_counter() - t0
        out[name] = {"s_per_ev": dt / len(mats), "pauli_sum": total,
                     "gbs": 8.0 * (1 << n) / (dt / len(mats)) / 1e9}
    return {
        "workload": f"layered U3 ({n} qubits) 40 layers, 8 controlled gates "
                    f"per layer, seed 3; {len(mats)} Pauli strings of weight "
                    "1..6",
        "circuit_s_per_run": circuit["learned_tc_f6_pairs"],
        "circuit_form": "learned_tc_f6_pairs",
        "circuit_plain_f4_s": circuit["plain_f4"],
        "passes": len(plan) - int(plan.tc_pair_next().sum()),
        "ev": out,
        "ev_speedup": out["dense"]["s_per_ev"] / out["monomial"]["s_per_ev"],
    }


def bench_plan_cache(ctx, ss, dist):
    """The headline circuit run through the fused-plan cache: the first run
    (fusion at f = 6 on the tensor-core path, CUDA-graph capture, replay)
    against later runs (key + hash + graph launch), wall seconds per run
    with the state zeroed and the device synchronised, and the host time of
    a cached call alone.  The reference fuses on every QSimRunner::Run."""
    from qsim_gb300 import engine as E
    c = E.Circuit.grid(GRID["rows"], GRID["cols"], GRID["extra"],
                       GRID["cycles"], GRID["seed"])
    n = c.num_qubits
    st = ss.Create(n)
    opts = dict(max_fused_size=6, tensor_path=True, tc_pairs=TC_PAIR_BITS)
    t0 = time.perf_counter()
    E.Plan(c, **opts)
    fuse_s = time.perf_counter() - t0
    pc = E.PlanCache()
    barrier(dist)
    ss.SetStateZero(st)
    ctx.sync()
    t0 = time.perf_counter()
    _, hit0 = pc.run(ctx, c, st, **opts)
    ctx.sync()
    first_s = time.perf_counter() - t0
    hits, host = [], []
    for _ in range(3):
        ss.SetStateZero(st)
        ctx.sync()
        t0 = time.perf_counter()
        _, hit = pc.run(ctx, c, st, **opts)
        t1 = time.perf_counter()
        ctx.sync()
        hits.append(time.perf_counter() - t0)
        host.append(t1 - t0)
        assert hit and not hit0
    del st
    return {"workload": "the headline circuit through qsg_plan_cache_run "
                        "(tensor-core f = 6, two-gate passes)",
            "fuse_s": fuse_s, "first_run_s": first_s,
            "hit_run_s": max_over_ranks(dist, statistics.median(hits)),
            "hit_host_call_ms": statistics.median(host) * 1e3,
            "stats": pc.stats()}


HYBRID = dict(rows=4, cols=8, extra=0, cycles=14, seed=1, prefix_gates=4,
              bitstrings=1000, batch_bits=16)


def bench_hybrid(ctx, dist, cpu: bool):
    """One qsimh job on the 32-qubit 4x8 grid depth-14 circuit cut into
    column halves (16 + 16 qubits, 12 fSim gates on the cut): the first 4
    cut gates fixed by the job's prefix, the other 8 (16 path bits = 65536
    paths) summed for 1000 bitstring amplitudes.  Wall seconds of the whole
    qsg_hybrid_run call (split, fusion, device runs, amplitude read-back),
    CUDA-core f = 4 and tensor-core f = 6.  CPU baseline: the oracle's
    OpenMP FP32 gate application over each part's post-checkpoint gates
    (fused to <= 2 qubits, as the reference's qsimh runner fuses), which the
    reference runs once per path (lib/hybrid.h:381-433), timed on sample
    paths and multiplied by the path count."""
    import numpy as np
    from qsim_gb300 import engine as E, hybrid
    h = HYBRID
    c = E.Circuit.grid(h["rows"], h["cols"], h["extra"], h["cycles"], h["seed"])
    n = c.num_qubits
    parts = [0 if (q % h["cols"]) < h["cols"] // 2 else 1 for q in range(n)]
    rng = np.random.default_rng(11)
    bits = rng.integers(0, 1 << n, h["bitstrings"], dtype=np.uint64)
    out = {}
    for name, kw in (("plain_f4", dict(max_fused_size=4)),
                     ("tc_f6", dict(max_fused_size=6, tensor_path=True))):
        args = dict(num_prefix_gatexs=h["prefix_gates"],
                    max_batch_bits=h["batch_bits"], **kw)
        hybrid.run(ctx, c, parts, bits[:8], **args)       # warm-up
        times = []
        for _ in range(2):
            barrier(dist)
            t0 = time.perf_counter()
            amps, info = hybrid.run(ctx, c, parts, bits, **args)
            times.append(time.perf_counter() - t0)
        t = max_over_ranks(dist, min(times))
        out[name] = {"s_per_job": t, "paths_per_s": info["paths_run"] / t,
                     "amplitudes_norm2": float(np.sum(np.abs(amps) ** 2))}
    best = min(out, key=lambda k: out[k]["s_per_job"])
    res = {"workload": f"qsimh job: {n}-qubit 4x8 grid depth 14 (seed 1), "
                       f"parts = column halves, {info['num_gatexs']} gates on "
                       f"the cut, {h['prefix_gates']} fixed by the prefix, "
                       f"{info['paths_run']} paths, {len(bits)} amplitudes",
           "info": info, "forms": out, "best": best}
    if cpu:
        res["cpu_baseline"] = hybrid_cpu_sample(c, parts, h["prefix_gates"],
                                                info["paths_run"])
        res["speedup_vs_cpu"] = (res["cpu_baseline"]["value"]
                                 / out[best]["s_per_job"])
    return res


def hybrid_cpu_sample(c, parts, num_prefix, paths, max_paths=16):
    """The reference's per-path work (both parts' gates after the root
    checkpoint, one path at a time) on the host cores with the oracle's
    OpenMP FP32 gate application; seconds per job = mean per path x paths."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from conftest import Oracle
    import hybrid_oracle as HO
    from qsim_gb300 import engine as E
    orc = Oracle()
    ops = c.ops()
    for i, o in enumerate(ops):
        o["schmidt"] = c.schmidt(i) if len(o["qs"]) == 2 else []
    n0, n1, _, part_ops, cuts = HO.split_lattice(c.num_qubits, ops, parts)
    P = C.POINTER
    rng = np.random.default_rng(2)
    t_total, done = 0.0, 0
    for _ in range(max_paths):
        for p, np_ in ((0, n0), (1, n1)):
            st = np.zeros(2 << np_, dtype=np.float32)
            st[0] = 1.0
            first = next(i for i, o in enumerate(part_ops[p])
                         if o["cut"] >= num_prefix)
            # One path's gates, fused into <= 2-qubit blocks as the
            # reference's qsimh runner does (BasicGateFuser).
            pc = E.Circuit(np_)
            for o in part_ops[p][first:]:
                if o["cut"] < 0:
                    pc.add_gate(o["time"], o["qs"], o["m"])
                else:
                    g = cuts[o["cut"]]
                    pc.add_gate(o["time"], [g["q"][p]],
                                g["f"][p][int(rng.integers(g["terms"]))])
            mats = [(o["qs"], np.ascontiguousarray(
                np.asarray(o["m"], np.complex64)).view(np.float32))
                for o in E.Plan(pc, max_fused_size=2).ops()]
            t0 = time.perf_counter()
            for qs, m in mats:
                qa = (C.c_uint * len(qs))(*qs)
                orc.L.orc_port_apply_gate_f32(st.ctypes.data_as(P(C.c_float)),
                                              np_, qa, len(qs),
                                              m.ctypes.data_as(P(C.c_float)))
            t_total += time.perf_counter() - t0
        done += 1
        if t_total > 15.0:
            break
    per_path = t_total / done
    return {"value": per_path * paths, "unit": "s/job",
            "cores": orc.L.orc_num_threads(), "kind": "port",
            "sample": f"{done} sample paths (both parts' post-checkpoint "
                      f"gates fused into <= 2-qubit blocks, the oracle's "
                      f"lane-batched FP32 port), x {paths} paths"}


def hybrid_case(tensor: bool):
    """One small qsimh job for ncu captures: the 24-qubit 4x6 grid depth-14
    circuit cut into column halves (12 + 12 qubits, 12 fSim gates on the
    cut), 5 gates fixed by the prefix, the other 7 (14 path bits = 16384
    paths, batch states of 2^26 amplitudes, 512 MiB per part) summed for 1000
    amplitudes; a warm-up job, then the job the capture looks at."""
    import numpy as np
    from qsim_gb300 import api, engine as E, hybrid
    c = E.Circuit.grid(4, 6, 0, 14, 1)
    n = c.num_qubits
    parts = [0 if (q % 6) < 3 else 1 for q in range(n)]
    bits = np.random.default_rng(11).integers(0, 1 << n, 1000, dtype=np.uint64)
    ctx = api.Context(0)
    kw = dict(num_prefix_gatexs=5, max_fused_size=6 if tensor else 4,
              tensor_path=tensor)
    hybrid.run(ctx, c, parts, bits, **kw)
    ctx.sync()
    before = ctx.launches()
    t0 = time.perf_counter()
    _, info = hybrid.run(ctx, c, parts, bits, **kw)
    ctx.sync()
    print(json.dumps({"hybrid_case": info, "s_per_job": time.perf_counter() - t0,
                      "launches_before": before,
                      "launches": ctx.launches() - before}), flush=True)


UNITARY_GRID = dict(rows=2, cols=7, extra=0, cycles=14, seed=1)


def bench_unitary(ctx, dist, cpu: bool):
    """Unitary of the 14-qubit 2x7 grid depth-14 circuit (2^28 complex64
    entries, 2 GiB > L2): seconds per unitary (SetIdentity + the fused plan
    applied by the unitary calculator) for the CUDA-core f = 4 plan and the
    tensor-core f = 6 plan, GB/s per pass (16 bytes per entry), and on rank
    0 the oracle's OpenMP FP32 port of the same gate passes on the host
    (the first fused ops of the f = 4 plan, extrapolated by op count)."""
    from qsim_gb300 import engine as E
    from qsim_gb300 import unitary as U
    g = UNITARY_GRID
    c = E.Circuit.grid(g["rows"], g["cols"], g["extra"], g["cycles"], g["seed"])
    n = c.num_qubits
    us, calc = U.UnitarySpace(ctx=ctx), U.UnitaryCalculator(ctx=ctx)
    u = us.CreateUnitary(n)
    entries = 1 << (2 * n)
    forms = {"plain_f4": E.Plan(c, max_fused_size=4),
             "tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True),
             "tc_f6_pairs": E.Plan(c, max_fused_size=6, tensor_path=True,
                                   tc_pairs=TC_PAIR_BITS)}
    out = {}
    for name, plan in forms.items():
        us.SetIdentity(u)
        calc.RunPlan(plan, u)       # warm-up (operand upload, attributes)
        ctx.sync()
        times = []
        for _ in range(3):
            barrier(dist)
            ctx.timer_start()
            us.SetIdentity(u)
            calc.RunPlan(plan, u)
            times.append(ctx.timer_stop() / 1e3)
        t = max_over_ranks(dist, statistics.median(times))
        passes = len(plan) - int(plan.tc_pair_next().sum())
        out[name] = {"s_per_unitary": t, "passes": passes,
                     "gbs_per_pass": 16.0 * entries * passes / t / 1e9}
    res = {"workload": f"unitary of the {n}-qubit 2x7 grid depth-14 circuit "
                       f"(seed 1), {entries} complex64 entries",
           "forms": out,
           "best": min(out, key=lambda k: out[k]["s_per_unitary"])}
    us_best = out[res["best"]]["s_per_unitary"]
    del u
    if cpu:
        import numpy as np
        ops = forms["plain_f4"].ops()
        port = CpuPort(2 * n)
        v = 0.0
        for o in ops:
            m = np.ascontiguousarray(np.asarray(o["m"], np.complex64)).view(np.float32)
            v += port.apply((len(o["qs"]), o["qs"], m))
        res["cpu_baseline"] = {
            "value": v, "unit": "s/unitary", "cores": port.threads,
            "kind": "port",
            "sample": f"every one of the {len(ops)} fused gates (f=4 plan) "
                      f"applied once to the 2 GiB FP32 host unitary by the "
                      f"oracle's lane-batched port of the reference's SIMD "
                      f"gate kernels (the diagonal start not timed)"}
        res["speedup_vs_cpu"] = v / us_best
    return res


LEARN_GRID = dict(rows=5, cols=6, extra=2, cycles=24, seed=1)


def pair_cost_factor(n, a, b):
    """Cost of a two-gate tensor-core pass relative to two one-gate passes,
    as the planner weighs it: the pair's 12-qubit tile is the union of both
    target sets completed with the lowest other qubits, its run bits rb the
    length of the prefix 0, 1, ... it holds; 0.80 at rb >= 4; shorter runs
    by the tile's other qubits below 12 (near) and in 12..20 (mid)."""
    u = set(a) | set(b)
    q = 0
    while len(u) < 12 and q < n:
        u.add(q)
        q += 1
    rb = 0
    while rb in u:
        rb += 1
    if rb >= 4:
        return 0.80
    near = sum(1 for x in u if rb <= x < 12)
    mid = sum(1 for x in u if 12 <= x < 21)
    if rb == 3:
        return 0.87 if near >= 1 else 1.28
    if rb == 2:
        if near >= 2 or (near == 1 and mid >= 2):
            return 0.95
        return 1.28 if near == 1 else 2.49
    return 1.11 if rb == 1 else 2.49


def bench_learned_planner(ctx, ss, model, dist):
    """Seconds per run of the 32-qubit 5x6+2 grid depth-24 circuit for the
    learned plan and the fixed-size plans (CUDA-core f = 4, 5, 6 and
    tensor-core f = 6), each replayed from a CUDA graph, and the fidelity of
    the learned plan's state against the plain f = 4 plan's."""
    import numpy as np
    from qsim_gb300 import engine as E
    from qsim_gb300 import _native as N
    c = E.Circuit.grid(*LEARN_GRID.values())
    n = c.num_qubits
    forms = {
        "plain_f4": E.Plan(c, max_fused_size=4),
        "plain_f5": E.Plan(c, max_fused_size=5),
        "plain_f6": E.Plan(c, max_fused_size=6),
        "tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5),
        "learned_tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True,
                                tc_min_k=2, cost_model=model),
        "tc_f6_pairs": E.Plan(c, max_fused_size=6, tensor_path=True,
                              tc_min_k=5, tc_pairs=TC_PAIR_BITS),
        "learned_tc_f6_pairs": E.Plan(c, max_fused_size=6, tensor_path=True,
                                      tc_min_k=2, cost_model=model,
                                      tc_pairs=TC_PAIR_BITS),
    }
    st = ss.Create(n)
    ref = ss.Create(n)
    if ss.IsNull(st) or ss.IsNull(ref):
        return {"skipped": "not enough device memory for two 32-qubit states"}
    times, spread, predicted = {}, {}, {}
    for name, p in forms.items():
        p.capture(ctx, st)
        ss.SetStateZero(st)
        p.replay(ctx)
        ctx.sync()
        # Tensor-core and learned forms (~0.5 s) 7 runs, CUDA-core forms
        # (1.5-2.3 s) 3 runs; the median is kept, the spread reported.
        runs = []
        for _ in range(3 if name.startswith("plain") else 7):
            barrier(dist)
            ctx.timer_start()
            ss.SetStateZero(st)
            p.replay(ctx)
            runs.append(ctx.timer_stop() / 1e3)
        times[name] = max_over_ranks(dist, statistics.median(runs))
        spread[name] = [min(runs), max(runs)]
        # Predicted time as the planner scores it: a two-gate pass costs its
        # two blocks times the measured pair factor of its tile's run bits.
        pn = p.tc_pair_next()
        ops = p.ops()
        costs = [model.cost_us(n, o["qs"], len(o["cqs"]), o["path"])
                 if o["kind"] != 2 else 0.0 for o in ops]
        pred, i = 0.0, 0
        while i < len(costs):
            if pn[i]:
                pred += (pair_cost_factor(n, ops[i]["qs"], ops[i + 1]["qs"])
                         * (costs[i] + costs[i + 1]))
                i += 2
            else:
                pred += costs[i]
                i += 1
        predicted[name] = pred / 1e6
        if name == "plain_f4":
            ss.Copy(st, ref)
    ip = C.c_double * 2
    r = ip()
    N.check(N.lib.qsg_inner_product(ctx.h, ref.get(), st.get(), n, r))
    fid = (r[0] ** 2 + r[1] ** 2) / (ss.Norm(ref) * ss.Norm(st))
    fixed = {k: v for k, v in times.items() if not k.startswith("learned")}
    fixed_np = {k: v for k, v in fixed.items() if not k.endswith("_pairs")}
    best_fixed = min(fixed_np, key=fixed_np.get)
    best_fixed_any = min(fixed, key=fixed.get)
    return {
        "workload": "grid5x6+2 (32 qubits) random circuit depth 24, seed 1, "
                    "complex64 (32 GiB)",
        "unit": "s/run", "forms_s": times, "forms_min_max_s": spread,
        "predicted_s": predicted,
        "passes": {k: len(v) - int(v.tc_pair_next().sum())
                   for k, v in forms.items()},
        "learned_vs_best_fixed": times[best_fixed] / times["learned_tc_f6"],
        "best_fixed": best_fixed,
        "learned_pairs_vs_best_fixed": (times[best_fixed_any]
                                        / times["learned_tc_f6_pairs"]),
        "best_fixed_with_pairs": best_fixed_any,
        "learned_vs_plain_f4": times["plain_f4"] / times["learned_tc_f6"],
        "fidelity_learned_vs_plain_f4": fid,
    }


def bench_learned_controlled(ctx, ss, model, dist):
    """The learned planner where its choices matter: the 28-qubit layered
    circuit (U3 on every qubit, CZ/CNOT on random disjoint pairs, 8 U3 gates
    with 1-2 controls per layer, 40 layers, seed 3).  Fixed fusers (plain
    f = 4, 5, 6 and tensor-core f = 6) pass the 320 controlled gates through
    unfused, as the reference's MultiQubitGateFuser does; the learned
    planner may absorb them into blocks, and its predicted times choose.
    Each tensor-core form also with two-gate passes.  Seconds per run
    (median of 5 graph replays each, min/max beside), host fusion time per
    plan, and the fidelity of the learned plan with two-gate passes against
    the plain f = 4 plan's state."""
    from qsim_gb300 import engine as E
    from qsim_gb300 import _native as N
    c = E.Circuit.layered_u3(EXPECT["n"], EXPECT["layers"],
                             EXPECT["controlled"], EXPECT["seed"])
    n = c.num_qubits
    opts = {
        "plain_f4": dict(max_fused_size=4),
        "plain_f5": dict(max_fused_size=5),
        "plain_f6": dict(max_fused_size=6),
        "tc_f6": dict(max_fused_size=6, tensor_path=True, tc_min_k=5),
        "learned_tc_f6": dict(max_fused_size=6, tensor_path=True, tc_min_k=2,
                              cost_model=model),
        "tc_f6_pairs": dict(max_fused_size=6, tensor_path=True, tc_min_k=5,
                            tc_pairs=TC_PAIR_BITS),
        "learned_tc_f6_pairs": dict(max_fused_size=6, tensor_path=True,
                                    tc_min_k=2, cost_model=model,
                                    tc_pairs=TC_PAIR_BITS),
    }
    forms, fuse_s = {}, {}
    for name, o in opts.items():
        t0 = time.perf_counter()
        forms[name] = E.Plan(c, **o)
        fuse_s[name] = time.perf_counter() - t0
    st, ref = ss.Create(n), ss.Create(n)
    times, spread = {}, {}
    for name, p in forms.items():
        p.capture(ctx, st)
        ss.SetStateZero(st)
        p.replay(ctx)
        ctx.sync()
        runs = []
        for _ in range(5):
            barrier(dist)
            ctx.timer_start()
            ss.SetStateZero(st)
            p.replay(ctx)
            runs.append(ctx.timer_stop() / 1e3)
        times[name] = max_over_ranks(dist, statistics.median(runs))
        spread[name] = [min(runs), max(runs)]
        if name == "plain_f4":
            ss.Copy(st, ref)
    r = (C.c_double * 2)()
    N.check(N.lib.qsg_inner_product(ctx.h, ref.get(), st.get(), n, r))
    fid = (r[0] ** 2 + r[1] ** 2) / (ss.Norm(ref) * ss.Norm(st))
    del st, ref
    fixed = {k: v for k, v in times.items() if not k.startswith("learned")}
    fixed_np = {k: v for k, v in fixed.items() if not k.endswith("_pairs")}
    best_fixed = min(fixed_np, key=fixed_np.get)
    best_fixed_any = min(fixed, key=fixed.get)
    return {
        "workload": f"layered U3 ({n} qubits) 40 layers, CZ/CNOT pairs, 8 "
                    "controlled U3 gates (1-2 controls) per layer, seed 3",
        "unit": "s/run", "forms_s": times, "forms_min_max_s": spread,
        "fuse_s": fuse_s,
        "passes": {k: len(v) - int(v.tc_pair_next().sum())
                   for k, v in forms.items()},
        "controlled_passes": {k: sum(1 for o in v.ops() if o["kind"] == 1)
                              for k, v in forms.items()},
        "learned_vs_best_fixed": times[best_fixed] / times["learned_tc_f6"],
        "best_fixed": best_fixed,
        "learned_pairs_vs_best_fixed": (times[best_fixed_any]
                                        / times["learned_tc_f6_pairs"]),
        "best_fixed_with_pairs": best_fixed_any,
        "learned_vs_plain_f4": times["plain_f4"] / times["learned_tc_f6_pairs"],
        "fidelity_learned_vs_plain_f4": fid,
    }


TRAJ = dict(circuits=128, reps=32, n_min=12, n_max=24, cycles=12,
            p_depol=1e-3, gamma=5e-3, seed=4)
TRAJ_WORKLOAD = ("4096 noisy trajectories: 128 chain random circuits, n ~ "
                 "U{12..24}, depth 12, depolarizing 1e-3 after each gate "
                 "qubit, amplitude damping 5e-3 per qubit per cycle, 32 "
                 "repetitions each")


def bench_trajectories(num_streams: int, max_fused_size: int = 0,
                       mode: str = "auto", ctas_per_sm: int = 0,
                       tile_kib: int = 0, split: int = -1, device: int = 0):
    """Batched-trajectory workload: every trajectory from |0..0>, its final
    state left normalised in HBM and its Kraus statistics copied to the
    host.  traj/s = trajectories / batch wall time (program compilation,
    upload, device work and the final synchronisation); latency =
    per-trajectory device time.

    mode "auto": the autotuner picks the stream path's form (fusion size,
    tensor cores), the split between the persistent packed kernel and the
    concurrent stream path, CTAs per SM and tile budget on an eighth of the
    repetitions (outside the timed run);
    "packed": every circuit in the persistent kernel; "streams": the stream
    path only."""
    import numpy as np
    from qsim_gb300 import engine as E
    from qsim_gb300 import autotune as AT
    rng = np.random.default_rng(TRAJ["seed"])
    ns = rng.integers(TRAJ["n_min"], TRAJ["n_max"] + 1, size=TRAJ["circuits"])
    made = {}

    def make_runners(f, tensor):
        if (f, tensor) not in made:
            rs = []
            for i, n in enumerate(ns):
                c = E.Circuit.chain(int(n), TRAJ["cycles"], 1000 + i)
                nc = E.NoisyCircuit.make(c, TRAJ["p_depol"], TRAJ["gamma"], 2)
                rs.append(E.Trajectories(nc, max_fused_size=f,
                                         tensor_path=tensor))
            made[(f, tensor)] = rs
        return made[(f, tensor)]

    t0 = time.perf_counter()
    tune = None
    tensor = max_fused_size >= 5
    if mode == "auto":
        forms = AT.FORMS if not max_fused_size else ((max_fused_size, tensor),)
        tune = AT.tune_trajectories(
            make_runners, ns, TRAJ["reps"], tag="chain d12 depol1e-3 ad5e-3",
            forms=forms, num_streams=num_streams, device=device,
            use_cache=False)
        cfg = dict(tune["best"])
    elif mode == "packed":
        cfg = dict(max_fused_size=4, tensor=False, split=int(ns.max()),
                   ctas_per_sm=ctas_per_sm, tile_kib=tile_kib)
    else:
        cfg = dict(max_fused_size=max_fused_size or 4, tensor=tensor, split=0,
                   ctas_per_sm=0, tile_kib=0)
    if split >= 0:
        cfg["split"] = split
    runners = AT.runners_for(make_runners, ns, cfg)
    setup_s = time.perf_counter() - t0
    items = [(i, r) for i in range(len(runners)) for r in range(TRAJ["reps"])]
    AT.run(runners, [(i, 10**6) for i in range(len(runners))], cfg, num_streams,
           device=device)
    per, lat, wall, launches, info = AT.run(runners, items, cfg, num_streams,
                                            device=device)
    amp_ops = sum(float(2 ** int(ns[i])) * runners[i].info()["num_fused_ops"]
                  for i, _ in items)
    escapes = 0
    for (i, _), st in zip(items, per):
        s = E.Trajectories.samples(st)
        escapes += int(np.sum(s == 1))
    per_n = {}
    for (i, _), t in zip(items, lat):
        per_n.setdefault(int(ns[i]), []).append(float(t))
    out = {
        "value": len(items) / wall, "unit": "traj/s",
        "wall_s": wall, "trajectories": len(items),
        "latency_ms_p50": float(np.percentile(lat, 50)),
        "latency_ms_p99": float(np.percentile(lat, 99)),
        "config": cfg, "streams": num_streams,
        "setup_s": setup_s, "gpu_launches": launches,
        "fused_pass_bytes_per_s": 16.0 * amp_ops / wall,
        "non_default_kraus_choices": escapes,
        "latency_ms_mean_by_n": {str(k): float(np.mean(v))
                                 for k, v in sorted(per_n.items())},
        "workload": TRAJ_WORKLOAD,
        "mode": mode,
        "packed": info,
    }
    if tune is not None:
        out["autotune"] = {"tune_s": tune["tune_s"],
                           "table": [dict(c, traj_s=round(v, 1))
                                     for c, v in tune["table"]]}
    return out


def traj_cpu_baseline(sample_reps: int = 3):
    """Trajectories per second of the reference's CPU trajectory loop on the
    host cores for the batched workload: the oracle's FP32 port of
    RunIteration (oracle/traj_port.py: deferred operators fused as the
    reference's default max_fused_size 2, one-qubit operators folded into
    two-qubit gates; the lane-batched port of the reference's SIMD gate
    kernels), timed on a bounded sample of the batch."""
    import numpy as np
    from qsim_gb300 import engine as E
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import traj_port
    _, lib = oracle_lib()
    rng = np.random.default_rng(TRAJ["seed"])
    ns = rng.integers(TRAJ["n_min"], TRAJ["n_max"] + 1, size=TRAJ["circuits"])
    circuits = [(int(n), E.Circuit.chain(int(n), TRAJ["cycles"], 1000 + i).ops())
                for i, n in enumerate(ns)]
    total, desc, mean_s = traj_port.time_batch(
        lib, circuits, TRAJ["reps"], sample_reps, TRAJ["p_depol"],
        TRAJ["gamma"], 2)
    return {"value": TRAJ["circuits"] * TRAJ["reps"] / total,
            "unit": "traj/s", "cores": lib.orc_num_threads(), "kind": "port",
            "sample": desc, "batch_s_estimate": total,
            "mean_s_by_n": {str(k): v for k, v in mean_s.items()}}


def kernel_case(spec: str, n: int, reps: int):
    """Small profiling case on a uniform n-qubit state, `reps` launches of
    one kind:

      gate:q0,q1,..           CUDA-core tile kernel (random unitary)
      tc:q0,..                tensor-core kernel (random unitary)
      tc2:q0,..:q0,..         two-gate tensor-core pass (random unitaries)
      ctrl:q0,..:c0,..        controlled gate, controls all 1
      ev:q0,..                ExpectationValue (tile kernel, mode 1)
      evp:q0,..:PAULIS        ExpectationValue of a Pauli string (letters
                              X, Y, Z, I per qubit; one-pass kernel)
      norm | ip | multiply    reductions / elementwise pass
      sample                  1000 samples (chunk sums, prefix, search)
      collapse:mask           Collapse on bits = 0 of `mask` (hex)
    """
    import ctypes as Cx
    import numpy as np
    import qsim_gb300 as q
    from qsim_gb300 import _native as N
    parts = spec.split(":")
    kind = parts[0]
    qs = [int(x) for x in parts[1].split(",")] if len(parts) > 1 and kind in (
        "gate", "tc", "tc2", "ctrl", "ev", "evp") else []
    qs2 = [int(x) for x in parts[2].split(",")] if kind == "tc2" else []
    cqs = [int(x) for x in parts[2].split(",")] if kind == "ctrl" else []
    ctx = q.Context(0)
    ss, sim = q.StateSpace(ctx=ctx), q.Simulator(ctx=ctx)
    st = ss.Create(n)
    ss.SetStateUniform(st)
    other = None
    if kind == "ip":
        other = ss.Create(n)
        ss.SetStateUniform(other)
    k = len(qs)
    rng = np.random.default_rng(0)
    u, _ = np.linalg.qr(rng.normal(size=(1 << k, 1 << k)) +
                        1j * rng.normal(size=(1 << k, 1 << k)))
    if kind == "evp":
        pm = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]),
              "Y": np.array([[0, -1j], [1j, 0]]), "Z": np.diag([1, -1])}
        u = np.eye(1)
        for letter in parts[2]:
            u = np.kron(pm[letter], u)
    m = np.ascontiguousarray(u.astype(np.complex64)).view(np.float32)
    u2, _ = np.linalg.qr(rng.normal(size=(1 << len(qs2), 1 << len(qs2))) +
                         1j * rng.normal(size=(1 << len(qs2), 1 << len(qs2))))
    m2 = np.ascontiguousarray(u2.astype(np.complex64)).view(np.float32)
    out2 = (Cx.c_double * 2)()
    smp = np.zeros(1000, dtype=np.uint64)
    for _ in range(reps):
        if kind == "tc":
            N.check(N.lib.qsg_apply_gate_tc(ctx.h, st.get(), n, N.u32_array(qs),
                                            k, m.ctypes.data_as(N.P_f32)))
        elif kind == "tc2":
            N.check(N.lib.qsg_apply_gate_tc2(
                ctx.h, st.get(), n, N.u32_array(qs), k,
                m.ctypes.data_as(N.P_f32), N.u32_array(qs2), len(qs2),
                m2.ctypes.data_as(N.P_f32)))
        elif kind == "gate":
            sim.ApplyGate(qs, m, st)
        elif kind == "ctrl":
            N.check(N.lib.qsg_apply_controlled_gate(
                ctx.h, st.get(), n, N.u32_array(qs), k, N.u32_array(cqs),
                len(cqs), (1 << len(cqs)) - 1, m.ctypes.data_as(N.P_f32)))
        elif kind in ("ev", "evp"):
            N.check(N.lib.qsg_expectation_value(
                ctx.h, st.get(), n, N.u32_array(qs), k,
                m.ctypes.data_as(N.P_f32), out2))
        elif kind == "norm":
            N.check(N.lib.qsg_norm(ctx.h, st.get(), n, out2))
        elif kind == "ip":
            N.check(N.lib.qsg_inner_product(ctx.h, st.get(), other.get(), n, out2))
        elif kind == "multiply":
            N.check(N.lib.qsg_multiply(ctx.h, 1.0, st.get(), n))
        elif kind == "sample":
            N.check(N.lib.qsg_sample(ctx.h, st.get(), n, 1000, 1,
                                     smp.ctypes.data_as(N.P_u64)))
        elif kind == "collapse":
            ss.SetStateUniform(st)
            N.check(N.lib.qsg_collapse(ctx.h, st.get(), n, int(parts[1], 16), 0))
        else:
            raise SystemExit(f"unknown kernel case {spec!r}")
    ctx.sync()
    print(json.dumps({"kernel_case": spec, "n": n, "reps": reps,
                      "norm": ss.Norm(st)}))


def pair_shapes(n: int, reps: int):
    """Two-gate tensor-core pass against two one-gate passes by tile shape,
    on a uniform n-qubit state: for run bits rb = 2, 3, 4 the tile holds
    qubits 0..rb-1, one qubit j (or none) and the rest on the highest
    qubits from 20 up; gate A takes qubit 0 and every other tile qubit, B
    the rest.  CUDA events on the context stream, `reps` launches, best of
    two; one JSON line per shape (milliseconds per launch)."""
    import numpy as np
    import qsim_gb300 as q
    from qsim_gb300 import _native as N
    ctx = q.Context(0)
    ss = q.StateSpace(ctx=ctx)
    st = ss.Create(n)
    ss.SetStateUniform(st)
    rng = np.random.default_rng(0)
    mats = []
    for _ in range(2):
        u, _ = np.linalg.qr(rng.normal(size=(64, 64)) +
                            1j * rng.normal(size=(64, 64)))
        mats.append(np.ascontiguousarray(u.astype(np.complex64)).view(np.float32))
    ma, mb = mats
    for rb in (2, 3, 4):
        for j in [rb + 1, 6, 8, 10, 11, 12, 14, 16, None]:
            tile = list(range(rb)) + ([j] if j is not None else [])
            tile += [x for x in range(n - 1, 19, -1) if x not in tile][
                :12 - len(tile)]
            tile = sorted(tile)
            if len(set(tile)) != 12:
                continue
            qa, qb = tile[0::2], tile[1::2]

            def one(qs, mat):
                N.check(N.lib.qsg_apply_gate_tc(ctx.h, st.get(), n,
                                                N.u32_array(qs), 6,
                                                mat.ctypes.data_as(N.P_f32)))

            def pair():
                N.check(N.lib.qsg_apply_gate_tc2(
                    ctx.h, st.get(), n, N.u32_array(qa), 6,
                    ma.ctypes.data_as(N.P_f32), N.u32_array(qb), 6,
                    mb.ctypes.data_as(N.P_f32)))

            one(qa, ma), one(qb, mb), pair()
            ctx.sync()
            out = {}
            for label, fn in (("two_passes_ms", lambda: (one(qa, ma),
                                                         one(qb, mb))),
                              ("pair_ms", pair)):
                ts = []
                for _ in range(2):
                    ctx.timer_start()
                    for _ in range(reps):
                        fn()
                    ts.append(ctx.timer_stop() / reps)
                out[label] = min(ts)
            print(json.dumps({"n": n, "run_bits": rb, "j": j, "qa": qa, "qb": qb,
                              **out, "ratio": out["pair_ms"] / out["two_passes_ms"],
                              "planner_factor": pair_cost_factor(n, qa, qb)}),
                  flush=True)


def ev_shapes(n: int, reps: int):
    """ExpectationValue per call (CUDA events on the context stream, the
    reduction and the read-back of the result included) on a uniform
    n-qubit state, one JSON line per operator: dense Hermitian and general
    matrices of 1..3 qubits (CUDA-core tile kernel), Pauli strings and
    phased permutations (the monomial kernels, every partner form)."""
    import ctypes as Cx
    import numpy as np
    import qsim_gb300 as q
    from qsim_gb300 import _native as N
    ctx = q.Context(0)
    ss = q.StateSpace(ctx=ctx)
    st = ss.Create(n)
    ss.SetStateUniform(st)
    rng = np.random.default_rng(0)
    pauli = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]),
             "Y": np.array([[0, -1j], [1j, 0]]), "Z": np.diag([1, -1])}
    cases = []
    for qs in ([0], [17], [0, 1], [5, 23], [0, 9, 28], [4, 12, 20]):
        d = 1 << len(qs)
        z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
        cases.append(("hermitian", qs, (z + z.conj().T) / 2))
        cases.append(("general", qs, z))
    for qs, word in (([0, 5, 9], "ZZZ"), ([0, 3, 6], "XYZ"),
                     ([0, 5, 11], "XZY"), ([1, 7, 13, 20, 26, 29], "XYZXYZ")):
        m = np.eye(1)
        for ch in word:
            m = np.kron(pauli[ch], m)
        cases.append(("pauli " + word, qs, m))
    for qs, xm in (([0, 5, 9], 0), ([3, 8], 1), ([2, 3, 19, 27], 0b1100)):
        d = 1 << len(qs)
        m = np.zeros((d, d), complex)
        for r in range(d):
            m[r, r ^ xm] = np.exp(1j * rng.uniform(0, 2 * np.pi))
        cases.append(("monomial", qs, m))
    out = (Cx.c_double * 2)()
    for kind, qs, mat in cases:
        qs = [x for x in qs if x < n]
        if len(qs) != int(np.log2(len(mat))):
            continue
        m32 = np.ascontiguousarray(mat.astype(np.complex64)).view(np.float32)

        def f():
            N.check(N.lib.qsg_expectation_value(
                ctx.h, st.get(), n, N.u32_array(qs), len(qs),
                m32.ctypes.data_as(N.P_f32), out))

        f(), f()
        ts = []
        for _ in range(3):
            ctx.timer_start()
            for _ in range(reps):
                f()
            ts.append(ctx.timer_stop() / reps)
        ms = min(ts)
        print(json.dumps({"n": n, "operator": kind, "qs": qs, "ms": ms,
                          "alg_gbs": 8 * (1 << n) / (ms * 1e-3) / 1e9,
                          "ev": [out[0], out[1]]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel-case", default=None,
                    help='profiling case "gate:q,..." or "tc:q,..."')
    ap.add_argument("--ev-shapes", action="store_true",
                    help="ExpectationValue per call by operator kind "
                         "(--qubits, --reps), then exit")
    ap.add_argument("--pair-shapes", action="store_true",
                    help="two-gate pass against two passes by tile shape "
                         "(--qubits, --reps), then exit")
    ap.add_argument("--qubits", type=int, default=26)
    ap.add_argument("--reps", type=int, default=4)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precision-all", action="store_true",
                    help="also check the learned plan of the 28-qubit layered "
                         "circuit against the FP64 oracle")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the planner and trajectory sections")
    ap.add_argument("--distinct-replicas", action="store_true")
    ap.add_argument("--traj-only", action="store_true",
                    help="run only the batched-trajectory workload")
    ap.add_argument("--traj-streams", type=int, default=8)
    ap.add_argument("--traj-f", type=int, default=0,
                    help="stream-path fusion size (0: autotuned; 5, 6 use "
                         "the tensor cores)")
    ap.add_argument("--traj-mode", default="auto",
                    choices=["auto", "packed", "streams"])
    ap.add_argument("--traj-split", type=int, default=-1,
                    help="largest qubit count run in the packed kernel")
    ap.add_argument("--hybrid-case", default=None, choices=["plain", "tc"],
                    help="one small qsimh job (for ncu captures), then exit")
    ap.add_argument("--traj-ctas-per-sm", type=int, default=0)
    ap.add_argument("--traj-tile-kib", type=int, default=0)
    args = ap.parse_args()
    if args.kernel_case:
        kernel_case(args.kernel_case, args.qubits, args.reps)
        return
    if args.pair_shapes:
        pair_shapes(args.qubits, args.reps)
        return
    if args.ev_shapes:
        ev_shapes(args.qubits, args.reps)
        return
    if args.hybrid_case:
        hybrid_case(args.hybrid_case == "tc")
        return
    if args.traj_only:
        print(json.dumps({"trajectories": bench_trajectories(
            args.traj_streams, args.traj_f, mode=args.traj_mode,
            ctas_per_sm=args.traj_ctas_per_sm, tile_kib=args.traj_tile_kib,
            split=args.traj_split)}), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    rc = self_launch(args)
    if rc is not None:
        sys.exit(rc)
    world, rank, local, dist = dist_setup()
    try:
        if args.impl == "reference":
            run_reference(args, world, rank, dist)
        else:
            run_engine(args, world, rank, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
