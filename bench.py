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
`e2e` is the same run through the public API with host buffers: plan
applied through the C ABI, 1000 samples and the full final state copied to
pinned host memory inside each timed step.

Multi-GPU: the path does not shard (one state per GPU), so N > 1 runs N
independent replicas; value = total runs / max-over-ranks time.

--impl reference times the reference's CPU algorithm on the host cores (the
oracle's OpenMP FP32 port of SimulatorBasic; the reference's own code is not
present on the GPU host), on a bounded sample of the same workload: the
first fused ops of the same f=4 plan, extrapolated to the whole circuit.
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


def traffic_from_profiles(n: int, kernel: str):
    """dram read+write bytes per launch of `kernel`, from its committed ncu
    summary (scaled from the capture's qubit count to n: traffic grows in
    proportion to the state)."""
    name = {"gate_tile_kernel": "gate_tile_k4_plain_pass.md",
            "tc_gate_kernel": "tc_gate_k6_pass.md"}.get(kernel)
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
def cpu_sample(n: int, plan_ops, max_ops: int, threads: int | None = None):
    """Times the oracle's OpenMP FP32 port on the first fused ops of the
    plan at full size; returns (seconds, ops timed, threads)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import Oracle
    orc = Oracle()
    if threads:
        orc.L.orc_set_num_threads(threads)
    nthreads = orc.L.orc_num_threads()
    st = np.zeros(2 << n, dtype=np.float32)
    st[0] = 1.0
    P = C.POINTER
    t_total, done = 0.0, 0
    for o in plan_ops[:max_ops]:
        m = np.ascontiguousarray(o["m"].astype(np.complex64)).view(np.float32)
        qs = (C.c_uint * max(1, len(o["qs"])))(*o["qs"])
        t0 = time.perf_counter()
        orc.L.orc_apply_gate_f32(st.ctypes.data_as(P(C.c_float)), n, qs,
                                 len(o["qs"]), m.ctypes.data_as(P(C.c_float)))
        t_total += time.perf_counter() - t0
        done += 1
        if t_total > 20.0:
            break
    return t_total, done, nthreads


def run_reference(args, world, rank, dist):
    if rank != 0:
        return
    from qsim_gb300 import engine as E
    c = E.Circuit.grid(GRID["rows"], GRID["cols"], GRID["extra"],
                       GRID["cycles"], GRID["seed"])
    n = c.num_qubits
    plan = E.Plan(c, max_fused_size=4)
    ops = plan.ops()
    per_step = []
    for _ in range(args.warmup + args.steps):
        t, done, threads = cpu_sample(n, ops, args.cpu_ops)
        per_step.append(t * len(ops) / done)
    vals = per_step[args.warmup:]
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "max_fused_size": 4,
                   "fused_ops": len(ops)},
        "cpu_baseline": {
            "value": v, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {done} of {len(ops)} fused ops (f=4 plan) of "
                      f"the 30-qubit circuit on an 8 GiB FP32 host state, "
                      f"extrapolated by op count"},
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
    ctx = q.Context(0)
    ss = q.StateSpace(ctx=ctx)
    c = E.Circuit.grid(GRID["rows"], GRID["cols"], GRID["extra"],
                       GRID["cycles"], GRID["seed"] + (rank if args.distinct_replicas else 0))
    n = c.num_qubits
    nbytes_state = 8 << n
    st = ss.Create(n)
    if ss.IsNull(st):
        raise RuntimeError("not enough device memory for the 30-qubit state")

    forms = {}
    forms["plain_f4"] = E.Plan(c, max_fused_size=4)
    forms["plain_f5"] = E.Plan(c, max_fused_size=5)
    forms["plain_f6"] = E.Plan(c, max_fused_size=6)
    # Tensor-core forms: blocks of >= tc_min_k qubits on tcgen05.
    forms["tc_f6"] = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=5)
    # Learned planner: block boundaries, sizes and paths from the cost model
    # trained on this engine's GB300 launch times.
    model = L.CostMLP.load()
    forms["learned_tc_f6"] = E.Plan(c, max_fused_size=6, tensor_path=True,
                                    tc_min_k=2, cost_model=model)
    forms["tc_f6_all"] = E.Plan(c, max_fused_size=6, tensor_path=True, tc_min_k=1)
    forms["tc_f5_all"] = E.Plan(c, max_fused_size=5, tensor_path=True, tc_min_k=1)

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
    best = min(results, key=results.get)
    head = forms[best]
    launches_before += args.warmup * (kernels[best] + 2)

    # Headline timed region: K steps of the best form.
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
    ms = max_over_ranks(dist, ms)
    value = ms / 1e3

    # Roofline of the dominant kernel of the headline plan: per-op CUDA-event
    # times; algorithmic bytes per launch = 16 * 2^n (one read + one write
    # of the state).
    ss.SetStateZero(st)
    prof = head.profile(ctx, st)
    hops = head.ops()
    kern_of = lambda o: "tc_gate_kernel" if o["path"] == 1 else "gate_tile_kernel"
    per_kernel = {}
    for t, o in zip(prof, hops):
        d = per_kernel.setdefault(kern_of(o), {"launches": 0, "total_ms": 0.0})
        d["launches"] += 1
        d["total_ms"] += float(t)
    dom = max(per_kernel, key=lambda kname: per_kernel[kname]["total_ms"])
    for kname, d in per_kernel.items():
        d["avg_ms"] = d["total_ms"] / d["launches"]
        d["gbs"] = 16.0 * (1 << n) / (d["avg_ms"] * 1e-3) / 1e9
        d["share"] = d["total_ms"] / float(np.sum(prof))
    achieved = per_kernel[dom]["gbs"]
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": traffic_from_profiles(n, dom),
                "kernel": dom, "peak_source": peak_kind,
                "bytes_per_launch": 16 * (1 << n),
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

    # End to end through the public API with host buffers.
    hbuf = C.c_void_p()
    N.check(N.lib.qsg_host_alloc(nbytes_state, C.byref(hbuf)))
    samples = np.zeros(1000, dtype=np.uint64)
    h2d = sum(8 * (1 << (2 * len(o["qs"]))) for o in head.ops())
    e2e_times, phases = [], []
    for i in range(args.warmup + args.steps):
        ctx.sync()
        barrier(dist)
        t0 = time.perf_counter()
        ss.SetStateZero(st)
        head.run(ctx, st)
        N.check(N.lib.qsg_sample(ctx.h, st.get(), n, 1000, 1,
                                 samples.ctypes.data_as(N.P_u64)))
        t1 = time.perf_counter()   # the samples synchronise the stream
        N.check(N.lib.qsg_copy_d2h(ctx.h, hbuf, st.get(), n))
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(dt)
            phases.append((t1 - t0, dt - (t1 - t0)))
    N.lib.qsg_host_free(hbuf)
    e2e = max_over_ranks(dist, statistics.median(e2e_times))
    e2e_phase = {"run_and_sample_s": statistics.median(p[0] for p in phases),
                 "state_d2h_s": statistics.median(p[1] for p in phases)}
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
                                  split=args.traj_split)
        traj["wall_s"] = max_over_ranks(dist, traj["wall_s"])
        traj["value"] = world * traj["trajectories"] / traj["wall_s"]
        alt = bench_trajectories(args.traj_streams, 4, mode="streams")
        traj["streams_only"] = {"value": alt["value"], "wall_s": alt["wall_s"],
                                "latency_ms_p50": alt["latency_ms_p50"],
                                "latency_ms_p99": alt["latency_ms_p99"],
                                "gpu_launches": alt["gpu_launches"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        t, done, threads = cpu_sample(n, ops4, args.cpu_ops)
        cpu = {"value": t * len(ops4) / done, "unit": UNIT, "cores": threads,
               "kind": "port",
               "sample": f"first {done} of {len(ops4)} fused ops of the f=4 "
                         f"plan on an 8 GiB FP32 host state (oracle OpenMP "
                         f"port of SimulatorBasic), extrapolated by op count"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value / 1.0, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": best,
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
    Pauli strings of weight 1..6: seconds per circuit run (plain f = 4 plan
    from a CUDA graph) and per expectation value, on the one-pass monomial
    kernel and, for comparison, on the dense tile kernel (the same operator
    with one off-pattern entry of 1e-30, which the monomial test rejects)."""
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

    c = E.Circuit.layered_u3(EXPECT["n"], EXPECT["layers"], EXPECT["controlled"],
                             EXPECT["seed"])
    n = c.num_qubits
    st = ss.Create(n)
    plan = E.Plan(c, max_fused_size=4)
    plan.capture(ctx, st)
    ss.SetStateZero(st)
    plan.replay(ctx)
    ctx.sync()
    barrier(dist)
    ctx.timer_start()
    ss.SetStateZero(st)
    plan.replay(ctx)
    circuit_s = max_over_ranks(dist, ctx.timer_stop() / 1e3)
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
        "circuit_s_per_run": circuit_s, "passes": len(plan),
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
    opts = dict(max_fused_size=6, tensor_path=True)
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
                        "(tensor-core f = 6)",
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
                orc.L.orc_apply_gate_f32(st.ctypes.data_as(P(C.c_float)), np_,
                                         qa, len(qs),
                                         m.ctypes.data_as(P(C.c_float)))
            t_total += time.perf_counter() - t0
        done += 1
        if t_total > 15.0:
            break
    per_path = t_total / done
    return {"value": per_path * paths, "unit": "s/job",
            "cores": orc.L.orc_num_threads(), "kind": "port",
            "sample": f"{done} sample paths (both parts' post-checkpoint "
                      f"gates fused into <= 2-qubit blocks, oracle OpenMP "
                      f"FP32 port), x {paths} paths"}


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
             "tc_f6": E.Plan(c, max_fused_size=6, tensor_path=True)}
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
        out[name] = {"s_per_unitary": t, "passes": len(plan),
                     "gbs_per_pass": 16.0 * entries * len(plan) / t / 1e9}
    res = {"workload": f"unitary of the {n}-qubit 2x7 grid depth-14 circuit "
                       f"(seed 1), {entries} complex64 entries",
           "forms": out,
           "best": min(out, key=lambda k: out[k]["s_per_unitary"])}
    us_best = out[res["best"]]["s_per_unitary"]
    del u
    if cpu:
        ops = forms["plain_f4"].ops()
        t, done, threads = cpu_sample(2 * n, ops, 4)
        v = t * len(ops) / done
        res["cpu_baseline"] = {
            "value": v, "unit": "s/unitary", "cores": threads, "kind": "port",
            "sample": f"first {done} of {len(ops)} fused ops (f=4 plan) on "
                      f"the 2 GiB FP32 host unitary, extrapolated by op count"}
        res["speedup_vs_cpu"] = v / us_best
    return res


LEARN_GRID = dict(rows=5, cols=6, extra=2, cycles=24, seed=1)


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
    }
    st = ss.Create(n)
    ref = ss.Create(n)
    if ss.IsNull(st) or ss.IsNull(ref):
        return {"skipped": "not enough device memory for two 32-qubit states"}
    times, predicted = {}, {}
    for name, p in forms.items():
        p.capture(ctx, st)
        ss.SetStateZero(st)
        p.replay(ctx)
        ctx.sync()
        barrier(dist)
        ctx.timer_start()
        ss.SetStateZero(st)
        p.replay(ctx)
        times[name] = max_over_ranks(dist, ctx.timer_stop() / 1e3)
        predicted[name] = sum(model.cost_us(n, o["qs"], len(o["cqs"]), o["path"])
                              for o in p.ops() if o["kind"] != 2) / 1e6
        if name == "plain_f4":
            ss.Copy(st, ref)
    ip = C.c_double * 2
    r = ip()
    N.check(N.lib.qsg_inner_product(ctx.h, ref.get(), st.get(), n, r))
    fid = (r[0] ** 2 + r[1] ** 2) / (ss.Norm(ref) * ss.Norm(st))
    fixed = {k: v for k, v in times.items() if k != "learned_tc_f6"}
    best_fixed = min(fixed, key=fixed.get)
    return {
        "workload": "grid5x6+2 (32 qubits) random circuit depth 24, seed 1, "
                    "complex64 (32 GiB)",
        "unit": "s/run", "forms_s": times, "predicted_s": predicted,
        "passes": {k: len(v) for k, v in forms.items()},
        "learned_vs_best_fixed": times[best_fixed] / times["learned_tc_f6"],
        "best_fixed": best_fixed,
        "learned_vs_plain_f4": times["plain_f4"] / times["learned_tc_f6"],
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
                       tile_kib: int = 0, split: int = -1):
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
            forms=forms, num_streams=num_streams, use_cache=False)
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
    AT.run(runners, [(i, 10**6) for i in range(len(runners))], cfg, num_streams)
    per, lat, wall, launches, info = AT.run(runners, items, cfg, num_streams)
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


def kernel_case(spec: str, n: int, reps: int):
    """Small profiling case on a uniform n-qubit state, `reps` launches of
    one kind:

      gate:q0,q1,..           CUDA-core tile kernel (random unitary)
      tc:q0,..                tensor-core kernel (random unitary)
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
        "gate", "tc", "ctrl", "ev", "evp") else []
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
    out2 = (Cx.c_double * 2)()
    smp = np.zeros(1000, dtype=np.uint64)
    for _ in range(reps):
        if kind == "tc":
            N.check(N.lib.qsg_apply_gate_tc(ctx.h, st.get(), n, N.u32_array(qs),
                                            k, m.ctypes.data_as(N.P_f32)))
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel-case", default=None,
                    help='profiling case "gate:q,..." or "tc:q,..."')
    ap.add_argument("--qubits", type=int, default=26)
    ap.add_argument("--reps", type=int, default=4)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-ops", type=int, default=4,
                    help="fused ops timed on the CPU for the baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
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
