"""Autotuner for batched trajectories on this GPU.

qsim has no tuner: its RunBatch (lib/qtrajectory.h:141-236) runs every
repetition the same way.  Here a batch can run three ways, all on the same
device code: one persistent kernel over the packed batch (each CTA a whole
trajectory, Kraus choices on the device), the stream path (one launch per
fused block, several host threads), or both at once with the circuits split
by qubit count.  The tuner times candidate configurations on a sample of
the batch and keeps the one with the most trajectories per second:

  * the stream path's form: fusion block size k (3 or 4 on CUDA cores),
    and ``tc_from``: circuits of at least that many qubits fuse at k = 6
    with blocks of >= 5 qubits on the tensor cores (a tensor-core pass
    needs 4096-amplitude tiles on every SM to pay off, so small circuits
    stay on CUDA cores);
  * ``split``: the largest qubit count sent to the persistent kernel (whose
    runners fuse at k = 4 on CUDA cores); the rest run concurrently on the
    stream path;
  * ``ctas_per_sm`` and ``tile_kib``: the persistent kernel's residency and
    the shared-memory tile budget of its pipelined gate passes.

Results are cached per (GPU, workload signature) in a JSON file
(``QSG_AUTOTUNE_CACHE`` or ``~/.cache/qsim_gb300/autotune.json``), so a
repeated workload is tuned once.  Tuning never changes results: every
configuration makes the reference's Kraus choices from the same draws.
"""
from __future__ import annotations

import hashlib
import json
import os
import time

from . import engine as E


def _cache_path() -> str:
    p = os.environ.get("QSG_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "qsim_gb300",
                        "autotune.json")


def _device_key(device: int) -> str:
    from . import _native as N
    import ctypes as C
    ctx = C.c_void_p()
    N.check(N.lib.qsg_ctx_create(device, None, C.byref(ctx)))
    sms = C.c_int()
    N.check(N.lib.qsg_ctx_num_sms(ctx, C.byref(sms)))
    N.lib.qsg_ctx_destroy(ctx)
    name = "gpu"
    try:
        import torch
        name = torch.cuda.get_device_name(device)
    except Exception:  # torch is optional here
        pass
    return f"{name}/{sms.value}sm"


def signature(qubits, reps: int, tag: str = "") -> str:
    """Workload signature: the circuits' qubit counts, repetitions and a
    caller tag (for example the noise model)."""
    h = hashlib.sha1(json.dumps([sorted(int(q) for q in qubits), int(reps),
                                 tag]).encode()).hexdigest()
    return h[:16]


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p + ".tmp", "w") as f:
            json.dump(db, f, indent=1)
        os.replace(p + ".tmp", p)
    except OSError:
        pass  # an unwritable cache only costs a re-tune


FORMS = ((3, False), (4, False), (6, True))


def candidates(max_n: int, forms=FORMS):
    """Configurations tried: each CUDA-core stream form alone or with the
    largest circuits on the tensor cores (tc_from), with or without the
    small circuits in the persistent kernel (split), and all circuits in the
    persistent kernel.  forms: (k, tensor) pairs; a tensor form enables the
    tc_from tiers."""
    cuda_fs = [f for f, tc in forms if not tc]
    tc_ok = any(tc for _, tc in forms)
    tc_froms = [0] + ([t for t in (20, 22, 24) if t <= max_n] if tc_ok else [])
    splits = [0] + [t for t in (14, 16) if t < max_n]
    out = []
    for f in cuda_fs or [4]:
        for tc_from in tc_froms:
            for split in splits:
                for per_sm in ((1, 2) if split else (0,)):
                    out.append(dict(max_fused_size=f, tensor=False,
                                    tc_from=tc_from, split=split,
                                    ctas_per_sm=per_sm,
                                    tile_kib=32 if split else 0))
    out.append(dict(max_fused_size=4, tensor=False, tc_from=0, split=max_n,
                    ctas_per_sm=2, tile_kib=32))
    return out


def runners_for(make_runners, qubits, cfg):
    """Per circuit: the packed kernel's runner (k = 4, CUDA cores) for
    circuits of at most cfg["split"] qubits, a tensor-core runner (k = 6)
    for circuits of at least cfg["tc_from"] qubits (0: none), the stream
    form's otherwise."""
    packed = make_runners(4, False)
    other = make_runners(cfg["max_fused_size"], cfg.get("tensor", False))
    tc_from = cfg.get("tc_from", 0)
    tcr = make_runners(6, True) if tc_from else None
    out = []
    for i, n in enumerate(qubits):
        n = int(n)
        if tc_from and n >= tc_from and n > cfg["split"]:
            out.append(tcr[i])
        elif n <= cfg["split"]:
            out.append(packed[i])
        else:
            out.append(other[i])
    return out


def run(runners, items, cfg, num_streams: int = 8, out_states=None,
        device: int = 0):
    """Runs `items` [(runner index, rep)] with configuration `cfg` (split 0:
    stream path only) on GPU `device`; returns (per-item stats, latency_ms,
    wall seconds, launches, info)."""
    if cfg["split"] == 0:
        per, lat, wall, launches = E.run_trajectory_batch(
            runners, items, num_streams=num_streams, device=device,
            out_states=out_states, return_launches=True)
        return per, lat, wall, launches, None
    return E.run_trajectory_batch_packed(
        runners, items, ctas_per_sm=cfg["ctas_per_sm"],
        max_qubits=cfg["split"], tile_kib=cfg["tile_kib"],
        num_streams=num_streams, device=device, overlap=True,
        out_states=out_states)


def tune_trajectories(make_runners, qubits, reps: int, tag: str = "",
                      sample_reps: int = 0, forms=FORMS, device: int = 0,
                      num_streams: int = 8, use_cache: bool = True):
    """Chooses the configuration with the most trajectories/s.

    make_runners(f, tensor) returns the runners (one per circuit, in the
    order of `qubits`) fused at max_fused_size f, with blocks of >= 5 qubits
    on the tensor cores when `tensor`; the batch is every circuit times
    `reps` repetitions.  Candidates are timed on `sample_reps` repetitions
    per circuit (default reps / 8, at least 1), after one warm-up run each.
    Returns {"best": cfg, "table": [(cfg, traj/s), ...], "cached": bool,
    "tune_s": seconds}."""
    key = _device_key(device) + "/" + signature(qubits, reps, tag)
    db = _load() if use_cache else {}
    if use_cache and key in db:
        return {"best": db[key]["best"], "table": db[key]["table"],
                "cached": True, "tune_s": 0.0}
    t0 = time.perf_counter()
    sample_reps = sample_reps or max(1, reps // 8)
    max_n = max(int(q) for q in qubits)
    table = []
    for cfg in candidates(max_n, forms):
        runners = runners_for(make_runners, qubits, cfg)
        items = [(i, 10**6 + r) for i in range(len(runners))
                 for r in range(sample_reps)]
        run(runners, items[:len(runners)], cfg, num_streams,
            device=device)  # warm-up
        _, _, wall, _, _ = run(runners, items, cfg, num_streams,
                               device=device)
        table.append((cfg, len(items) / wall))
    best = max(table, key=lambda x: x[1])[0]
    if use_cache:
        db[key] = {"best": best, "table": table}
        _store(db)
    return {"best": best, "table": table, "cached": False,
            "tune_s": time.perf_counter() - t0}
