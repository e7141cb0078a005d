"""Learned fusion planner: the cost-model network, the engine-recorded
training data, and training on the device.

    python -m qsim_gb300.learned collect --circuits 2000 --out timings.npz
    python -m qsim_gb300.learned train --data timings.npz --out cost_mlp.npz

`collect` fuses seeded random grid circuits of 24..32 qubits with random
block-size limits and paths, runs each plan with a CUDA event around every
launch (qsg_plan_profile) and records, per launch, the block's features and
its time.  `train` fits the network with the library's own device kernels
(forward, backward, Adam).  A trained network, passed to
engine.Plan(cost_model=...), makes the planner pick block boundaries, block
sizes and paths by predicted time; the weights trained on GB300 timings are
kept in qsim_gb300/data/cost_mlp_gb300.npz.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import time

import numpy as np

from . import _native as N
from ._native import check

N_FEATURES = 16
DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DEFAULT_WEIGHTS = os.path.join(DATA_DIR, "cost_mlp_gb300.npz")


def _f32p(a):
    return a.ctypes.data_as(N.P_f32)


class CostMLP:
    """The cost-model network (qsg_mlp)."""

    def __init__(self, seed: int = 1):
        h = C.c_void_p()
        check(N.lib.qsg_mlp_create(seed, C.byref(h)))
        self.h = h

    @property
    def num_params(self) -> int:
        return int(N.lib.qsg_mlp_num_params())

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, dtype=np.float32)
        check(N.lib.qsg_mlp_get_params(self.h, _f32p(p)))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params
        check(N.lib.qsg_mlp_set_params(self.h, _f32p(p)))

    def save(self, path: str, **meta) -> None:
        np.savez(path, params=self.get_params(), **meta)

    @classmethod
    def load(cls, path: str = DEFAULT_WEIGHTS) -> "CostMLP":
        m = cls()
        with np.load(path) as z:
            m.set_params(z["params"])
        return m

    # ---- device work --------------------------------------------------
    def gradient(self, ctx, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_double()
        check(N.lib.qsg_mlp_gradient(ctx.h, self.h, _f32p(x), _f32p(y), len(y),
                                     _f32p(g), C.byref(loss)))
        return loss.value, g

    def train(self, ctx, x, y, steps=4000, batch=1024, lr=1e-3, seed=1):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_double()
        check(N.lib.qsg_mlp_train(ctx.h, self.h, _f32p(x), _f32p(y), len(y),
                                  steps, batch, lr, seed, C.byref(loss)))
        return loss.value

    def predict(self, ctx, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros(len(x), dtype=np.float32)
        check(N.lib.qsg_mlp_predict(ctx.h, self.h, _f32p(x), len(x), _f32p(out)))
        return out

    # ---- host inference -------------------------------------------------
    def cost_us(self, n, qs, ncontrols=0, path=0) -> float:
        out = C.c_double()
        check(N.lib.qsg_mlp_cost_us(self.h, n, N.u32_array(qs), len(qs),
                                    ncontrols, path, C.byref(out)))
        return out.value

    def __del__(self):
        try:
            N.lib.qsg_mlp_destroy(self.h)
        except Exception:
            pass


def features(n, qs, ncontrols=0, path=0) -> np.ndarray:
    """Feature vector of one launch (qs as launched: padded to six for the
    tensor-core path)."""
    out = np.zeros(N_FEATURES, dtype=np.float32)
    check(N.lib.qsg_block_features(n, N.u32_array(qs), len(qs), ncontrols, path,
                                   _f32p(out)))
    return out


def time_target(n, us):
    """log(us) - (n - 24) log 2: the network's output for a launch."""
    return np.log(us) - (np.asarray(n, dtype=np.float64) - 24.0) * np.log(2.0)


GRID_SHAPES = {}  # n -> list of (rows, cols, extra)
for _r in range(3, 9):
    for _c in range(_r, 9):
        for _e in range(0, _c):
            GRID_SHAPES.setdefault(_r * _c + _e, []).append((_r, _c, _e))


def collect(ctx, num_circuits=2000, seed=7, n_min=24, n_max=32, log=None):
    """Engine-recorded launch times of seeded random grid circuits.

    The qubit count of circuit i is drawn with probability proportional to
    2^-(n - n_min) (so that the large states, whose launches are slow, take
    a bounded share of the time); the depth, block-size limit (1..6), path
    and tensor-core threshold are drawn uniformly; 15 % of the circuits are
    layered U3 circuits with controlled gates, the rest grid circuits.  Every plan is profiled
    twice and the smaller time of each launch kept.  Returns (X, y, n, us)."""
    from . import api
    from .engine import Circuit, Plan
    rng = np.random.default_rng(seed)
    ns = np.arange(n_min, n_max + 1)
    w = 2.0 ** -(ns - n_min)
    w /= w.sum()
    ss = api.StateSpace(ctx=ctx)
    states = {}
    X, Y, NQ, US = [], [], [], []
    t0 = time.time()
    for i in range(num_circuits):
        n = int(rng.choice(ns, p=w))
        shapes = GRID_SHAPES[n]
        rows, cols, extra = shapes[int(rng.integers(len(shapes)))]
        depth = int(rng.integers(4, 13))
        f = int(rng.integers(1, 7))
        tensor = bool(rng.integers(0, 2)) and f >= 2
        tc_min = int(rng.integers(2, 7))
        if rng.random() < 0.15:
            # Layered U3 circuits bring controlled gates into the data.
            c = Circuit.layered_u3(n, max(2, depth // 2), 4, 10_000 + i)
        else:
            c = Circuit.grid(rows, cols, extra, depth, 10_000 + i)
        plan = Plan(c, max_fused_size=f, tensor_path=tensor, tc_min_k=tc_min)
        if n not in states:
            st = ss.Create(n)
            if ss.IsNull(st):
                continue
            ss.SetStateUniform(st)
            states[n] = st
        st = states[n]
        t1 = plan.profile(ctx, st)
        t2 = plan.profile(ctx, st)
        ms = np.minimum(t1, t2)
        for o, t in zip(plan.ops(), ms):
            if o["kind"] == 2 or t <= 0:
                continue
            X.append(features(n, o["qs"], len(o["cqs"]), o["path"]))
            us = float(t) * 1e3
            Y.append(time_target(n, us))
            NQ.append(n)
            US.append(us)
        if log and (i + 1) % 100 == 0:
            log(f"{i + 1}/{num_circuits} circuits, {len(Y)} launches, "
                f"{time.time() - t0:.1f} s")
    return (np.array(X, np.float32), np.array(Y, np.float32),
            np.array(NQ, np.int32), np.array(US, np.float64))


def _main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("collect")
    a.add_argument("--circuits", type=int, default=2000)
    a.add_argument("--seed", type=int, default=7)
    a.add_argument("--out", required=True)
    b = sub.add_parser("train")
    b.add_argument("--data", required=True)
    b.add_argument("--out", required=True)
    b.add_argument("--steps", type=int, default=6000)
    b.add_argument("--batch", type=int, default=1024)
    b.add_argument("--lr", type=float, default=1e-3)
    b.add_argument("--seed", type=int, default=1)
    args = ap.parse_args()
    from . import api
    ctx = api.Context(0)
    if args.cmd == "collect":
        X, y, nq, us = collect(ctx, args.circuits, args.seed, log=print)
        np.savez_compressed(args.out, X=X, y=y, n=nq, us=us,
                            circuits=args.circuits, seed=args.seed)
        print(f"{len(y)} launches written to {args.out}")
    else:
        with np.load(args.data) as z:
            X, y = z["X"], z["y"]
        # Hold out every tenth launch to report generalisation.
        test = np.arange(len(y)) % 10 == 0
        m = CostMLP(args.seed)
        t0 = time.time()
        loss = m.train(ctx, X[~test], y[~test], args.steps, args.batch, args.lr,
                       args.seed)
        dt = time.time() - t0
        held = float(np.mean((m.predict(ctx, X[test]) - y[test]) ** 2))
        m.save(args.out, train_mse=loss, test_mse=held, steps=args.steps,
               batch=args.batch, lr=args.lr, seed=args.seed,
               samples=int((~test).sum()), train_seconds=dt)
        print(f"train mse {loss:.5f}, held-out mse {held:.5f} "
              f"(rms {np.sqrt(held):.3f} in log time), {dt:.2f} s")


if __name__ == "__main__":
    _main()
