"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of qsim's hybrid
Schrodinger-Feynman simulator (lib/hybrid.h, lib/run_qsimh.h).

Used by tests/ to check the GPU hybrid simulator; pinned to the reference's
own outputs (tests/golden/hybrid*.npz, written by tests/golden/make_golden.py
from the reference's QSimHRunner and from its known-answer tests).

The circuit arrives as operations (dicts with "kind", "time", "qs" sorted,
"m" the 2^k x 2^k matrix with bit j <-> qs[j], and for two-qubit gates
"schmidt": a list of (A, B) 2x2 factors, A on qs[0], with m = sum A (x) B).

  * SplitLattice (lib/hybrid.h:131-277): gates inside a part go to that part
    (local qubits numbered in global order within the part); gates across
    the cut become one factor on each side; cut gates are ordered by time,
    then circuit order, and take 0, 1 or 2 path bits (Schmidt rank 1, 2,
    3-4: SchmidtBits, :586-600).
  * Run (:290-437): with the first num_prefix gates' terms fixed by
    `prefix` and the root and suffix gates' terms enumerated, the amplitude
    of bitstring x is sum over paths of a0[path][x0] * a1[path][x1]; paths
    whose index selects a missing term are skipped (SetSchmidtMatrices,
    :512-541).  Here all paths run at once along a batch axis (paths whose
    term is missing contribute zero), each part simulated densely.
"""
from __future__ import annotations

import numpy as np


def _bits(terms: int) -> int:
    return 0 if terms <= 1 else 1 if terms == 2 else 2


def _apply(state: np.ndarray, n: int, qs, m: np.ndarray) -> np.ndarray:
    """state (B, 2^n); m (2^k, 2^k) or per path (B, 2^k, 2^k)."""
    B, k = state.shape[0], len(qs)
    t = state.reshape([B] + [2] * n)
    axes = [1 + (n - 1 - q) for q in reversed(qs)]
    front = list(range(1, k + 1))
    t = np.moveaxis(t, axes, front).reshape(B, 1 << k, -1)
    if m.ndim == 2:
        t = np.einsum("ij,bjr->bir", m, t)
    else:
        t = np.einsum("bij,bjr->bir", m, t)
    t = np.moveaxis(t.reshape([B] + [2] * n), front, axes)
    return np.ascontiguousarray(t).reshape(B, 1 << n)


def split_lattice(n: int, ops, parts):
    """Returns (n0, n1, local map, part op lists, cut gates)."""
    assert len(parts) == n
    local, cnt = [], [0, 0]
    for q in range(n):
        local.append(cnt[parts[q]])
        cnt[parts[q]] += 1
    part_ops = [[], []]
    cuts = []
    for i, o in enumerate(ops):
        if o["kind"] != 0 or len(o["qs"]) not in (1, 2):
            raise ValueError("only one- and two-qubit matrix gates")
        qs = o["qs"]
        p0 = parts[qs[0]]
        if len(qs) == 1 or parts[qs[1]] == p0:
            part_ops[p0].append(dict(time=o["time"], cut=-1,
                                     qs=[local[q] for q in qs], m=o["m"]))
            continue
        terms = o["schmidt"]
        if not terms:
            raise ValueError("no Schmidt decomposition")
        f = [None, None]
        f[p0] = [a for a, _ in terms]
        f[1 - p0] = [b for _, b in terms]
        q = [None, None]
        q[p0], q[1 - p0] = local[qs[0]], local[qs[1]]
        cuts.append(dict(time=o["time"], order=i, f=f, q=q, terms=len(terms),
                         bits=_bits(len(terms))))
    cuts.sort(key=lambda g: (g["time"], g["order"]))
    for j, g in enumerate(cuts):
        for p in (0, 1):
            part_ops[p].append(dict(time=g["time"], cut=j))
    for p in (0, 1):
        part_ops[p].sort(key=lambda o: (o["time"], o["cut"] >= 0, o["cut"]))
    return cnt[0], cnt[1], local, part_ops, cuts


def hybrid_amplitudes(n: int, ops, parts, bitstrings, prefix: int = 0,
                      num_prefix: int = 0, num_root: int = 0) -> np.ndarray:
    n0, n1, local, part_ops, cuts = split_lattice(n, ops, parts)
    G = len(cuts)
    if num_prefix + num_root > G:
        raise ValueError("num_prefix + num_root > gates on the cut")
    # Prefix terms from `prefix`; every later gate's bits come from the
    # enumerated path index (root bits first, then suffix bits).
    k_fixed = {}
    sh = 0
    for j in range(num_prefix):
        g = cuts[j]
        if g["bits"] == 0:
            k_fixed[j] = 0
            continue
        k = (prefix >> sh) & ((1 << g["bits"]) - 1)
        sh += g["bits"]
        if k >= g["terms"]:
            raise ValueError("invalid prefix")
        k_fixed[j] = k
    offs, tot = {}, 0
    for j in range(num_prefix, G):
        offs[j] = tot
        tot += cuts[j]["bits"]
    B = 1 << tot
    b = np.arange(B, dtype=np.int64)
    states = []
    for p, np_ in ((0, n0), (1, n1)):
        s = np.zeros((B, 1 << np_), np.complex128)
        s[:, 0] = 1.0
        for o in part_ops[p]:
            if o["cut"] < 0:
                s = _apply(s, np_, o["qs"], np.asarray(o["m"], np.complex128))
                continue
            j = o["cut"]
            g = cuts[j]
            fac = np.asarray(g["f"][p], np.complex128)           # (terms, 2, 2)
            if j in k_fixed:
                s = _apply(s, np_, [g["q"][p]], fac[k_fixed[j]])
                continue
            k = (b >> offs[j]) & ((1 << g["bits"]) - 1)
            m = np.zeros((B, 2, 2), np.complex128)
            ok = k < g["terms"]
            m[ok] = fac[k[ok]]
            s = _apply(s, np_, [g["q"][p]], m)
        states.append(s)
    out = np.zeros(len(bitstrings), np.complex128)
    for i, x in enumerate(bitstrings):
        i0 = i1 = 0
        for q in range(n):
            bit = (int(x) >> q) & 1
            if parts[q]:
                i1 |= bit << local[q]
            else:
                i0 |= bit << local[q]
        out[i] = np.sum(states[0][:, i0] * states[1][:, i1])
    return out
