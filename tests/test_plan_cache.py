"""Fused-plan cache (qsg_plan_cache): QSimRunner::Run (lib/run_qsim.h:225-289)
with the fused plan kept per circuit content.

CPU: the cache's bookkeeping calls need no GPU, and a run without a context
is a status code.  GPU: a text circuit (every gate of the text format, the
reference's own final state in tests/golden/text_gates9.npz) run twice hits
the cache and replays its CUDA graph with the same result (bit-identical to
an uncached plan run, relative L2 <= 1e-5 against the reference); options,
maxtime and circuit content are part of the key; measurements inside a
cached plan draw the same bits as qsg_plan_run; LRU eviction; a new state
recaptures."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden, rel_l2

TOL = 1e-5


def test_cache_bookkeeping_without_gpu():
    from qsim_gb300 import engine as E
    from qsim_gb300 import _native as N
    pc = E.PlanCache(capacity=4)
    assert pc.stats() == dict(hits=0, misses=0, evictions=0, captures=0,
                              size=0)
    pc.clear()
    # A run without a context or state is an argument error, not a crash.
    hit = C.c_int()
    o = N.FuseOptions(4, 0, 0, 5, None)
    rc = N.lib.qsg_plan_cache_run_text(None, pc.h, b"1\n0 h 0\n", 0, C.byref(o),
                                       None, 1, None, 0, None, C.byref(hit))
    assert rc == 1
    o = N.FuseOptions(9, 0, 0, 5, None)   # max_fused_size out of range
    rc = N.lib.qsg_plan_cache_run(None, pc.h, None, C.byref(o), None, 1, None,
                                  0, None, C.byref(hit))
    assert rc == 1


# ------------------------------------------------------------------ GPU --

@pytest.fixture(scope="module")
def eng():
    import qsim_gb300 as q
    from qsim_gb300 import engine as E
    ctx = q.Context(0)
    return q, E, ctx, q.StateSpace(ctx=ctx)


def gates_only(text):
    """The text circuit without its measurement lines (the reference's
    state in the fixture is the state before them)."""
    lines = text.splitlines()
    return "\n".join(lines[:1] + [l for l in lines[1:]
                                   if l.split()[1:2] != ["m"]]) + "\n"


def test_gates_only_text_keeps_the_reference_state(oracle):
    from qsim_gb300 import engine as E
    d = load_golden("text_gates9")
    c = E.Circuit.parse(gates_only(str(d["text"])))
    n = c.num_qubits
    s = oracle.zero_state(n)
    for o in c.ops():
        assert o["kind"] in (0, 1)
        if o["kind"] == 0:
            oracle.apply_gate(s, n, o["qs"], o["m"])
        else:
            oracle.apply_controlled_gate(s, n, o["qs"], o["cqs"], o["cvals"],
                                         o["m"])
    assert rel_l2(s, d["f64"]) < 1e-12


@pytest.mark.gpu
def test_text_circuit_hits_and_replays(eng):
    q, E, ctx, ss = eng
    d = load_golden("text_gates9")
    text, n = gates_only(str(d["text"])), int(d["n"])
    pc = E.PlanCache()
    st = ss.Create(n)
    outs = []
    for i in range(3):
        ss.SetStateZero(st)
        _, hit = pc.run(ctx, text, st)
        assert hit == (i > 0)
        outs.append(ss.to_numpy(st))
    assert pc.stats() == dict(hits=2, misses=1, evictions=0, captures=1,
                              size=1)
    assert rel_l2(outs[0], d["f64"]) < TOL
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    # The same plan run directly gives the same bits.
    ss.SetStateZero(st)
    E.Plan(E.Circuit.parse(text), max_fused_size=4).run(ctx, st)
    assert np.array_equal(ss.to_numpy(st), outs[0])


@pytest.mark.gpu
def test_key_covers_options_maxtime_and_content(eng):
    q, E, ctx, ss = eng
    d = load_golden("text_gates9")
    text, n = gates_only(str(d["text"])), int(d["n"])
    pc = E.PlanCache()
    st = ss.Create(n)
    runs = [dict(), dict(max_fused_size=3), dict(maxtime=4), dict()]
    hits = []
    for kw in runs:
        ss.SetStateZero(st)
        hits.append(pc.run(ctx, text, st, **kw)[1])
    assert hits == [False, False, False, True]
    # maxtime = 4 keeps the gates of times 0..4 only.
    ss.SetStateZero(st)
    pc.run(ctx, text, st, maxtime=4)
    want = E.Circuit.parse(text, maxtime=4)
    s2 = ss.Create(n)
    ss.SetStateZero(s2)
    E.Plan(want, max_fused_size=4).run(ctx, s2)
    assert np.array_equal(ss.to_numpy(st), ss.to_numpy(s2))
    # Circuit objects: equal content hits, one changed gate misses.
    a = E.Circuit.grid(3, 4, 0, 6, 7)
    b = E.Circuit.grid(3, 4, 0, 6, 7)
    c = E.Circuit.grid(3, 4, 0, 6, 8)
    s12 = ss.Create(12)
    got = []
    for circ in (a, b, c):
        ss.SetStateZero(s12)
        got.append(pc.run(ctx, circ, s12)[1])
    assert got == [False, True, False]


@pytest.mark.gpu
def test_measurements_in_cached_plans(eng):
    q, E, ctx, ss = eng
    text = ("6\n0 h 0\n0 h 1\n0 h 2\n0 h 3\n0 h 4\n0 h 5\n"
            "1 cz 0 1\n1 cz 2 3\n2 rx 4 0.7\n2 fs 1 2 0.5 0.25\n"
            "3 m 0 2 4\n4 h 0\n4 cnot 1 5\n5 m 1 5\n")
    pc = E.PlanCache()
    st, ref = ss.Create(6), ss.Create(6)
    plan = E.Plan(E.Circuit.parse(text), max_fused_size=4)
    for seed in (5, 6, 5):
        ss.SetStateZero(st)
        bits, _ = pc.run(ctx, text, st, seed=seed)
        ss.SetStateZero(ref)
        want = plan.run(ctx, ref, seed=seed)
        assert np.array_equal(bits, want)
        assert np.array_equal(ss.to_numpy(st), ss.to_numpy(ref))
    s = pc.stats()
    assert (s["hits"], s["misses"], s["captures"]) == (2, 1, 0)


@pytest.mark.gpu
def test_lru_eviction_and_recapture(eng, oracle):
    q, E, ctx, ss = eng
    pc = E.PlanCache(capacity=2)
    circs = [E.Circuit.chain(8, 4, s) for s in (1, 2, 3)]
    st = ss.Create(8)
    for c in circs + circs[:1]:
        ss.SetStateZero(st)
        pc.run(ctx, c, st)
    s = pc.stats()
    assert (s["misses"], s["hits"], s["evictions"], s["size"]) == (4, 0, 2, 2)
    # circs[0] is cached again: a second state recaptures its graph.
    s2 = ss.Create(8)
    ss.SetStateZero(s2)
    _, hit = pc.run(ctx, circs[0], s2)
    assert hit and pc.stats()["captures"] == 5
    want = oracle.zero_state(8)
    for o in circs[0].ops():
        if o["kind"] == 0:
            oracle.apply_gate(want, 8, o["qs"], o["m"])
        else:
            oracle.apply_controlled_gate(want, 8, o["qs"], o["cqs"],
                                         o["cvals"], o["m"])
    assert rel_l2(ss.to_numpy(s2), want) < TOL
    ctx.sync()
