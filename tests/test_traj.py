"""Noisy circuits and quantum trajectories.

CPU: the trajectory oracle (oracle/traj_oracle.py) is pinned against the
reference's own QuantumTrajectorySimulator outputs (tests/golden/traj_*.npz,
made by tests/golden/make_golden.py), and the engine's noisy-circuit builder
and runner set-up are checked.  GPU: the engine's trajectories reproduce the
reference's Kraus-operator choices (exactly where the lower probability
bounds decide; statistically where the state decides) and final states
(relative L2 <= 1e-5 against the reference's FP64 run)."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_l2, unpack_ops

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import traj_oracle  # noqa: E402

from qsim_gb300 import engine as E  # noqa: E402

CASES = ["traj_depol8", "traj_ad8", "traj_mixed6", "traj_chain12",
         "traj_depol2q_reg"]
# Fraction of repetitions whose choices must agree: all of them when every
# channel is unitary, nearly all when a choice can depend on round-off.
MIN_AGREE = {"traj_depol8": 1.0, "traj_ad8": 0.95, "traj_mixed6": 0.95,
             "traj_chain12": 1.0, "traj_depol2q_reg": 1.0}
STATE_TOL = 1e-5


def ref_samples(d, suffix):
    counts = d["stat_count" + suffix]
    flat = d["stat" + suffix]
    offs = np.concatenate([[0], np.cumsum(counts)])
    return [flat[offs[i]:offs[i + 1]] for i in range(len(counts))]


def build_noisy(d):
    n = int(d["n"])
    nc = E.NoisyCircuit(n)
    gates = iter(unpack_ops(d))
    qmask = d["op_qmask"] if "op_qmask" in d else np.zeros(len(d["op_q"]))
    for code, t, q, p, qm in zip(d["op_channel"], d["op_time"], d["op_q"],
                                 d["op_p"], qmask):
        qs = [b for b in range(64) if (int(qm) >> b) & 1] or [int(q)]
        if code < 0:
            o = next(gates)
            if o["kind"] == 0:
                nc.add_gate(int(t), o["qs"], o["m"])
            elif o["kind"] == 1:
                nc.add_controlled_gate(int(t), o["qs"], o["cqs"], o["cvals"], o["m"])
            else:
                nc.add_measurement(int(t), o["qs"])
        else:
            nc.add_channel(int(code), int(t), qs, float(p))
    return nc


# ------------------------------------------------------------------ CPU --

@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case, oracle):
    d = load_golden(case)
    n = int(d["n"])
    ops = traj_oracle.ops_from_fixture(d, unpack_ops)
    ref64 = ref_samples(d, "64")
    agree = 0
    for i, rep in enumerate(range(int(d["r0"]), int(d["r1"]))):
        s, stats = traj_oracle.run_trajectory(oracle, n, ops, rep, fp32=False)
        if list(stats) == [int(x) for x in ref64[i]]:
            agree += 1
            want = d["f64"][i].astype(np.complex128)
            assert rel_l2(s, want) < (1e-6 if d["f64"].dtype == np.complex64
                                      else 1e-10), (case, rep)
    assert agree >= MIN_AGREE[case] * len(ref64), (case, agree, len(ref64))


def test_reference_choices_depend_on_noise():
    """The fixtures exercise what they are meant to: Pauli errors, device-side
    (state-dependent) choices and measurements."""
    d = load_golden("traj_ad8")
    samples = np.concatenate(ref_samples(d, "32"))
    assert (samples == 1).sum() > 10       # K1 of amplitude damping / X
    d = load_golden("traj_depol8")
    samples = np.concatenate(ref_samples(d, "32"))
    assert set(np.unique(samples).tolist()) >= {0, 1, 2, 3}


def test_make_noisy_matches_op_rule():
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import noisy_chain_ops
    want = noisy_chain_ops(7, 3, 9, 1e-3, 5e-3)
    nc = E.NoisyCircuit.make(E.Circuit.chain(7, 3, 9), 1e-3, 5e-3, 2)
    assert len(nc) == len(want)
    for i, w in enumerate(want):
        o = nc.op(i)
        assert o["time"] == w["time"]
        assert o["qs"] == list(w["qs"])
        assert o["is_channel"] == (w["kind"] in "DAPBFR")
        if w["kind"] == "D":
            assert o["num_kops"] == 4
        elif w["kind"] == "A":
            assert o["num_kops"] == 2
    # Without damping the times are MakeNoisy's 2t / 2t+1.
    nc = E.NoisyCircuit.make(E.Circuit.chain(5, 2, 1), 0.01, 0.0, 2)
    c = E.Circuit.chain(5, 2, 1)
    assert nc.op(0)["time"] == 2 * c.op(0)["time"]
    assert nc.op(1)["time"] == 2 * c.op(0)["time"] + 1


def test_runner_fuses_channels_as_slots():
    nc = E.NoisyCircuit.make(E.Circuit.chain(10, 6, 2), 1e-3, 5e-3, 2)
    t = E.Trajectories(nc, max_fused_size=4)
    info = t.info()
    assert info["num_ops"] == len(nc)
    # Channels ride in the blocks of their gates: no more blocks than the
    # clean circuit fused alone would need, plus a few.
    clean = E.Plan(E.Circuit.chain(10, 6, 2), max_fused_size=4)
    assert info["num_fused_ops"] <= len(clean) + 4


def test_runner_rejects_unsupported_channels():
    nc = E.NoisyCircuit(3)
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    # Non-unitary Kraus operator whose K^dagger K is not diagonal.
    k0 = np.array([[0.9, 0.1], [0.0, 0.8]])
    k1 = np.array([[0.3, 0.0], [0.2, 0.4]])
    nc.add_kraus_channel(0, [1], [(False, 0.5, k0), (False, 0.0, k1)])
    with pytest.raises(E.N.QsgError) as e:
        E.Trajectories(nc)
    assert e.value.status == 4  # QSG_ERR_UNSUPPORTED
    # A unitary channel with a general matrix is fine.
    nc = E.NoisyCircuit(3)
    nc.add_kraus_channel(0, [0, 2], [(True, 0.7, np.eye(4)),
                                     (True, 0.3, np.kron(h, h))])
    E.Trajectories(nc)


def test_noisy_argument_errors():
    nc = E.NoisyCircuit(4)
    with pytest.raises(E.N.QsgError):
        nc.add_channel(E.CHANNEL_AMPLITUDE_DAMPING, 0, [4], 0.1)
    with pytest.raises(E.N.QsgError):
        nc.add_channel(E.CHANNEL_BIT_FLIP, 0, [0], 1.5)
    with pytest.raises(E.N.QsgError):
        nc.add_channel(E.CHANNEL_PHASE_FLIP, 0, [0, 1], 0.1)
    with pytest.raises(E.N.QsgError):
        nc.add_channel(99, 0, [0], 0.1)


# ------------------------------------------------------------------ GPU --

@pytest.fixture(scope="module")
def ctx():
    from qsim_gb300 import api
    return api.Context()


@pytest.fixture(scope="module")
def ss(ctx):
    from qsim_gb300 import api
    return api.StateSpace(ctx=ctx)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_trajectories_match_reference(case, ctx, ss):
    d = load_golden(case)
    n = int(d["n"])
    t = E.Trajectories(build_noisy(d), max_fused_size=int(d["fsize"]))
    ref32 = ref_samples(d, "32")
    ref64 = ref_samples(d, "64")
    st = ss.Create(n)
    agree = 0
    for i, rep in enumerate(range(int(d["r0"]), int(d["r1"]))):
        stats = t.run(ctx, st, rep)
        got = [int(x) for x in E.Trajectories.samples(stats)]
        if got == [int(x) for x in ref32[i]]:
            agree += 1
        if got == [int(x) for x in ref64[i]]:
            s = ss.to_numpy(st)
            want = d["f64"][i].astype(np.complex128)
            assert rel_l2(s, want) < STATE_TOL, (case, rep, rel_l2(s, want))
    assert agree >= MIN_AGREE[case] * len(ref32), (case, agree, len(ref32))


@pytest.mark.gpu
def test_gpu_batch_matches_single_runs(ctx, ss):
    runners, circuits = [], []
    for n, seed in ((9, 1), (12, 2), (7, 3)):
        nc = E.NoisyCircuit.make(E.Circuit.chain(n, 6, seed), 0.02, 0.05, 2)
        circuits.append(n)
        runners.append(E.Trajectories(nc, max_fused_size=3))
    items = [(i % 3, 100 + i) for i in range(12)]
    outs = [ss.Create(circuits[r]) for r, _ in items]
    per, lat, wall = E.run_trajectory_batch(runners, items, num_streams=4,
                                            out_states=outs)
    assert wall > 0 and np.all(lat > 0)
    for (r, rep), stats, out in zip(items, per, outs):
        st = ss.Create(circuits[r])
        single = runners[r].run(ctx, st, rep)
        assert np.array_equal(single, stats)
        np.testing.assert_array_equal(ss.to_numpy(st), ss.to_numpy(out))


@pytest.mark.gpu
def test_gpu_batched_workload_noise_vs_oracle(ctx, ss, oracle):
    """The batched-trajectory workload's noise model (depolarizing 1e-3 after
    each gate qubit, amplitude damping 5e-3 per qubit per cycle) at n = 14,
    depth 12, against the FP64 oracle."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import noisy_chain_ops
    n = 14
    nc = E.NoisyCircuit.make(E.Circuit.chain(n, 12, 11), 1e-3, 5e-3, 2)
    t = E.Trajectories(nc, max_fused_size=4)
    ops = []
    for o in noisy_chain_ops(n, 12, 11, 1e-3, 5e-3):
        if o["kind"] in "DA":
            ops.append(dict(channel="DA".index(o["kind"]), q=o["qs"][0], p=o["p"]))
        else:
            ops.append(dict(kind=0, qs=o["qs"], m=o["m"]))
    st = ss.Create(n)
    agree = 0
    for rep in range(6):
        stats = t.run(ctx, st, rep)
        s_ref, stats_ref = traj_oracle.run_trajectory(oracle, n, ops, rep)
        if [int(x) for x in E.Trajectories.samples(stats)] == list(stats_ref):
            agree += 1
            assert rel_l2(ss.to_numpy(st), s_ref) < STATE_TOL
    assert agree >= 5


@pytest.mark.parametrize("case", ["traj_depol8", "traj_ad8", "traj_chain12"])
def test_cpu_port_matches_reference(case, oracle):
    """The timed FP32 CPU port of RunIteration (oracle/traj_port.py, the
    trajectories' CPU baseline) makes the reference's Kraus choices and
    reaches its final states."""
    import traj_port
    d = load_golden(case)
    n = int(d["n"])
    ops = traj_oracle.ops_from_fixture(d, unpack_ops)
    is_chan = np.array(["channel" in op for op in ops])
    ref32 = ref_samples(d, "32")
    port = traj_port.TrajectoryPort(oracle.L, n)
    agree = 0
    for i, rep in enumerate(range(int(d["r0"]), int(d["r1"]))):
        choices = port.run(ops, rep)
        want = [int(x) for x, c in zip(ref32[i], is_chan) if c]
        if choices == want:
            agree += 1
            got = port.state().astype(np.complex128)
            assert rel_l2(got, d["f64"][i].astype(np.complex128)) < 1e-5
    assert agree >= MIN_AGREE[case] * len(ref32), (case, agree, len(ref32))


def test_cpu_port_noisy_ops_follow_make_noisy():
    """traj_port.noisy_ops inserts channels by the engine's MakeNoisy rule:
    the same channel count as the engine's noisy circuit."""
    import traj_port
    c = E.Circuit.chain(9, 6, 3)
    nc = E.NoisyCircuit.make(c, 1e-3, 5e-3, 2)
    ops = traj_port.noisy_ops(c.ops(), 9, 1e-3, 5e-3, 2)
    assert sum("channel" in o for o in ops) == nc.info()["num_channels"]
    assert sum("channel" not in o for o in ops) == len(c.ops())
