"""Packed trajectory batches (one persistent kernel over the batch) against
the reference's own QuantumTrajectorySimulator outputs, the FP64
trajectory oracle and the stream path.

Tolerances as the other trajectory tests: Kraus choices identical where the
lower probability bounds decide (unitary channels) and in >= 95 % of the
repetitions where the state decides (a probability within round-off of a
threshold may flip); final states within relative L2 1e-5 of FP64 whenever
the choices agree."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_l2

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import traj_oracle  # noqa: E402

from qsim_gb300 import engine as E  # noqa: E402
from test_traj import CASES, MIN_AGREE, STATE_TOL, build_noisy, ref_samples  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ss():
    from qsim_gb300 import api
    return api.StateSpace(ctx=api.Context())


@pytest.mark.parametrize("case", CASES)
def test_packed_matches_reference(case, ss):
    d = load_golden(case)
    n = int(d["n"])
    t = E.Trajectories(build_noisy(d), max_fused_size=int(d["fsize"]))
    reps = list(range(int(d["r0"]), int(d["r1"])))
    outs = [ss.Create(n) for _ in reps]
    per, lat, wall, launches, info = E.run_trajectory_batch_packed(
        [t], [(0, r) for r in reps], out_states=outs)
    assert info["packed_items"] + info["stream_items"] == len(reps)
    ref32, ref64 = ref_samples(d, "32"), ref_samples(d, "64")
    agree = 0
    for i, stats in enumerate(per):
        got = [int(x) for x in E.Trajectories.samples(stats)]
        agree += got == [int(x) for x in ref32[i]]
        if got == [int(x) for x in ref64[i]]:
            s = ss.to_numpy(outs[i])
            want = d["f64"][i].astype(np.complex128)
            assert rel_l2(s, want) < STATE_TOL, (case, i, rel_l2(s, want))
    assert agree >= MIN_AGREE[case] * len(reps), (case, agree, len(reps))


def _mixed_runners(noise=(0.02, 0.05)):
    runners, sizes = [], []
    for n, seed in ((9, 1), (12, 2), (7, 3), (14, 4), (5, 5)):
        nc = E.NoisyCircuit.make(E.Circuit.chain(n, 6, seed), noise[0], noise[1], 2)
        runners.append(E.Trajectories(nc, max_fused_size=3 if n % 2 else 4))
        sizes.append(n)
    return runners, sizes


def test_packed_matches_stream_batch(ss):
    """Strong noise (many device-side choices): the packed kernel and the
    stream path make the same choices and reach the same states."""
    runners, sizes = _mixed_runners()
    items = [(i % len(runners), 200 + i) for i in range(40)]
    outs_p = [ss.Create(sizes[r]) for r, _ in items]
    outs_s = [ss.Create(sizes[r]) for r, _ in items]
    per_p, lat_p, _, launches, info = E.run_trajectory_batch_packed(
        runners, items, out_states=outs_p)
    assert info["packed_items"] == len(items) and launches == 1
    assert np.all(lat_p > 0)
    per_s, _, _ = E.run_trajectory_batch(runners, items, num_streams=4,
                                         out_states=outs_s)
    same = 0
    for (r, _), sp, st, op, os_ in zip(items, per_p, per_s, outs_p, outs_s):
        if np.array_equal(sp, st):
            same += 1
            assert rel_l2(ss.to_numpy(op), ss.to_numpy(os_)) < STATE_TOL
    assert same >= 0.95 * len(items)
    escapes = sum(int(np.sum(E.Trajectories.samples(s) != 0)) for s in per_p)
    assert escapes > 0  # the workload does exercise non-default choices


def test_packed_slots_give_same_choices(ss):
    """Without out_states every CTA runs in its own slot buffer; the choices
    are those of the run into per-item buffers."""
    runners, sizes = _mixed_runners()
    items = [(i % len(runners), 300 + i) for i in range(25)]
    outs = [ss.Create(sizes[r]) for r, _ in items]
    per_a, _, _, _, _ = E.run_trajectory_batch_packed(runners, items, out_states=outs)
    for per_sm in (1, 2):
        per_b, _, _, _, info = E.run_trajectory_batch_packed(
            runners, items, ctas_per_sm=per_sm)
        assert info["ctas"] >= 1
        for a, b in zip(per_a, per_b):
            assert np.array_equal(a, b)


def test_packed_routes_unpackable_items_to_streams(ss):
    """Circuits with measurements or above max_qubits run on the stream path
    inside the same call; results equal single runs."""
    from qsim_gb300 import api
    ctx = api.Context()
    c = E.Circuit.chain(8, 4, 7)
    c.add_measurement(100, [0, 3])
    nc_meas = E.NoisyCircuit.make(c, 0.02, 0.0, 2)
    nc_big = E.NoisyCircuit.make(E.Circuit.chain(13, 4, 8), 0.02, 0.05, 2)
    nc_small = E.NoisyCircuit.make(E.Circuit.chain(6, 4, 9), 0.02, 0.05, 2)
    runners = [E.Trajectories(x, max_fused_size=3) for x in (nc_meas, nc_big, nc_small)]
    sizes = [8, 13, 6]
    items = [(i % 3, 10 + i) for i in range(9)]
    outs = [ss.Create(sizes[r]) for r, _ in items]
    per, _, _, launches, info = E.run_trajectory_batch_packed(
        runners, items, max_qubits=12, out_states=outs)
    assert info["packed_items"] == 3 and info["stream_items"] == 6
    assert launches > 1
    for (r, rep), stats, out in zip(items, per, outs):
        st = ss.Create(sizes[r])
        single = runners[r].run(ctx, st, rep)
        assert np.array_equal(single, stats)
        assert rel_l2(ss.to_numpy(out), ss.to_numpy(st)) < STATE_TOL


def test_packed_workload_noise_vs_oracle(ss, oracle):
    """The batched-trajectory workload's noise model (depolarizing 1e-3 after
    each gate qubit, amplitude damping 5e-3 per qubit per cycle) at n = 14,
    depth 12, in the packed kernel against the FP64 oracle."""
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
    reps = list(range(8))
    outs = [ss.Create(n) for _ in reps]
    per, _, _, _, _ = E.run_trajectory_batch_packed(
        [t], [(0, r) for r in reps], out_states=outs)
    agree = 0
    for rep, stats, out in zip(reps, per, outs):
        s_ref, stats_ref = traj_oracle.run_trajectory(oracle, n, ops, rep)
        if [int(x) for x in E.Trajectories.samples(stats)] == list(stats_ref):
            agree += 1
            assert rel_l2(ss.to_numpy(out), s_ref) < STATE_TOL
    assert agree >= 7


def test_autotuned_configurations_agree(ss):
    """Every configuration the autotuner may pick (stream path, persistent
    kernel, split with both running at once) makes the same choices and
    reaches the same states; the tuner returns one of them."""
    from qsim_gb300 import autotune as AT
    sizes = [6, 9, 12, 15, 17]
    made = {}

    def make(f, tensor):
        if (f, tensor) not in made:
            made[(f, tensor)] = [
                E.Trajectories(E.NoisyCircuit.make(E.Circuit.chain(n, 6, 40 + n),
                                                   0.01, 0.03, 2),
                               max_fused_size=f, tensor_path=tensor)
                for n in sizes]
        return made[(f, tensor)]
    items = [(i % len(sizes), 500 + i) for i in range(30)]
    ref = None
    extra = [dict(max_fused_size=4, tensor=False, tc_from=12, split=9,
                  ctas_per_sm=1, tile_kib=32),
             dict(max_fused_size=3, tensor=False, tc_from=15, split=0,
                  ctas_per_sm=0, tile_kib=0)]
    for cfg in AT.candidates(max(sizes), forms=((4, False), (6, True))) + extra:
        runners = AT.runners_for(make, sizes, cfg)
        outs = [ss.Create(sizes[r]) for r, _ in items]
        per, lat, wall, launches, info = AT.run(runners, items, cfg, 4, outs)
        states = [ss.to_numpy(o) for o in outs]
        if ref is None:
            ref = (per, states)
            continue
        same = 0
        for a, b, sa, sb in zip(per, ref[0], states, ref[1]):
            if np.array_equal(a, b):
                same += 1
                assert rel_l2(sa, sb) < STATE_TOL, cfg
        assert same >= 0.95 * len(items), cfg
    tune = AT.tune_trajectories(make, sizes, 4, num_streams=4,
                                use_cache=False)
    assert tune["best"] in [c for c, _ in tune["table"]]
    assert all(v > 0 for _, v in tune["table"])


@pytest.mark.parametrize("case", [c for c in CASES if int(load_golden(c)["n"]) >= 12])
def test_tensor_core_trajectories_match_reference(case, ss):
    """Trajectories whose fused blocks run on the tensor cores (blocks of
    >= 2 qubits, padded to six targets) make the reference's choices and
    reach its FP64 states within relative L2 1e-5."""
    from qsim_gb300 import api
    ctx = api.Context()
    d = load_golden(case)
    n = int(d["n"])
    t = E.Trajectories(build_noisy(d), max_fused_size=6, tensor_path=True,
                       tc_min_k=2)
    ref32, ref64 = ref_samples(d, "32"), ref_samples(d, "64")
    st = ss.Create(n)
    agree = 0
    for i, rep in enumerate(range(int(d["r0"]), int(d["r1"]))):
        stats = t.run(ctx, st, rep)
        got = [int(x) for x in E.Trajectories.samples(stats)]
        agree += got == [int(x) for x in ref32[i]]
        if got == [int(x) for x in ref64[i]]:
            s = ss.to_numpy(st)
            want = d["f64"][i].astype(np.complex128)
            assert rel_l2(s, want) < STATE_TOL, (case, rep, rel_l2(s, want))
    assert agree >= MIN_AGREE[case] * len(ref32), (case, agree, len(ref32))
