"""Pins the oracle (oracle/qsim_oracle.c) to golden outputs of the reference
itself (tests/golden/*.npz, produced by tests/golden/make_golden.py through
oracle/ref_driver.cc).  CPU only."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, pauli_matrix, rel_l2, unpack_ops


def test_mt19937_and_canonical(oracle):
    """std::mt19937 outputs and uniform_real_distribution<double>(0,1) draws
    are bit-identical to libstdc++ (reference lib/util.h:61-85)."""
    d = load_golden("mt19937")
    for seed in (0, 1, 5489, 123456789, 4294967295):
        g = oracle.mt(seed)
        raw = [oracle.L.orc_mt_next(g) for _ in range(2000)]
        assert np.array_equal(np.array(raw, np.uint32), d[f"raw_{seed}"])
        g = oracle.mt(seed)
        u = np.array([oracle.L.orc_canonical(g) for _ in range(2000)])
        assert np.array_equal(u, d[f"u01_{seed}"])


def test_float_uniforms_match_libstdcxx(oracle):
    """GenerateRandomValues<float> (lib/util.h:67-85), the draws of
    Sample<float>: uniform_real_distribution<float>(0, 0.73) from
    mt19937(seed), sorted, bit-identical to the reference's build."""
    import ctypes as C
    d = load_golden("mt19937")
    f = oracle.L.orc_generate_random_values_f32
    f.argtypes = [C.c_uint64, C.c_uint32, C.c_float, C.POINTER(C.c_float)]
    for seed in (0, 1, 5489, 123456789, 4294967295):
        out = np.zeros(2000, np.float32)
        f(2000, seed, np.float32(0.73), out.ctypes.data_as(C.POINTER(C.c_float)))
        assert np.array_equal(out, np.sort(d[f"f073_{seed}"]))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_state_matches_reference_fp64(oracle, case):
    """Unfused FP64 application equals SimulatorBasic<For,double>."""
    d = load_golden(case)
    n = int(d["n"])
    s = oracle.run_ops(n, unpack_ops(d))
    assert rel_l2(s, d["f64"]) < 1e-12


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_reference_fp32_fused_within_tolerance(case):
    """The reference's own FP32 fused path is within the parity bar
    (relative L2 <= 1e-5) of its FP64 oracle: the bar is attainable."""
    d = load_golden(case)
    assert rel_l2(d["f32"].astype(np.complex128), d["f64"]) < 1e-5


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_samples_match_reference(oracle, case):
    d = load_golden(case)
    if "s64" not in d:
        pytest.skip("no samples in this case")
    n = int(d["n"])
    s = d["f64"].copy()
    got = oracle.sample(s, n, d["s64"].size, int(d["sample_seed"]))
    assert np.array_equal(got, d["s64"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_expectation_values(oracle, case):
    d = load_golden(case)
    if "ev64" not in d:
        pytest.skip("no expectation values in this case")
    n = int(d["n"])
    s = d["f64"].copy()
    for i, ops in enumerate(d["ev_ops"]):
        qs = d["ev_qpool"][d["ev_qoff"][i]:d["ev_qoff"][i + 1]].tolist()
        ev = oracle.expectation_value(s, n, qs, pauli_matrix(str(ops)))
        assert abs(ev - d["ev64"][i]) < 1e-12


def test_oracle_measurement_sequence(oracle):
    """Repeated Measure with one mt19937 (lib/statespace.h:84-140) gives the
    reference's bits and collapsed state."""
    d = load_golden("rand14_k2")
    n = int(d["n"])
    s = d["f64"].copy()
    mask = 0
    for q in d["meas_qs"]:
        mask |= 1 << int(q)
    g = oracle.mt(int(d["meas_seed"]))
    for want in d["meas_bits"]:
        norm = oracle.norm(s, n)
        r = oracle.L.orc_uniform(g, norm)
        bits = oracle.find_index(s, n, r) & mask
        assert bits == int(want)
        oracle.collapse(s, n, mask, bits)
    assert rel_l2(s, d["meas_state"]) < 1e-12
