"""The C++ drop-in: header-only StateSpace / Simulator / Factory adapters in
include/qsim_gb300/ that the reference's QSimRunner, MultiQubitGateFuser,
ExpectationValue and QuantumTrajectorySimulator templates accept unchanged.

CPU: both test programs compile and link against libqsim_gb300.so (the
reference-runner program only where a qsim checkout is present: it includes
the reference's own headers).  GPU: the adapter program runs a golden gate
list through the adapters and matches the reference's outputs."""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_l2, unpack_ops

LIBDIR = os.path.join(ROOT, "qsim_gb300", "_build")
REF = os.environ.get("QSG_REFERENCE",
                     os.path.join(os.path.dirname(ROOT), "reference"))


def compile_prog(src, out, extra=()):
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
           *extra, os.path.join(ROOT, "tests", "cpp", src), "-o", out,
           "-L" + LIBDIR, "-lqsim_gb300", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_adapter_program_compiles(tmp_path):
    compile_prog("adapter_run.cc", str(tmp_path / "adapter_run"))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "lib")),
                    reason="qsim checkout (reference headers) not present")
def test_reference_runner_compiles_with_gb300_factory(tmp_path):
    """QSimRunner<IO, MultiQubitGateFuser<IO>, FactoryGB300>,
    ExpectationValue<IO, MultiQubitGateFuser<IO>> (both variants) and
    QuantumTrajectorySimulator<IO, Runner> instantiate with the adapters."""
    compile_prog("dropin_qsim_runner.cc", str(tmp_path / "dropin"),
                 extra=("-I" + os.path.join(REF, "lib"),))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "lib")),
                    reason="qsim checkout (reference headers) not present")
def test_reference_apply_gate_compiles_with_gb300_unitary(tmp_path):
    """lib/gate_appl.h's ApplyGate(calculator, gate, unitary) and the
    text-format parser instantiate with UnitaryCalculatorGB300."""
    compile_prog("dropin_unitary.cc", str(tmp_path / "dropin_unitary"),
                 extra=("-I" + os.path.join(REF, "lib"),))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "lib")),
                    reason="qsim checkout (reference headers) not present")
def test_reference_circuits_compile_with_gb300_hybrid_runner(tmp_path):
    """qsim's Circuit<Operation<float>> and text parser drive
    QSimHRunnerGB300 with the Parameter fields of apps/qsimh_base.cc."""
    exe = str(tmp_path / "dropin_hybrid")
    compile_prog("dropin_hybrid.cc", exe, extra=("-I" + os.path.join(REF, "lib"),))
    # The adapter's circuit conversion (no GPU) against the reference's own
    # SplitLattice counts and gate matrices, on every hybrid fixture.
    cases = [(load_golden(c), None) for c in ("hybrid6", "hybrid8", "hybrid10")]
    kd = load_golden("hybrid_known")
    cases += [(None, (str(kd[f"text{i}"]), kd[f"parts{i}"].tolist()))
              for i in (0, 4)]
    for d, known in cases:
        text, parts = (str(d["text"]), d["parts"].tolist()) if d is not None else known
        cp = tmp_path / "c.txt"
        cp.write_text(text)
        r = subprocess.run([exe, "--check", str(cp), "".join(str(p) for p in parts)],
                           capture_output=True, text=True)
        assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout)


@pytest.mark.gpu
def test_adapter_program_matches_reference(tmp_path, oracle):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import write_gate_list
    d = load_golden("rand14_k2")
    n = int(d["n"])
    ops = unpack_ops(d)
    gl_ops = [dict(kind={0: "g", 1: "c"}[o["kind"]], time=i, qs=o["qs"],
                   cqs=o["cqs"], cvals=o["cvals"], m=o["m"])
              for i, o in enumerate(ops)]
    gl = tmp_path / "gates.txt"
    write_gate_list(str(gl), n, gl_ops)
    exe = str(tmp_path / "adapter_run")
    compile_prog("adapter_run.cc", exe)
    out = str(tmp_path / "out")
    qs = [int(q) for q in d["meas_qs"]]
    r = subprocess.run([exe, str(gl), out, str(int(d["meas_seed"]))] +
                       [str(q) for q in qs], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    state = np.fromfile(out + ".state", np.float32).view(np.complex64)
    assert rel_l2(state.astype(np.complex128), d["f64"]) < 1e-5
    # First Measure(qubits, mt19937(seed)) on the final state is the first
    # of the reference's measurement sequence.
    bits = np.fromfile(out + ".bits", np.uint64)[0]
    assert int(bits) == int(d["meas_bits"][0])
    samples = np.fromfile(out + ".samples", np.uint64)
    want = oracle.sample(state.astype(np.complex128), n, 1000, 7)
    assert np.mean(samples == want) >= 0.999
    # InternalToNormalOrder / NormalToInternalOrder: the internal order is
    # the normal order (lib/statespace_cuda.h:85-107 transposes the
    # reference's 32/32 blocks), so both leave the amplitudes in place.
    for ext in (".normal", ".internal"):
        assert np.array_equal(np.fromfile(out + ext, np.float32).view(np.complex64),
                              state)
    # Sample<float>: draws of uniform_real_distribution<float>(0, norm).
    import ctypes as C
    s128 = state.astype(np.complex128)
    rs = np.zeros(1000, np.float32)
    oracle.L.orc_generate_random_values_f32.argtypes = [
        C.c_uint64, C.c_uint32, C.c_float, C.POINTER(C.c_float)]
    oracle.L.orc_generate_random_values_f32(
        1000, 7, np.float32(np.vdot(s128, s128).real),
        rs.ctypes.data_as(C.POINTER(C.c_float)))
    r64 = rs.astype(np.float64)
    want32 = np.zeros(1000, np.uint64)
    oracle.L.orc_sample_thresholds_f64.argtypes = [
        C.POINTER(C.c_double), C.c_uint, C.c_uint64, C.POINTER(C.c_double),
        C.POINTER(C.c_uint64)]
    oracle.L.orc_sample_thresholds_f64(
        s128.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)), n, 1000,
        r64.ctypes.data_as(C.POINTER(C.c_double)),
        want32.ctypes.data_as(C.POINTER(C.c_uint64)))
    samples32 = np.fromfile(out + ".samples_f32", np.uint64)
    assert np.mean(samples32 == want32) >= 0.999
    assert not np.array_equal(samples32, samples)   # float draws differ
