"""Hybrid Schrodinger-Feynman simulation (qsimh) on the GPU, mirroring the
reference's QSimHRunner (lib/run_qsimh.h) and HybridSimulator
(lib/hybrid.h): amplitudes of chosen bitstrings of a circuit whose qubits
are cut into two parts, summed over the paths of the gates on the cut.

    from qsim_gb300 import engine as E, hybrid
    c = E.Circuit.parse(text)
    amps, info = hybrid.run(ctx, c, parts, bitstrings, num_prefix_gatexs=2,
                            num_root_gatexs=1, prefix=1)
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from ._native import check


def _info(i: N.HybridInfo) -> dict:
    return {f: getattr(i, f) for f, _ in N.HybridInfo._fields_}


def split_lattice(circuit, parts: Sequence[int]) -> dict:
    """HybridSimulator::SplitLattice counts: qubits and operations per part
    (cut gates counted in both) and gates on the cut."""
    p = N.u32_array(parts)
    info = N.HybridInfo()
    check(N.lib.qsg_hybrid_split(circuit.h, p, len(parts), C.byref(info)))
    return _info(info)


def run(ctx, circuit, parts: Sequence[int], bitstrings, prefix: int = 0,
        num_prefix_gatexs: int = 0, num_root_gatexs: int = 0,
        max_fused_size: int = 4, tensor_path: bool = False,
        max_batch_bits: int = 0, results: Optional[np.ndarray] = None):
    """QSimHRunner::Run: returns (amplitudes, info).  The amplitudes are
    added to `results` when given (complex128, one per bitstring), as the
    reference adds to its results vector."""
    bits = np.ascontiguousarray(np.asarray(bitstrings, dtype=np.uint64))
    m = len(bits)
    if results is None:
        results = np.zeros(m, dtype=np.complex128)
    if results.dtype != np.complex128 or len(results) != m:
        raise ValueError("results must be complex128, one per bitstring")
    o = N.HybridOptions(prefix, num_prefix_gatexs, num_root_gatexs,
                        max_fused_size, int(tensor_path), max_batch_bits)
    info = N.HybridInfo()
    check(N.lib.qsg_hybrid_run(
        ctx.h, circuit.h, N.u32_array(parts), len(parts), C.byref(o),
        bits.ctypes.data_as(N.P_u64), m,
        results.view(np.float64).ctypes.data_as(N.P_f64), C.byref(info)))
    return results, _info(info)
