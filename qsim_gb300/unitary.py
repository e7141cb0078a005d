"""Unitary calculator on the GPU, mirroring the reference's
UnitarySpaceBasic (lib/unitaryspace_basic.h) and UnitaryCalculatorBasic
(lib/unitary_calculator_basic.h) member for member.

Entry (i, j) of an n-qubit unitary sits at complex index i * 2^n + j, as in
the reference; gates mix the entries of every row over the column bits at
their qubits, so from the identity entry (i, j) after gates G1..Gm is
(Gm ... G1)[j][i].  The engine runs the unitary as a 2n-qubit state on the
same GB300 kernels as state vectors.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .api import Context, default_context
from ._native import check


class Unitary:
    """Device unitary (UnitarySpace::Unitary, lib/unitaryspace.h:38)."""

    def __init__(self, ptr: Optional[int], num_qubits: int, owned: bool,
                 ctx: Context):
        self._ptr, self._n, self._owned, self._ctx = ptr, num_qubits, owned, ctx

    def get(self) -> Optional[int]:
        return self._ptr

    def num_qubits(self) -> int:
        return self._n

    def free(self) -> None:
        if self._owned and self._ptr:
            check(N.lib.qsg_unitary_free(self._ctx.h, self._ptr))
        self._ptr, self._owned = None, False

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _f32(matrix):
    m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float32).ravel())
    return m, m.ctypes.data_as(N.P_f32)


def _u32(xs):
    a = (C.c_uint * max(1, len(xs)))(*[int(x) for x in xs])
    return a


class UnitarySpace:
    """UnitarySpaceBasic equivalent (lib/unitaryspace_basic.h:34-100)."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()

    @staticmethod
    def Size(num_qubits: int) -> int:
        return 1 << num_qubits

    @staticmethod
    def MinRowSize(num_qubits: int) -> int:
        return 2 * (1 << num_qubits)

    @staticmethod
    def MinSize(num_qubits: int) -> int:
        return int(N.lib.qsg_unitary_min_size(num_qubits))

    def CreateUnitary(self, num_qubits: int) -> Unitary:
        p = C.c_void_p()
        rc = N.lib.qsg_unitary_create(self.ctx.h, num_qubits, C.byref(p))
        if rc == 2:  # out of memory: the reference returns NullUnitary()
            return self.NullUnitary()
        check(rc)
        return Unitary(p.value, num_qubits, True, self.ctx)

    def NullUnitary(self) -> Unitary:
        return Unitary(None, 0, False, self.ctx)

    def SetAllZeros(self, u: Unitary) -> None:
        check(N.lib.qsg_unitary_set_all_zeros(self.ctx.h, u.get(), u.num_qubits()))

    def SetIdentity(self, u: Unitary) -> None:
        check(N.lib.qsg_unitary_set_identity(self.ctx.h, u.get(), u.num_qubits()))

    def GetEntry(self, u: Unitary, i: int, j: int) -> complex:
        out = (C.c_float * 2)()
        check(N.lib.qsg_unitary_get_entry(self.ctx.h, u.get(), u.num_qubits(),
                                          i, j, out))
        return complex(out[0], out[1])

    def SetEntry(self, u: Unitary, i: int, j: int, value: complex) -> None:
        value = complex(value)
        check(N.lib.qsg_unitary_set_entry(self.ctx.h, u.get(), u.num_qubits(),
                                          i, j, value.real, value.imag))

    def CopyUnitary(self, src: Unitary, dest: Unitary) -> None:
        check(N.lib.qsg_copy_d2d(self.ctx.h, dest.get(), src.get(),
                                 2 * src.num_qubits()))

    def to_numpy(self, u: Unitary) -> np.ndarray:
        """The whole unitary as a (2^n, 2^n) complex128 array, [i, j] being
        GetEntry(u, i, j)."""
        n = u.num_qubits()
        buf = np.empty(self.MinSize(n), dtype=np.float32)
        check(N.lib.qsg_copy_d2h(self.ctx.h, buf.ctypes.data_as(N.P_f32),
                                 u.get(), 2 * n))
        d = 1 << n
        return buf[: 2 * d * d].view(np.complex64).astype(np.complex128).reshape(d, d)


class UnitaryCalculator:
    """UnitaryCalculatorBasic equivalent (lib/unitary_calculator_basic.h:33-124)."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()

    def ApplyGate(self, qs: Sequence[int], matrix, u: Unitary) -> None:
        m, mp = _f32(matrix)
        check(N.lib.qsg_unitary_apply_gate(self.ctx.h, u.get(), u.num_qubits(),
                                           _u32(qs), len(qs), mp))

    def ApplyControlledGate(self, qs: Sequence[int], cqs: Sequence[int],
                            cvals: int, matrix, u: Unitary) -> None:
        m, mp = _f32(matrix)
        check(N.lib.qsg_unitary_apply_controlled_gate(
            self.ctx.h, u.get(), u.num_qubits(), _u32(qs), len(qs), _u32(cqs),
            len(cqs), cvals, mp))

    def RunPlan(self, plan, u: Unitary) -> None:
        """Every op of a fused plan (engine.Plan of an n-qubit circuit)."""
        check(N.lib.qsg_unitary_run_plan(self.ctx.h, plan.h, u.get(),
                                         u.num_qubits()))

    @staticmethod
    def SIMDRegisterSize() -> int:
        return 1
