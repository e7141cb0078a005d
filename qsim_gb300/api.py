"""Python mirror of qsim's Simulator / StateSpace template API on the GB300
engine.  Method names, argument meaning and error behaviour follow the
reference (lib/simulator_cuda.h, lib/statespace_cuda.h, lib/statespace.h,
lib/vectorspace_cuda.h); every call goes through the C ABI of
libqsim_gb300.so.

Differences that follow from the C ABI: a failed allocation returns a Null
state (as the reference); CUDA errors raise QsgError instead of exiting.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N
from ._native import check


class Context:
    """Owns a CUDA stream, device scratch and timing events (qsg_ctx)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(N.lib.qsg_ctx_create(device, None, C.byref(h)))
        self.h = h

    def sync(self) -> None:
        check(N.lib.qsg_ctx_sync(self.h))

    def launches(self) -> int:
        return int(N.lib.qsg_ctx_launch_count(self.h))

    def timer_start(self) -> None:
        check(N.lib.qsg_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = C.c_float()
        check(N.lib.qsg_timer_stop(self.h, C.byref(ms)))
        return float(ms.value)

    def num_sms(self) -> int:
        v = C.c_int()
        check(N.lib.qsg_ctx_num_sms(self.h, C.byref(v)))
        return int(v.value)

    def close(self) -> None:
        if self.h:
            N.lib.qsg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class State:
    """Device state vector (VectorSpaceCUDA::Vector, lib/vectorspace_cuda.h:51-82)."""

    def __init__(self, ptr: Optional[int], num_qubits: int, owned: bool,
                 ctx: Context):
        self._ptr = ptr
        self._n = num_qubits
        self._owned = owned
        self._ctx = ctx

    def get(self) -> Optional[int]:
        return self._ptr

    def release(self) -> Optional[int]:
        p, self._ptr, self._n, self._owned = self._ptr, None, 0, False
        return p

    def num_qubits(self) -> int:
        return self._n

    @staticmethod
    def requires_copy_to_host() -> bool:
        return True

    def free(self) -> None:
        if self._owned and self._ptr:
            check(N.lib.qsg_state_free(self._ctx.h, self._ptr))
        self._ptr, self._owned = None, False

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


@dataclass
class MeasurementResult:
    """lib/statespace.h:45-68."""
    mask: int = 0
    bits: int = 0
    bitstring: List[int] = field(default_factory=list)
    valid: bool = False


class Rng:
    """std::mt19937 stand-in used by Measure: draws come from the C++
    standard library through the engine (qsg_rng_*), so measurement
    outcomes follow the reference's generator stream."""

    def __init__(self, seed: int):
        from . import engine
        self._r = engine.Rng(seed)

    def uniform(self, max_value: float) -> float:
        return self._r.uniform(max_value)


def _f32_matrix(matrix) -> "C.Array":
    m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float32).ravel())
    return m, m.ctypes.data_as(N.P_f32)


class StateSpace:
    """StateSpaceCUDA equivalent (lib/statespace_cuda.h:44-472)."""

    @dataclass
    class Parameter:
        # Accepted for interface compatibility (lib/statespace_cuda.h:59-70);
        # the engine sizes its own grids.
        num_threads: int = 512
        num_dblocks: int = 16

    def __init__(self, param: Optional["StateSpace.Parameter"] = None,
                 ctx: Optional[Context] = None):
        self.param = param or StateSpace.Parameter()
        self.ctx = ctx or default_context()

    # ---- vector space -------------------------------------------------
    @staticmethod
    def MinSize(num_qubits: int) -> int:
        return int(N.lib.qsg_min_size(num_qubits))

    def Create(self, num_qubits: int) -> State:
        p = C.c_void_p()
        rc = N.lib.qsg_state_create(self.ctx.h, num_qubits, C.byref(p))
        if rc == 2:  # QSG_ERR_OOM -> Null, as lib/vectorspace_cuda.h:90-95
            return self.Null()
        check(rc)
        return State(p.value, num_qubits, True, self.ctx)

    def Null(self) -> State:
        return State(None, 0, False, self.ctx)

    @staticmethod
    def IsNull(state: State) -> bool:
        return state.get() is None

    def Free(self, state: State) -> None:
        state.free()

    def Copy(self, *args) -> bool:
        """Copy(src, dest) D2D; Copy(src, ndarray) D2H; Copy(ndarray, dest)
        H2D; Copy(ndarray, size, dest) partial H2D (lib/vectorspace_cuda.h:116-160)."""
        if len(args) == 2 and isinstance(args[0], State) and isinstance(args[1], State):
            src, dest = args
            if src.num_qubits() != dest.num_qubits():
                return False
            check(N.lib.qsg_copy_d2d(self.ctx.h, dest.get(), src.get(),
                                     src.num_qubits()))
            return True
        if len(args) == 2 and isinstance(args[0], State):
            src, host = args
            assert host.dtype == np.float32 and host.flags.c_contiguous
            assert host.size >= self.MinSize(src.num_qubits())
            check(N.lib.qsg_copy_d2h(self.ctx.h, host.ctypes.data, src.get(),
                                     src.num_qubits()))
            return True
        if len(args) == 2:
            host, dest = args
            host = np.ascontiguousarray(host, dtype=np.float32)
            assert host.size >= self.MinSize(dest.num_qubits())
            check(N.lib.qsg_copy_h2d(self.ctx.h, dest.get(), host.ctypes.data,
                                     dest.num_qubits()))
            return True
        host, size, dest = args
        host = np.ascontiguousarray(host, dtype=np.float32)
        check(N.lib.qsg_copy_h2d_partial(self.ctx.h, dest.get(),
                                         host.ctypes.data, size,
                                         dest.num_qubits()))
        return True

    def DeviceSync(self) -> None:
        self.ctx.sync()

    # ---- convenience: whole state as complex128 numpy --------------------
    def to_numpy(self, state: State) -> np.ndarray:
        buf = np.empty(self.MinSize(state.num_qubits()), dtype=np.float32)
        self.Copy(state, buf)
        n = 1 << state.num_qubits()
        return buf[: 2 * n].view(np.complex64).astype(np.complex128)

    def from_numpy(self, amps: np.ndarray, state: State) -> None:
        n = state.num_qubits()
        buf = np.zeros(self.MinSize(n), dtype=np.float32)
        a = np.asarray(amps, dtype=np.complex64)
        assert a.size == (1 << n)
        buf[: 2 * a.size] = a.view(np.float32)
        self.Copy(buf, state)

    # ---- state space ------------------------------------------------------
    def InternalToNormalOrder(self, state: State) -> None:
        check(N.lib.qsg_internal_to_normal(self.ctx.h, state.get(),
                                           state.num_qubits()))

    def NormalToInternalOrder(self, state: State) -> None:
        check(N.lib.qsg_normal_to_internal(self.ctx.h, state.get(),
                                           state.num_qubits()))

    def SetAllZeros(self, state: State) -> None:
        check(N.lib.qsg_set_all_zeros(self.ctx.h, state.get(),
                                      state.num_qubits()))

    def SetStateUniform(self, state: State) -> None:
        check(N.lib.qsg_set_state_uniform(self.ctx.h, state.get(),
                                          state.num_qubits()))

    def SetStateZero(self, state: State) -> None:
        check(N.lib.qsg_set_state_zero(self.ctx.h, state.get(),
                                       state.num_qubits()))

    def GetAmpl(self, state: State, i: int) -> complex:
        out = (C.c_float * 2)()
        check(N.lib.qsg_get_ampl(self.ctx.h, state.get(), state.num_qubits(),
                                 i, out))
        return complex(out[0], out[1])

    def SetAmpl(self, state: State, i: int, *val) -> None:
        if len(val) == 1:
            re, im = float(np.real(val[0])), float(np.imag(val[0]))
        else:
            re, im = float(val[0]), float(val[1])
        check(N.lib.qsg_set_ampl(self.ctx.h, state.get(), state.num_qubits(),
                                 i, re, im))

    def BulkSetAmpl(self, state: State, mask: int, bits: int, *val,
                    exclude: bool = False) -> None:
        if len(val) == 1:
            re, im = float(np.real(val[0])), float(np.imag(val[0]))
        else:
            re, im = float(val[0]), float(val[1])
        check(N.lib.qsg_bulk_set_ampl(self.ctx.h, state.get(),
                                      state.num_qubits(), mask, bits, re, im,
                                      int(exclude)))

    def Add(self, src: State, dest: State) -> bool:
        if src.num_qubits() != dest.num_qubits():
            return False
        check(N.lib.qsg_add(self.ctx.h, src.get(), dest.get(),
                            src.num_qubits()))
        return True

    def Multiply(self, a: float, state: State) -> None:
        check(N.lib.qsg_multiply(self.ctx.h, float(a), state.get(),
                                 state.num_qubits()))

    def InnerProduct(self, s1: State, s2: State) -> complex:
        if s1.num_qubits() != s2.num_qubits():
            return complex(float("nan"))
        out = (C.c_double * 2)()
        check(N.lib.qsg_inner_product(self.ctx.h, s1.get(), s2.get(),
                                      s1.num_qubits(), out))
        return complex(out[0], out[1])

    def RealInnerProduct(self, s1: State, s2: State) -> float:
        if s1.num_qubits() != s2.num_qubits():
            return float("nan")
        out = C.c_double()
        check(N.lib.qsg_real_inner_product(self.ctx.h, s1.get(), s2.get(),
                                           s1.num_qubits(), C.byref(out)))
        return out.value

    def Norm(self, state: State) -> float:
        out = C.c_double()
        check(N.lib.qsg_norm(self.ctx.h, state.get(), state.num_qubits(),
                             C.byref(out)))
        return out.value

    def Sample(self, state: State, num_samples: int, seed: int) -> List[int]:
        out = np.zeros(max(1, num_samples), dtype=np.uint64)
        check(N.lib.qsg_sample(self.ctx.h, state.get(), state.num_qubits(),
                               num_samples, seed & 0xFFFFFFFF,
                               out.ctypes.data_as(N.P_u64)))
        return [int(x) for x in out[:num_samples]]

    def SampleSorted(self, state: State, sorted_u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(sorted_u, dtype=np.float64)
        out = np.zeros(max(1, u.size), dtype=np.uint64)
        check(N.lib.qsg_sample_sorted(self.ctx.h, state.get(),
                                      state.num_qubits(), u.size,
                                      u.ctypes.data_as(N.P_f64),
                                      out.ctypes.data_as(N.P_u64)))
        return out[: u.size]

    def Collapse(self, mr: MeasurementResult, state: State) -> None:
        check(N.lib.qsg_collapse(self.ctx.h, state.get(), state.num_qubits(),
                                 mr.mask, mr.bits))

    def PartialNorms(self, state: State) -> np.ndarray:
        nc = int(N.lib.qsg_num_chunks(state.num_qubits()))
        out = np.zeros(nc, dtype=np.float64)
        check(N.lib.qsg_partial_norms(self.ctx.h, state.get(),
                                      state.num_qubits(),
                                      out.ctypes.data_as(N.P_f64)))
        return out

    def FindMeasuredBits(self, m: int, r: float, mask: int,
                         state: State) -> int:
        out = C.c_uint64()
        check(N.lib.qsg_find_measured_bits(self.ctx.h, state.get(),
                                           state.num_qubits(), m, r, mask,
                                           C.byref(out)))
        return int(out.value)

    def VirtualMeasure(self, qubits: Sequence[int], rgen,
                       state: State) -> MeasurementResult:
        """lib/statespace.h:97-140 on the device: one uniform draw from
        `rgen`, CDF search over the whole state."""
        res = MeasurementResult(valid=True)
        for q in qubits:
            if q >= state.num_qubits():
                return MeasurementResult(valid=False)
            res.mask |= 1 << q
        u = rgen.uniform(1.0)
        out = C.c_uint64()
        check(N.lib.qsg_measure(self.ctx.h, state.get(), state.num_qubits(),
                                res.mask, u, 0, C.byref(out)))
        res.bits = int(out.value)
        res.bitstring = [(res.bits >> q) & 1 for q in qubits]
        return res

    def Measure(self, qubits: Sequence[int], rgen,
                state: State) -> MeasurementResult:
        res = self.VirtualMeasure(qubits, rgen, state)
        if res.valid:
            self.Collapse(res, state)
        return res


class Simulator:
    """SimulatorCUDA equivalent (lib/simulator_cuda.h:34-267)."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()

    def ApplyGate(self, qs: Sequence[int], matrix, state: State) -> None:
        m, mp = _f32_matrix(matrix)
        q = N.u32_array(qs)
        check(N.lib.qsg_apply_gate(self.ctx.h, state.get(),
                                   state.num_qubits(), q, len(qs), mp))

    def ApplyControlledGate(self, qs: Sequence[int], cqs: Sequence[int],
                            cvals: int, matrix, state: State) -> None:
        m, mp = _f32_matrix(matrix)
        check(N.lib.qsg_apply_controlled_gate(
            self.ctx.h, state.get(), state.num_qubits(), N.u32_array(qs),
            len(qs), N.u32_array(cqs), len(cqs), cvals, mp))

    def ExpectationValue(self, qs: Sequence[int], matrix,
                         state: State) -> complex:
        m, mp = _f32_matrix(matrix)
        out = (C.c_double * 2)()
        check(N.lib.qsg_expectation_value(self.ctx.h, state.get(),
                                          state.num_qubits(),
                                          N.u32_array(qs), len(qs), mp, out))
        return complex(out[0], out[1])

    @staticmethod
    def SIMDRegisterSize() -> int:
        return int(N.lib.qsg_simd_register_size())
