"""ctypes binding of libqsim_gb300.so (the C ABI declared in
include/qsim_gb300.h).  There is no fallback: if the library is missing,
importing this module raises."""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libqsim_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build it with `python qsim_gb300/build.py` "
        "(nvcc, sm_103a). The engine has no CPU fallback.")

lib = C.CDLL(LIB_PATH)

u32, u64, i32 = C.c_uint, C.c_uint64, C.c_int
f32, f64 = C.c_float, C.c_double
vp = C.c_void_p
P_u32 = C.POINTER(C.c_uint)
P_u64 = C.POINTER(C.c_uint64)
P_f32 = C.POINTER(C.c_float)
P_f64 = C.POINTER(C.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "qsg_last_error": (C.c_char_p, []),
    "qsg_version": (C.c_char_p, []),
    "qsg_ctx_create": (i32, [i32, vp, C.POINTER(vp)]),
    "qsg_ctx_destroy": (i32, [vp]),
    "qsg_ctx_sync": (i32, [vp]),
    "qsg_ctx_num_sms": (i32, [vp, C.POINTER(C.c_int)]),
    "qsg_ctx_stream": (vp, [vp]),
    "qsg_ctx_launch_count": (u64, [vp]),
    "qsg_ctx_scratch_bytes": (i32, [vp, C.POINTER(C.c_size_t),
                                    C.POINTER(C.c_size_t)]),
    "qsg_min_size": (u64, [u32]),
    "qsg_state_create": (i32, [vp, u32, C.POINTER(vp)]),
    "qsg_state_free": (i32, [vp, vp]),
    "qsg_host_alloc": (i32, [C.c_size_t, C.POINTER(vp)]),
    "qsg_host_alloc_near": (i32, [i32, C.c_size_t, C.POINTER(vp)]),
    "qsg_host_numa_node": (i32, [i32, C.POINTER(C.c_int)]),
    "qsg_host_free": (i32, [vp]),
    "qsg_copy_d2d": (i32, [vp, vp, vp, u32]),
    "qsg_copy_d2h": (i32, [vp, vp, vp, u32]),
    "qsg_copy_h2d": (i32, [vp, vp, vp, u32]),
    "qsg_copy_h2d_partial": (i32, [vp, vp, vp, u64, u32]),
    "qsg_internal_to_normal": (i32, [vp, vp, u32]),
    "qsg_normal_to_internal": (i32, [vp, vp, u32]),
    "qsg_set_all_zeros": (i32, [vp, vp, u32]),
    "qsg_set_state_uniform": (i32, [vp, vp, u32]),
    "qsg_set_state_zero": (i32, [vp, vp, u32]),
    "qsg_get_ampl": (i32, [vp, vp, u32, u64, P_f32]),
    "qsg_set_ampl": (i32, [vp, vp, u32, u64, f32, f32]),
    "qsg_bulk_set_ampl": (i32, [vp, vp, u32, u64, u64, f32, f32, i32]),
    "qsg_add": (i32, [vp, vp, vp, u32]),
    "qsg_multiply": (i32, [vp, f32, vp, u32]),
    "qsg_inner_product": (i32, [vp, vp, vp, u32, P_f64]),
    "qsg_real_inner_product": (i32, [vp, vp, vp, u32, P_f64]),
    "qsg_norm": (i32, [vp, vp, u32, P_f64]),
    "qsg_norm_noalloc": (i32, [vp, vp, u32, P_f64]),
    "qsg_num_chunks": (u64, [u32]),
    "qsg_partial_norms": (i32, [vp, vp, u32, P_f64]),
    "qsg_find_measured_bits": (i32, [vp, vp, u32, u64, f64, u64, P_u64]),
    "qsg_sample_sorted": (i32, [vp, vp, u32, u64, P_f64, P_u64]),
    "qsg_sample": (i32, [vp, vp, u32, u64, u32, P_u64]),
    "qsg_sample_thresholds": (i32, [vp, vp, u32, u64, P_f64, P_u64]),
    "qsg_collapse": (i32, [vp, vp, u32, u64, u64]),
    "qsg_measure": (i32, [vp, vp, u32, u64, f64, i32, P_u64]),
    "qsg_apply_gate": (i32, [vp, vp, u32, P_u32, u32, P_f32]),
    "qsg_apply_controlled_gate": (i32, [vp, vp, u32, P_u32, u32, P_u32, u32,
                                        u64, P_f32]),
    "qsg_expectation_value": (i32, [vp, vp, u32, P_u32, u32, P_f32, P_f64]),
    "qsg_apply_gate_tc": (i32, [vp, vp, u32, P_u32, u32, P_f32]),
    "qsg_apply_gate_tc2": (i32, [vp, vp, u32, P_u32, u32, P_f32, P_u32, u32,
                                 P_f32]),
    "qsg_expectation_value_tc": (i32, [vp, vp, u32, P_u32, u32, P_f32, P_f64]),
    "qsg_tc_error": (i32, [vp, C.POINTER(C.c_int)]),
    "qsg_tc_stall_test": (i32, [vp, vp, u32, C.c_longlong]),
    "qsg_simd_register_size": (u32, []),
    "qsg_rng_create": (vp, [u32]),
    "qsg_rng_destroy": (None, [vp]),
    "qsg_rng_next_u32": (u32, [vp]),
    "qsg_rng_uniform": (f64, [vp, f64]),
    "qsg_generate_random_values": (None, [u64, u32, f64, P_f64]),
    "qsg_circuit_create": (i32, [u32, C.POINTER(vp)]),
    "qsg_circuit_destroy": (i32, [vp]),
    "qsg_circuit_info": (i32, [vp, P_u32, P_u64]),
    "qsg_circuit_add_gate": (i32, [vp, u32, P_u32, u32, P_f64]),
    "qsg_circuit_add_controlled_gate": (i32, [vp, u32, P_u32, u32, P_u32, u32,
                                              u64, P_f64]),
    "qsg_circuit_add_measurement": (i32, [vp, u32, P_u32, u32]),
    "qsg_circuit_add_named_gate": (i32, [vp, u32, C.c_char_p, P_u32, u32,
                                         P_f64, u32]),
    "qsg_circuit_parse": (i32, [C.c_char_p, u32, C.POINTER(vp)]),
    "qsg_circuit_grid": (i32, [u32, u32, u32, u32, u64, C.POINTER(vp)]),
    "qsg_circuit_chain": (i32, [u32, u32, u64, C.POINTER(vp)]),
    "qsg_circuit_layered_u3": (i32, [u32, u32, u32, u64, C.POINTER(vp)]),
    "qsg_circuit_get_op": (i32, [vp, u64, C.POINTER(C.c_int), P_u32, P_u32,
                                 P_u32, P_u32, P_u32, P_u64, P_f64]),
    "qsg_pauli_sum": (i32, [u32, u32, u32, u64, P_u32, P_u32, C.c_char_p,
                            P_f64]),
    "qsg_plan_create": (i32, [vp, vp, C.POINTER(vp)]),
    "qsg_plan_create_unfused": (i32, [vp, C.POINTER(vp)]),
    "qsg_plan_destroy": (i32, [vp]),
    "qsg_plan_info": (i32, [vp, P_u64, P_u32, P_u64]),
    "qsg_plan_tc_pairs": (i32, [vp, P_u64, C.POINTER(C.c_ubyte)]),
    "qsg_plan_get_op": (i32, [vp, u64, C.POINTER(C.c_int), P_u32, P_u32,
                              P_u32, P_u32, P_u64, C.POINTER(C.c_int), P_u64,
                              P_f64]),
    "qsg_plan_run": (i32, [vp, vp, vp, u32, P_u64, u64, P_u64]),
    "qsg_plan_capture": (i32, [vp, vp, vp]),
    "qsg_plan_replay": (i32, [vp, vp]),
    "qsg_plan_profile": (i32, [vp, vp, vp, P_f32, u64]),
    "qsg_plan_cache_create": (i32, [u32, C.POINTER(vp)]),
    "qsg_plan_cache_destroy": (i32, [vp]),
    "qsg_plan_cache_clear": (i32, [vp]),
    "qsg_plan_cache_stats": (i32, [vp, P_u64, P_u64, P_u64, P_u64, P_u64]),
    "qsg_plan_cache_run": (i32, [vp, vp, vp, vp, vp, u32, P_u64, u64, P_u64,
                                 C.POINTER(C.c_int)]),
    "qsg_plan_cache_run_text": (i32, [vp, vp, C.c_char_p, u32, vp, vp, u32,
                                      P_u64, u64, P_u64, C.POINTER(C.c_int)]),
    "qsg_noisy_create": (i32, [u32, C.POINTER(vp)]),
    "qsg_noisy_destroy": (i32, [vp]),
    "qsg_noisy_info": (i32, [vp, P_u32, P_u64, P_u64]),
    "qsg_noisy_append_circuit": (i32, [vp, vp]),
    "qsg_noisy_add_channel": (i32, [vp, i32, u32, P_u32, u32, f64]),
    "qsg_noisy_add_kraus_channel": (i32, [vp, u32, P_u32, u32, u32,
                                          C.POINTER(C.c_int), P_f64, P_f64]),
    "qsg_noisy_make": (i32, [vp, f64, f64, u32, C.POINTER(vp)]),
    "qsg_noisy_get_op": (i32, [vp, u64, C.POINTER(C.c_int), P_u32, P_u32,
                               P_u32, P_u32]),
    "qsg_traj_create": (i32, [vp, vp, C.POINTER(vp)]),
    "qsg_traj_destroy": (i32, [vp]),
    "qsg_traj_info": (i32, [vp, P_u32, P_u64, P_u64]),
    "qsg_traj_run": (i32, [vp, vp, vp, u64, P_u64]),
    "qsg_traj_run_from": (i32, [vp, vp, vp, u64, P_u64]),
    "qsg_traj_run_batch": (i32, [i32, C.POINTER(vp), u64, P_u32, P_u64, u64,
                                 vp, P_u64, C.POINTER(vp), P_f32, P_f64,
                                 P_u64]),
    "qsg_unitary_min_size": (u64, [u32]),
    "qsg_unitary_create": (i32, [vp, u32, C.POINTER(vp)]),
    "qsg_unitary_free": (i32, [vp, vp]),
    "qsg_unitary_set_identity": (i32, [vp, vp, u32]),
    "qsg_unitary_set_all_zeros": (i32, [vp, vp, u32]),
    "qsg_unitary_get_entry": (i32, [vp, vp, u32, u64, u64, P_f32]),
    "qsg_unitary_set_entry": (i32, [vp, vp, u32, u64, u64, f32, f32]),
    "qsg_unitary_apply_gate": (i32, [vp, vp, u32, P_u32, u32, P_f32]),
    "qsg_unitary_apply_controlled_gate": (i32, [vp, vp, u32, P_u32, u32, P_u32,
                                                u32, u64, P_f32]),
    "qsg_unitary_run_plan": (i32, [vp, vp, vp, u32]),
    "qsg_hybrid_split": (i32, [vp, P_u32, u32, vp]),
    "qsg_hybrid_run": (i32, [vp, vp, P_u32, u32, vp, P_u64, u64, P_f64, vp]),
    "qsg_circuit_get_schmidt": (i32, [vp, u64, P_u32, P_f64]),
    "qsg_circuit_set_schmidt": (i32, [vp, u64, u32, P_f64]),
    "qsg_traj_run_packed": (i32, [i32, C.POINTER(vp), u64, P_u32, P_u64, u64,
                                  vp, P_u64, C.POINTER(vp), P_f32, P_f64,
                                  P_u64, vp]),
    "qsg_mlp_num_params": (u64, []),
    "qsg_mlp_create": (i32, [u64, C.POINTER(vp)]),
    "qsg_mlp_destroy": (i32, [vp]),
    "qsg_mlp_get_params": (i32, [vp, P_f32]),
    "qsg_mlp_set_params": (i32, [vp, P_f32]),
    "qsg_mlp_gradient": (i32, [vp, vp, P_f32, P_f32, u64, P_f32, P_f64]),
    "qsg_mlp_train": (i32, [vp, vp, P_f32, P_f32, u64, u32, u32, f32, u64,
                            P_f64]),
    "qsg_mlp_predict": (i32, [vp, vp, P_f32, u64, P_f32]),
    "qsg_block_features": (i32, [u32, P_u32, u32, u32, i32, P_f32]),
    "qsg_mlp_cost_us": (i32, [vp, u32, P_u32, u32, u32, i32, P_f64]),
    "qsg_timer_start": (i32, [vp]),
    "qsg_timer_stop": (i32, [vp, P_f32]),
}

for _name, (_res, _args) in SIGNATURES.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


class FuseOptions(C.Structure):
    """qsg_fuse_options."""
    _fields_ = [("max_fused_size", C.c_uint), ("seeds", C.c_uint),
                ("tensor_path", C.c_int), ("tc_min_k", C.c_uint),
                ("cost_model", C.c_void_p), ("tc_pair_bits", C.c_uint)]


class HybridOptions(C.Structure):
    _fields_ = [("prefix", C.c_uint64), ("num_prefix_gatexs", C.c_uint),
                ("num_root_gatexs", C.c_uint), ("max_fused_size", C.c_uint),
                ("tensor_path", C.c_int), ("max_batch_bits", C.c_uint)]


class HybridInfo(C.Structure):
    _fields_ = [("num_qubits0", C.c_uint), ("num_qubits1", C.c_uint),
                ("num_ops0", C.c_uint), ("num_ops1", C.c_uint),
                ("num_gatexs", C.c_uint), ("prefix_bits", C.c_uint),
                ("root_bits", C.c_uint), ("suffix_bits", C.c_uint),
                ("batch_bits", C.c_uint), ("paths_run", C.c_uint64)]


class TrajOptions(C.Structure):
    """qsg_traj_options."""
    _fields_ = [("max_fused_size", C.c_uint), ("seeds", C.c_uint),
                ("collect_kop_stat", C.c_int), ("collect_mea_stat", C.c_int),
                ("normalize_before_mea_gates", C.c_int),
                ("tensor_path", C.c_int), ("tc_min_k", C.c_uint)]


class BatchOptions(C.Structure):
    """qsg_batch_options."""
    _fields_ = [("num_streams", C.c_uint), ("big_qubits", C.c_uint),
                ("big_streams", C.c_uint)]


class PackedOptions(C.Structure):
    """qsg_packed_options."""
    _fields_ = [("ctas_per_sm", C.c_uint), ("max_qubits", C.c_uint),
                ("host_threads", C.c_uint), ("tile_kib", C.c_uint),
                ("overlap", C.c_int), ("streams", BatchOptions)]


class PackedInfo(C.Structure):
    """qsg_packed_info."""
    _fields_ = [("packed_items", C.c_uint64), ("stream_items", C.c_uint64),
                ("ops", C.c_uint64), ("ctas", C.c_uint), ("tile_kib", C.c_uint),
                ("build_s", C.c_double), ("upload_s", C.c_double),
                ("kernel_s", C.c_double), ("stream_s", C.c_double)]


class QsgError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"status {status}: {msg}")
        self.status = status


def check(status: int) -> None:
    if status != 0:
        raise QsgError(status, lib.qsg_last_error().decode())


def u32_array(xs):
    xs = list(xs)
    return (C.c_uint * max(1, len(xs)))(*xs)
