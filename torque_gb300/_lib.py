"""ctypes binding of libtorque_gb300.so (the C ABI in include/torque_gb300.h).

Loading fails loudly: there is no CPU fallback for any operation.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtorque_gb300.so")

TQ_OK, TQ_ERR_INVALID, TQ_ERR_CUDA, TQ_ERR_OOM, TQ_ERR_RANGE, TQ_ERR_UNSUPPORTED, \
    TQ_ERR_TIMEOUT = range(7)
TQ_F32, TQ_F64, TQ_F16 = 0, 1, 2
TQ_MEM_HOST, TQ_MEM_DEVICE = 0, 1
PRECISIONS = {"native": 0, "fp64": 0, "ozaki": 1, "bf16x3": 2, "tensor": 3}
LAYOUTS = {"reference": 0, "reduced": 1}

# Every exported symbol of include/torque_gb300.h with its ctypes signature.
P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
P64 = ctypes.POINTER(ctypes.c_int64)
PP = ctypes.POINTER(ctypes.c_void_p)
ST = ctypes.c_int


class ContractOpts(ctypes.Structure):
    _fields_ = [("precision", I32), ("layout", I32), ("slices", I32), ("tile_n", I32),
                ("native_fill", I32), ("reserved", I32)]


class TuneEntry(ctypes.Structure):
    _fields_ = [("opts", ContractOpts), ("status", I32), ("ms", ctypes.c_float),
                ("rel_err", ctypes.c_double)]


TQ_N_FEATURES = 32

SIGNATURES = {
    "tq_bs_create_empty": (ST, [I32, I32, P64, PP]),
    "tq_bs_create": (ST, [I32, I32, P64, I64, P64, P64, P64, P, I32, P, PP]),
    "tq_bs_clone": (ST, [P, P, PP]),
    "tq_bs_create_zeros": (ST, [I32, I32, P64, I64, P64, P64, P64, P, PP]),
    "tq_bs_adopt": (ST, [I32, I32, P64, I64, P64, P64, P64, P64, P, PP]),
    "tq_bs_set_data": (ST, [P, P, I32, P]),
    "tq_bs_set_data_async": (ST, [P, P, I32, P]),
    "tq_bs_destroy": (ST, [P]),
    "tq_bs_append_blocks": (ST, [P, I64, P64, P64, P64, P, I32, P]),
    "tq_bs_query": (ST, [P, P64, P]),
    "tq_bs_modify": (ST, [P, P64, P]),
    "tq_bs_to_number": (ST, [P, P]),
    "tq_bs_shape": (ST, [P, ctypes.POINTER(I32), ctypes.POINTER(I32), P64, P64]),
    "tq_bs_metadata": (ST, [P, P64, P64, P64, P64, P64]),
    "tq_bs_device_data": (ST, [P, PP]),
    "tq_bs_copy_data": (ST, [P, P, I32, P]),
    "tq_bs_contract": (ST, [P, P, I32, P64, P64, ctypes.POINTER(ContractOpts), P, PP]),
    "tq_bs_split_leg": (ST, [P, I32, I64, P64, I64, P64, P64, P, PP]),
    "tq_bs_contract_elements": (ST, [P, P, I32, P64, P64, P, PP]),
    "tq_bs_svd": (ST, [P, I32, P64, I64, ctypes.c_double, P, PP, PP, PP]),
    "tq_bs_qr": (ST, [P, I32, P64, P, PP, PP]),
    "tq_charge_blocks": (ST, [I32, P64, P64, P64, ctypes.POINTER(ctypes.c_int32), I64, I64, I64,
                              P64, P64, P64]),
    "tq_bs_create_charges": (ST, [I32, I32, P64, P64, P64, ctypes.POINTER(ctypes.c_int32), I64,
                                  I64, P, I32, P, PP]),
    "tq_contract_blocks": (ST, [P, P, I32, P64, P64, I32, I64, P64, P64, P64, P64, P64, P64,
                                P64, P]),
    "tq_bs_hard_transpose": (ST, [P, P64, P, PP]),
    "tq_bs_slice": (ST, [P, P64, P, PP]),
    "tq_bs_fuse_legs": (ST, [P, I32, I64, P64, I64, P64, P64, P, PP]),
    "tq_nest_sum": (ST, [P, I64, P, P, P]),
    "tq_nest_sum_noalloc": (ST, [P, I64, P, P, P]),
    "tq_plan_create": (ST, [P, P, I32, P64, P64, ctypes.POINTER(ContractOpts), P, PP, PP]),
    "tq_plan_execute": (ST, [P, P]),
    "tq_plan_execute_to": (ST, [P, P, ctypes.c_int32, P]),
    "tq_plan_flops": (ST, [P, ctypes.POINTER(ctypes.c_double), P64]),
    "tq_plan_destroy": (ST, [P]),
    "tq_plan_set_profiling": (ST, [P, I32]),
    "tq_plan_last_timings": (ST, [P, ctypes.POINTER(ctypes.c_float),
                                  ctypes.POINTER(ctypes.c_float)]),
    "tq_plan_check": (ST, [P, P]),
    "tq_plan_reschedule": (ST, [P, ctypes.POINTER(ContractOpts), P]),
    "tq_plan_features": (ST, [P, ctypes.c_double, ctypes.POINTER(ctypes.c_float), P]),
    "tq_autotune": (ST, [P, ctypes.c_double, P, I32, I32, ctypes.POINTER(I32), P]),
    "tq_mlp_create": (ST, [I32, I32, I32, ctypes.c_uint64, PP]),
    "tq_mlp_destroy": (ST, [P]),
    "tq_mlp_num_params": (ST, [P, P64]),
    "tq_mlp_get_params": (ST, [P, P]),
    "tq_mlp_set_params": (ST, [P, P]),
    "tq_mlp_forward": (ST, [P, P, I64, P, P]),
    "tq_mlp_gradients": (ST, [P, P, P, P, I64, P, P, P]),
    "tq_mlp_train_step": (ST, [P, P, P, P, I64, ctypes.c_float, P, P]),
    "tq_batch_create": (ST, [PP, I32, ctypes.POINTER(I32), P, PP]),
    "tq_batch_execute": (ST, [P, P]),
    "tq_batch_graph_launch": (ST, [P, P]),
    "tq_batch_check": (ST, [P, P]),
    "tq_batch_kernels": (ST, [P, P64]),
    "tq_batch_destroy": (ST, [P]),
    "tq_last_error_string": (ctypes.c_char_p, []),
    "tq_release_cached_memory": (ST, []),
    "tq_debug_fail_alloc_after": (None, [I64]),
    "tq_debug_set_waits": (None, [ctypes.c_uint64, ctypes.c_uint64]),
    "tq_debug_kernel_launches": (I64, []),
}


class TorqueError(RuntimeError):
    """A call of the C ABI failed; .status holds the tq_status code."""

    def __init__(self, status: int, msg: str):
        super().__init__("Error: " + msg)
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Load the shared library (build it first with torque_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libtorque_gb300.so is not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int):
    if status != TQ_OK:
        msg = load().tq_last_error_string().decode()
        raise TorqueError(status, msg)
