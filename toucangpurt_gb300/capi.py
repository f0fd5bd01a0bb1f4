"""ctypes binding of the C ABI declared in include/toucan_gb300.h.

This is the only way Python reaches the simulator: every call goes through
``libtoucan_gb300.so``.  Loading fails loudly when the library is missing;
there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libtoucan_gb300.so"
_lib = None

u8p = C.POINTER(C.c_uint8)
u16p = C.POINTER(C.c_uint16)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i64p = C.POINTER(C.c_int64)

# status codes (toucan_gb300.h)
OK = 0
ERR_ARG, ERR_IO, ERR_FORMAT, ERR_INVALID_DESIGN, ERR_CUDA, ERR_NO_DEVICE = -1, -2, -3, -4, -5, -6
ERR_RESOURCES, ERR_TIMEOUT, ERR_STATE, ERR_NOT_FOUND, ERR_RANGE, ERR_DEVICE_FAULT = -7, -8, -9, -10, -11, -12

SCHED_GREEDY, SCHED_LEARNED = 0, 1
MODE_PERSISTENT, MODE_GRAPH = 0, 1
BATCH_CYCLE_DIGESTS, BATCH_ROLLING, BATCH_FINAL_STATE, BATCH_CONTINUE, BATCH_STOP_EXIT = 1, 2, 4, 8, 16


class TgsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Options(C.Structure):
    _fields_ = [
        ("n_streams", C.c_uint32), ("warps_per_block", C.c_uint32), ("groups_per_item", C.c_uint32),
        ("blocks_per_sm", C.c_uint32), ("schedule", C.c_uint32), ("mode", C.c_uint32),
        ("barrier_timeout_ms", C.c_uint32), ("validate", C.c_uint32), ("resident_netlist", C.c_uint32),
        ("value_pool", C.c_uint32), ("capture_signals", C.c_uint32), ("lane_packing", C.c_uint32),
        ("fast_luts", C.c_uint32), ("mpart_lanes", C.c_uint32), ("levels_per_barrier", C.c_uint32),
        ("stage_words", C.c_uint32),
    ]


class Stimulus(C.Structure):
    _fields_ = [
        ("base_seed", C.c_uint64), ("n_inputs", C.c_uint32), ("reg", u32p), ("bits", u8p), ("toggle", u16p),
        ("table", u8p),
    ]


class Batch(C.Structure):
    _fields_ = [
        ("n_streams", C.c_uint32), ("cycles", u32p), ("stim", C.POINTER(Stimulus)), ("flags", C.c_uint32),
        ("slots", C.c_uint32),
    ]


class BatchResult(C.Structure):
    _fields_ = [
        ("final_reg_digest", u64p), ("final_mem_digest", u64p), ("rolling_digest", u64p), ("cycle_digest", u64p),
        ("cycle_stride", C.c_uint32), ("stop_cycle", u32p), ("final_regs", u8p), ("final_mems", u8p),
        ("device_ms", C.c_double), ("stream_cycles", C.c_uint64), ("launches", C.c_uint32),
    ]


class GenConfig(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64), ("n_lut", C.c_uint64), ("levels", C.c_uint32), ("operands", C.c_uint32),
        ("ff_bits", C.c_uint32), ("pi_bits", C.c_uint32), ("reset_inputs", C.c_uint32),
        ("n_mems", C.c_uint32), ("mem_depth", C.c_uint32), ("mem_width", C.c_uint32),
        ("mem_read_ports", C.c_uint32), ("mem_write_ports", C.c_uint32), ("mem_multi_writer", C.c_uint32),
        ("n_vec_ops", C.c_uint32), ("vec_nibbles", C.c_uint32), ("palette_pct", C.c_uint32),
        ("fanout_alpha", C.c_float), ("max_fanout", C.c_uint32), ("luts_per_part", C.c_uint32),
        ("mpart_width", C.c_uint32), ("cone_depth", C.c_uint32), ("mixed", C.c_uint32), ("with_stop", C.c_uint32),
        ("signals", C.c_uint32), ("reserved", C.c_uint32 * 5),
    ]


class GenInfo(C.Structure):
    _fields_ = [
        ("lut_ops", C.c_uint64), ("nop_ops", C.c_uint64), ("mparts", C.c_uint64), ("partitions", C.c_uint64),
        ("mem_read_ops", C.c_uint64), ("mem_write_ops", C.c_uint64), ("vec_ops", C.c_uint64), ("l0_ops", C.c_uint64),
        ("reg_pool", C.c_uint32), ("mem_pool", C.c_uint32), ("exchange_pool", C.c_uint32),
        ("max_value_pool", C.c_uint32), ("n_pi_nibbles", C.c_uint32), ("reserved", C.c_uint32 * 7),
    ]


class DesignStats(C.Structure):
    _fields_ = [
        ("lut_ops", C.c_uint64), ("nop_ops", C.c_uint64), ("writeback_ops", C.c_uint64),
        ("l0_reg_reads", C.c_uint64), ("l0_exg_reads", C.c_uint64), ("reg_copy_slots", C.c_uint64),
        ("exg_copy_slots", C.c_uint64), ("mem_read_ops", C.c_uint64), ("mem_write_ops", C.c_uint64),
        ("vec_ops", C.c_uint64), ("vec_read_ops", C.c_uint64), ("print_ops", C.c_uint64), ("stop_ops", C.c_uint64),
        ("op_slots", C.c_uint64), ("partitions", C.c_uint32), ("mparts", C.c_uint32), ("max_value_pool", C.c_uint32),
        ("max_exec_levels", C.c_uint32), ("blocks", C.c_uint32), ("threads", C.c_uint32),
        ("groups_per_item", C.c_uint32), ("streams_per_word", C.c_uint32), ("block_barriers", C.c_uint64),
        ("exec_levels", C.c_uint64), ("makespan", C.c_double * 2), ("smem_per_block", C.c_uint32),
        ("stage_words", C.c_uint32), ("resident_words", C.c_uint32), ("fused_levels", C.c_uint32),
        ("reserved", C.c_uint32 * 4),
    ]


class TrainOpts(C.Structure):
    _fields_ = [("epochs", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_float), ("seed", C.c_uint64),
                ("val_frac", C.c_float), ("reserved", C.c_uint32 * 4)]


class TrainReport(C.Structure):
    _fields_ = [("train_mse", C.c_float), ("val_mse", C.c_float), ("val_corr", C.c_float), ("gate_corr", C.c_float),
                ("samples", C.c_uint32), ("epochs", C.c_uint32), ("train_ms", C.c_double), ("reserved", C.c_uint32 * 4)]


class TuneOpts(C.Structure):
    _fields_ = [("cycles", C.c_uint32), ("warmup", C.c_uint32), ("modes", C.c_uint32), ("try_unstaged", C.c_uint32),
                ("reserved", C.c_uint32 * 4)]


class TuneTrial(C.Structure):
    _fields_ = [("groups_per_item", C.c_uint32), ("warps_per_block", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("mode", C.c_uint32), ("staged", C.c_uint32), ("blocks", C.c_uint32), ("ms_per_cycle", C.c_float),
                ("mpart_lanes", C.c_uint32), ("levels_per_barrier", C.c_uint32)]


MLP_PARAMS = 5313

# (name, argtypes) of every exported entry point; all return int status
# except tgs_last_error / tgs_version.
class ScheduleStats(C.Structure):
    _fields_ = [
        ("exec_levels", C.c_uint64), ("blocks", C.c_uint64), ("barriers", C.c_uint64), ("fused_levels", C.c_uint64),
        ("schedule_words", C.c_uint64), ("max_level_words", C.c_uint32), ("reserved0", C.c_uint32),
        ("makespan", C.c_double), ("work", C.c_double), ("level_bound", C.c_double), ("list_bound", C.c_double),
        ("reserved", C.c_uint64 * 3),
    ]


class RepackStats(C.Structure):
    _fields_ = [("mparts_before", C.c_uint64), ("mparts_after", C.c_uint64), ("lut_ops", C.c_uint64),
                ("fast_lut_ops", C.c_uint64), ("fast_mparts", C.c_uint64), ("exec_levels", C.c_uint64),
                ("reserved", C.c_uint64 * 2)]


SIGNATURES = {
    "tgs_create": [C.POINTER(C.c_void_p)],
    "tgs_destroy": [C.c_void_p],
    "tgs_default_options": [C.POINTER(Options)],
    "tgs_set_options": [C.c_void_p, C.POINTER(Options)],
    "tgs_autotune": [C.c_void_p, C.POINTER(TuneOpts), C.POINTER(TuneTrial), C.c_uint32, C.POINTER(C.c_uint32),
                     C.POINTER(TuneTrial)],
    "tgs_get_options": [C.c_void_p, C.POINTER(Options)],
    "tgs_init": [C.c_void_p, C.c_int, C.c_char_p, C.c_char_p, C.c_int, C.c_int],
    "tgs_init_from_memory": [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int, C.c_int],
    "tgs_eval": [C.c_void_p, C.POINTER(C.c_int)],
    "tgs_eval_free_running": [C.c_void_p, C.c_uint32, C.POINTER(C.c_int)],
    "tgs_set_register": [C.c_void_p, C.c_char_p, C.c_uint64],
    "tgs_read_register": [C.c_void_p, C.c_char_p, u64p],
    "tgs_set_register_stream": [C.c_void_p, C.c_uint32, C.c_char_p, C.c_uint64],
    "tgs_read_register_stream": [C.c_void_p, C.c_uint32, C.c_char_p, u64p],
    "tgs_read_registers": [C.c_void_p, C.c_uint32, C.POINTER(C.c_char_p), C.c_uint32, u64p],
    "tgs_read_signal": [C.c_void_p, C.c_char_p, u64p],
    "tgs_get_real_cycles": [C.c_void_p, u32p],
    "tgs_get_cycle_cnt": [C.c_void_p, u64p],
    "tgs_set_enable_print": [C.c_void_p, C.c_int],
    "tgs_get_eval_done": [C.c_void_p, C.POINTER(C.c_int)],
    "tgs_copy_profile_data": [C.c_void_p, i64p, i64p, C.c_size_t],
    "tgs_get_pool_sizes": [C.c_void_p, u32p, u32p, u32p],
    "tgs_read_reg_pool": [C.c_void_p, C.c_uint32, u8p, C.c_size_t],
    "tgs_write_reg_pool": [C.c_void_p, C.c_uint32, u8p, C.c_size_t],
    "tgs_read_mem_pool": [C.c_void_p, C.c_uint32, u8p, C.c_size_t],
    "tgs_write_mem_pool": [C.c_void_p, C.c_uint32, u8p, C.c_size_t],
    "tgs_state_digest": [C.c_void_p, C.c_uint32, u64p, u64p],
    "tgs_reset_state": [C.c_void_p],
    "tgs_pool_digests_noalloc": [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint32, u64p],
    "tgs_batch_run": [C.c_void_p, C.POINTER(Batch), C.POINTER(BatchResult)],
    "tgs_get_design_stats": [C.c_void_p, C.POINTER(DesignStats)],
    "tgs_host_alloc": [C.c_size_t, C.POINTER(C.c_void_p)],
    "tgs_host_free": [C.c_void_p],
    "tgs_device_reset": [C.c_int],
    "tgs_num_mparts": [C.c_void_p, u32p],
    "tgs_mpart_features": [C.c_void_p, C.POINTER(C.c_float), C.c_uint32],
    "tgs_profile_mparts": [C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.c_uint32],
    "tgs_cost_model_train": [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32,
                             C.POINTER(TrainOpts), C.POINTER(TrainReport)],
    "tgs_cost_model_state": [C.c_void_p, C.POINTER(C.c_float), C.c_size_t, C.c_int],
    "tgs_mlp_forward": [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_float)],
    "tgs_mlp_grad": [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32,
                     C.POINTER(C.c_float), C.POINTER(C.c_float)],
    "tgs_default_gen_config": [C.POINTER(GenConfig)],
    "tgs_generate": [C.POINTER(GenConfig), C.c_char_p, C.c_char_p, C.POINTER(GenInfo)],
    "tgs_gen_inputs": [C.POINTER(GenConfig), u32p, u8p, C.c_uint32],
    "tgs_validate_file": [C.c_char_p, C.c_char_p, u64p],
    "tgs_compact_design": [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)],
    "tgs_pack_design": [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)],
    "tgs_repack_design": [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(RepackStats)],
    "tgs_plan_schedule": [C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_uint32,
                          C.POINTER(ScheduleStats)],
    "tgs_dump_state": [C.c_void_p, C.c_char_p],
    "tgs_read_signal_stream": [C.c_void_p, C.c_uint32, C.c_char_p, C.POINTER(C.c_uint64)],
    "tgs_enable_vcd": [C.c_void_p, C.c_char_p],
    "tgs_eval_until_stop": [C.c_void_p, C.c_uint32, C.POINTER(C.c_int), C.POINTER(C.c_uint32)],
    "tgs_load_state": [C.c_void_p, C.c_char_p],
    "tgs_resave_design": [C.c_char_p, C.c_char_p],
    "tgs_resave_symbols": [C.c_char_p, C.c_char_p],
    "tgs_initial_state": [C.c_char_p, C.c_char_p, C.c_int, u8p, C.c_size_t, u8p, C.c_size_t],
}


def library_path() -> Path:
    return _LIB_PATH


def lib() -> C.CDLL:
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"{_LIB_PATH} is missing: run toucangpurt_gb300.build.build() first")
        L = C.CDLL(str(_LIB_PATH))
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.tgs_last_error.restype = C.c_char_p
        L.tgs_last_error.argtypes = []
        L.tgs_version.restype = C.c_char_p
        L.tgs_version.argtypes = []
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != OK:
        raise TgsError(rc, lib().tgs_last_error().decode(errors="replace"))
