"""Python host API mirroring toucanGPUSim::ToucanSimulator (reference
include/ToucanGPUSim.h:10-74), plus batched stimulus runs and the synthetic
design generator.  Everything calls the C ABI (capi.py); nothing here
evaluates a design.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import capi
from .capi import check, lib


def _ptr(a: np.ndarray | None, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


class Simulator:
    """One simulator handle (the reference's ToucanSimulator)."""

    def __init__(self, **options):
        self._h = C.c_void_p()
        check(lib().tgs_create(C.byref(self._h)))
        self._opt = capi.Options()
        check(lib().tgs_default_options(C.byref(self._opt)))
        self.set_options(**options)

    # -- lifetime -------------------------------------------------------
    def cleanup(self) -> None:
        if self._h:
            lib().tgs_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.cleanup()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # -- options ----------------------------------------------------------
    def set_options(self, **kw) -> None:
        for k, v in kw.items():
            if not hasattr(self._opt, k):
                raise TypeError(f"unknown option {k}")
            setattr(self._opt, k, int(v))
        check(lib().tgs_set_options(self._h, C.byref(self._opt)))

    def options(self) -> dict:
        o = capi.Options()
        check(lib().tgs_get_options(self._h, C.byref(o)))
        return {f: getattr(o, f) for f, _ in capi.Options._fields_ if f != "reserved"}

    # -- ToucanSimulator API ---------------------------------------------
    def init(self, gpu_id: int, design_bin: str | Path, symbol_bin: str | Path | None, should_randomize: bool = False,
             enable_print: bool = False) -> int:
        """ToucanSimulator::init: 0 on success; raises TgsError otherwise."""
        sym = str(symbol_bin).encode() if symbol_bin is not None else None
        check(lib().tgs_init(self._h, gpu_id, str(design_bin).encode(), sym, int(should_randomize), int(enable_print)))
        return 0

    def eval(self) -> bool:
        stop = C.c_int()
        check(lib().tgs_eval(self._h, C.byref(stop)))
        return bool(stop.value)

    def eval_free_running(self, max_cycles: int) -> bool:
        stop = C.c_int()
        check(lib().tgs_eval_free_running(self._h, int(max_cycles), C.byref(stop)))
        return bool(stop.value)

    def eval_until_stop(self, max_cycles: int) -> tuple[bool, int]:
        """Free running that ends once every stream executed a stop op
        (stopped streams freeze).  Returns (stop flag, cycles run)."""
        stop, ran = C.c_int(), C.c_uint32()
        check(lib().tgs_eval_until_stop(self._h, int(max_cycles), C.byref(stop), C.byref(ran)))
        return bool(stop.value), ran.value

    def set_register(self, name: str, value: int, stream: int = 0) -> None:
        check(lib().tgs_set_register_stream(self._h, stream, name.encode(), int(value)))

    def read_register(self, name: str, stream: int = 0) -> int:
        v = C.c_uint64()
        check(lib().tgs_read_register_stream(self._h, stream, name.encode(), C.byref(v)))
        return v.value

    def read_registers(self, names, stream: int = 0) -> list[int]:
        """Many registers of one stream with one gather and one copy back."""
        arr = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
        out = np.zeros(max(1, len(names)), np.uint64)
        check(lib().tgs_read_registers(self._h, stream, arr, len(names), _ptr(out, C.c_uint64)))
        return [int(v) for v in out[: len(names)]]

    # reference spellings
    setRegister = set_register
    readRegister = read_register

    def read_signal(self, name: str, stream: int = 0) -> int:
        """Value of a symbol-file signal in the last evaluated cycle (needs
        the capture_signals option)."""
        v = C.c_uint64()
        check(lib().tgs_read_signal_stream(self._h, stream, name.encode(), C.byref(v)))
        return v.value

    readSignal = read_signal

    def enable_vcd(self, path) -> None:
        """VCD dump of every signal of stream 0 (ToucanSimulator::enableVCDDump)."""
        check(lib().tgs_enable_vcd(self._h, str(path).encode()))

    def real_cycles(self) -> int:
        v = C.c_uint32()
        check(lib().tgs_get_real_cycles(self._h, C.byref(v)))
        return v.value

    def cycle_cnt(self) -> int:
        v = C.c_uint64()
        check(lib().tgs_get_cycle_cnt(self._h, C.byref(v)))
        return v.value

    def eval_done(self) -> bool:
        v = C.c_int()
        check(lib().tgs_get_eval_done(self._h, C.byref(v)))
        return bool(v.value)

    def set_enable_print(self, on: bool) -> None:
        check(lib().tgs_set_enable_print(self._h, int(on)))

    def profile(self, n_parts: int) -> tuple[np.ndarray, np.ndarray]:
        u = np.zeros(n_parts, np.int64)
        t = np.zeros(n_parts, np.int64)
        check(lib().tgs_copy_profile_data(self._h, _ptr(u, C.c_int64), _ptr(t, C.c_int64), n_parts))
        return u, t

    def autotune(self, cycles: int = 16, warmup: int = 2, modes: int = 0, try_unstaged: bool = False):
        """Times the launch configurations on the loaded design; keeps the
        fastest (options updated, state reset).  Returns (best, trials) as dicts."""
        o = capi.TuneOpts(cycles, warmup, modes, int(try_unstaged))
        trials = (capi.TuneTrial * 256)()
        n, best = C.c_uint32(), capi.TuneTrial()
        check(lib().tgs_autotune(self._h, C.byref(o), trials, 256, C.byref(n), C.byref(best)))
        conv = lambda t: {f: getattr(t, f) for f, _ in capi.TuneTrial._fields_}
        check(lib().tgs_get_options(self._h, C.byref(self._opt)))
        return conv(best), [conv(trials[i]) for i in range(min(n.value, 256))]

    def design_stats(self) -> dict:
        st = capi.DesignStats()
        check(lib().tgs_get_design_stats(self._h, C.byref(st)))
        d = {f: getattr(st, f) for f, _ in capi.DesignStats._fields_ if f not in ("reserved", "makespan")}
        d["makespan"] = [st.makespan[0], st.makespan[1]]
        return d

    # -- state --------------------------------------------------------------
    def pool_sizes(self) -> tuple[int, int, int]:
        r, m, e = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().tgs_get_pool_sizes(self._h, C.byref(r), C.byref(m), C.byref(e)))
        return r.value, m.value, e.value

    def reg_pool(self, stream: int = 0) -> np.ndarray:
        n = self.pool_sizes()[0]
        a = np.zeros(n, np.uint8)
        check(lib().tgs_read_reg_pool(self._h, stream, _ptr(a, C.c_uint8), n))
        return a

    def write_reg_pool(self, data: np.ndarray, stream: int = 0) -> None:
        a = np.ascontiguousarray(data, np.uint8)
        check(lib().tgs_write_reg_pool(self._h, stream, _ptr(a, C.c_uint8), a.size))

    def mem_pool(self, stream: int = 0) -> np.ndarray:
        n = self.pool_sizes()[1]
        a = np.zeros(n, np.uint8)
        check(lib().tgs_read_mem_pool(self._h, stream, _ptr(a, C.c_uint8), n))
        return a

    def write_mem_pool(self, data: np.ndarray, stream: int = 0) -> None:
        a = np.ascontiguousarray(data, np.uint8)
        check(lib().tgs_write_mem_pool(self._h, stream, _ptr(a, C.c_uint8), a.size))

    def digest(self, stream: int = 0) -> tuple[int, int]:
        r, m = C.c_uint64(), C.c_uint64()
        check(lib().tgs_state_digest(self._h, stream, C.byref(r), C.byref(m)))
        return r.value, m.value

    def reset_state(self) -> None:
        check(lib().tgs_reset_state(self._h))

    def dump_state(self, path) -> None:
        """Checkpoint every stream's state and the cycle counters to a file."""
        check(lib().tgs_dump_state(self._h, str(path).encode()))

    def load_state(self, path) -> None:
        """Restore a checkpoint of the same design (takes its stream count)."""
        check(lib().tgs_load_state(self._h, str(path).encode()))
        check(lib().tgs_get_options(self._h, C.byref(self._opt)))

    # -- batched runs ---------------------------------------------------------
    def batch_run(self, cycles, stim: "StimulusSpec | None" = None, *, cycle_digests: bool = False,
                  rolling: bool = True, final_state: bool = False, slots: int = 0, continue_: bool = False,
                  final_digests: bool = True, stop_exit: bool = False) -> "BatchOutput":
        cyc = np.ascontiguousarray(cycles, np.uint32)
        n = int(cyc.size)
        out = BatchOutput(n)
        stride = int(cyc.max()) if cycle_digests else 0
        if cycle_digests:
            out.cycle_digest = np.zeros((n, stride), np.uint64)
        if final_state:
            r, m, _ = self.pool_sizes()
            out.final_regs = np.zeros((n, r), np.uint8)
            out.final_mems = np.zeros((n, m), np.uint8)
        flags = (capi.BATCH_CYCLE_DIGESTS if cycle_digests else 0) | (capi.BATCH_ROLLING if rolling else 0) | (
            capi.BATCH_FINAL_STATE if final_state else 0) | (capi.BATCH_CONTINUE if continue_ else 0) | (
            capi.BATCH_STOP_EXIT if stop_exit else 0)
        st_ptr = C.cast(None, C.POINTER(capi.Stimulus))
        keep = []
        if stim is not None:
            s = stim.to_c()
            keep.append(s)
            st_ptr = C.pointer(s[0])
        job = capi.Batch(n, _ptr(cyc, C.c_uint32), st_ptr, flags, slots)
        res = capi.BatchResult()
        res.final_reg_digest = _ptr(out.final_reg_digest if final_digests else None, C.c_uint64)
        res.final_mem_digest = _ptr(out.final_mem_digest if final_digests else None, C.c_uint64)
        res.rolling_digest = _ptr(out.rolling_digest, C.c_uint64)
        res.cycle_digest = _ptr(out.cycle_digest, C.c_uint64)
        res.cycle_stride = stride
        res.stop_cycle = _ptr(out.stop_cycle, C.c_uint32)
        res.final_regs = _ptr(out.final_regs, C.c_uint8)
        res.final_mems = _ptr(out.final_mems, C.c_uint8)
        check(lib().tgs_batch_run(self._h, C.byref(job), C.byref(res)))
        out.device_ms = res.device_ms
        out.stream_cycles = res.stream_cycles
        out.launches = res.launches
        return out


@dataclass
class StimulusSpec:
    """Primary inputs rewritten before every cycle (see tgs_stimulus)."""

    base_seed: int
    reg: np.ndarray
    bits: np.ndarray
    toggle: np.ndarray | None = None
    table: np.ndarray | None = None  # [cycle][input][stream] nibbles (replaces the seeded values)

    def to_c(self):
        reg = np.ascontiguousarray(self.reg, np.uint32)
        bits = np.ascontiguousarray(self.bits, np.uint8)
        tog = None if self.toggle is None else np.ascontiguousarray(self.toggle, np.uint16)
        tab = None if self.table is None else self.table
        if tab is not None and not (tab.flags.c_contiguous and tab.dtype == np.uint8):
            raise ValueError("stimulus table must be a C-contiguous uint8 array")
        s = capi.Stimulus(self.base_seed, reg.size, _ptr(reg, C.c_uint32), _ptr(bits, C.c_uint8), _ptr(tog, C.c_uint16),
                          _ptr(tab, C.c_uint8))
        return (s, reg, bits, tog, tab)


@dataclass
class BatchOutput:
    n: int
    final_reg_digest: np.ndarray = field(init=False)
    final_mem_digest: np.ndarray = field(init=False)
    rolling_digest: np.ndarray = field(init=False)
    stop_cycle: np.ndarray = field(init=False)
    cycle_digest: np.ndarray | None = None
    final_regs: np.ndarray | None = None
    final_mems: np.ndarray | None = None
    device_ms: float = 0.0
    stream_cycles: int = 0
    launches: int = 0

    def __post_init__(self):
        self.final_reg_digest = np.zeros(self.n, np.uint64)
        self.final_mem_digest = np.zeros(self.n, np.uint64)
        self.rolling_digest = np.zeros(self.n, np.uint64)
        self.stop_cycle = np.zeros(self.n, np.uint32)


# ---- synthetic designs ---------------------------------------------------------
def gen_config(**kw) -> capi.GenConfig:
    c = capi.GenConfig()
    check(lib().tgs_default_gen_config(C.byref(c)))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise TypeError(f"unknown generator field {k}")
        setattr(c, k, v)
    return c


def generate(design_path: str | Path, symbol_path: str | Path, **kw) -> dict:
    """Writes a seeded synthetic design (reference file format)."""
    c = gen_config(**kw)
    info = capi.GenInfo()
    check(lib().tgs_generate(C.byref(c), str(design_path).encode(), str(symbol_path).encode(), C.byref(info)))
    d = {f: getattr(info, f) for f, _ in capi.GenInfo._fields_ if f != "reserved"}
    ids = np.zeros(info.n_pi_nibbles, np.uint32)
    bits = np.zeros(info.n_pi_nibbles, np.uint8)
    check(lib().tgs_gen_inputs(C.byref(c), _ptr(ids, C.c_uint32), _ptr(bits, C.c_uint8), info.n_pi_nibbles))
    d["pi_ids"] = ids
    d["pi_bits"] = bits
    return d


def validate_file(design_path, symbol_path=None) -> int:
    n = C.c_uint64()
    sym = str(symbol_path).encode() if symbol_path else None
    check(lib().tgs_validate_file(str(design_path).encode(), sym, C.byref(n)))
    return n.value


# ---- seeded stimulus on the host ------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def repack_design(design_path, out_path, lane_packing: int = 0, fast_luts: int = 0) -> dict:
    """The design as tgs_init rewrites it, as a file (tgs_repack_design);
    returns the micro-partition and LUT-op counts."""
    st = capi.RepackStats()
    check(lib().tgs_repack_design(str(design_path).encode(), str(out_path).encode(), lane_packing, fast_luts,
                                  C.byref(st)))
    return {f: getattr(st, f) for f, _ in capi.RepackStats._fields_ if f != "reserved"}


def plan_schedule(design_path, warps: int = 6, groups: int = 4, mpart_lanes: int = 0, levels_per_barrier: int = 0,
                  lane_packing: int = 0, fast_luts: int = 0, n_streams: int = 64) -> dict:
    """The exec-level schedule tgs_init would build, computed on the host
    (tgs_plan_schedule): level blocks, barriers, fused levels, and the plan's
    makespan with its bounds (gate counts)."""
    st = capi.ScheduleStats()
    check(lib().tgs_plan_schedule(str(design_path).encode(), warps, groups, mpart_lanes, levels_per_barrier,
                                  lane_packing, fast_luts, n_streams, C.byref(st)))
    return {f: getattr(st, f) for f, _ in capi.ScheduleStats._fields_ if not f.startswith("reserved")}


def device_reset(device: int = 0) -> None:
    """Releases everything the library holds on the device (tgs_device_reset):
    destroy every Simulator on it first."""
    check(lib().tgs_device_reset(device))


def mix64(z: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (Steele, Lea, Flood), vectorised over uint64."""
    with np.errstate(over="ignore"):
        z = (z + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def symbol_registers(symbol_path) -> dict:
    """regDebugInfo of a symbol file: name -> [(register nibble id, width)],
    most significant nibble first."""
    return _symbol_maps(symbol_path)[0]


def symbol_signals(symbol_path) -> dict:
    """signalDebugInfo of a symbol file: name -> [(partition, slot, width)],
    most significant section first."""
    return _symbol_maps(symbol_path)[1]


def _symbol_maps(symbol_path):
    """Register and signal maps of a symbol file (host-side reader of the
    reference's symbol format: three maps of u64 count, then per entry a
    u64-length string, a u64 tuple count and u32 tuples)."""
    import struct

    b = Path(symbol_path).read_bytes()
    at = 0

    def u64():
        nonlocal at
        v = struct.unpack_from("<Q", b, at)[0]
        at += 8
        return v

    def read_map(arity):
        nonlocal at
        out = {}
        for _ in range(u64()):
            n = u64()
            key = b[at:at + n].decode()
            at += n
            k = u64()
            vals = struct.unpack_from("<%dI" % (k * arity), b, at)
            at += 4 * k * arity
            out[key] = [tuple(vals[i:i + arity]) for i in range(0, len(vals), arity)]
        return out

    regs = read_map(2)
    return regs, read_map(3)


def stimulus_table(spec: StimulusSpec, n_streams: int, c0: int, cycles: int, out: np.ndarray | None = None,
                   prev: np.ndarray | None = None) -> np.ndarray:
    """The seeded input values of cycles [c0, c0 + cycles) as a host table
    [cycle][input][stream] of nibble values, identical to what the device
    computes from the seed.  Toggle inputs flip the previous value: `prev`
    [input][stream] holds the values before cycle c0 (the initial register
    nibbles for c0 = 0, else the last row of the previous table)."""
    n_in = len(spec.reg)
    tog = None
    if spec.toggle is not None and np.any(spec.toggle):
        if prev is None:
            raise ValueError("toggle inputs need the values before cycle c0 (prev)")
        tog = np.asarray(spec.toggle, np.uint64)
        cur = np.array(prev, np.uint8).reshape(n_in, n_streams).copy()
    seeds = mix64(np.uint64(spec.base_seed) ^ np.arange(n_streams, dtype=np.uint64))
    masks = ((np.uint32(1) << np.asarray(spec.bits, np.uint32)) - 1).astype(np.uint64)
    if out is None:
        out = np.empty((cycles, n_in, n_streams), np.uint8)
    inp = np.arange(n_in, dtype=np.uint64)
    for c in range(cycles):
        key = mix64((np.uint64(c0 + c) << np.uint64(32)) | inp)           # [n_in]
        h = mix64(seeds[None, :] ^ key[:, None])                          # [n_in, n_streams]
        uni = (h & masks[:, None]).astype(np.uint8)
        if tog is None:
            out[c] = uni
        else:
            flip = (h >> np.uint64(48)) < tog[:, None]
            toggled = np.where(flip, cur ^ masks[:, None].astype(np.uint8), cur)
            cur = np.where(tog[:, None] == 0, uni, toggled).astype(np.uint8)
            out[c] = cur
    return out


class PinnedBuffer:
    """Page-locked host buffer from tgs_host_alloc, viewed as a numpy array."""

    def __init__(self, shape, dtype=np.uint8):
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._p = C.c_void_p()
        check(lib().tgs_host_alloc(n, C.byref(self._p)))
        buf = (C.c_uint8 * n).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            lib().tgs_host_free(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---- learned cost model ------------------------------------------------------------
def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def mlp_forward(params: np.ndarray, X: np.ndarray) -> np.ndarray:
    """The cost model's forward kernel on host arrays (standardised output)."""
    p, x = _f32(params), _f32(X)
    out = np.zeros(x.shape[0], np.float32)
    check(lib().tgs_mlp_forward(_ptr(p, C.c_float), _ptr(x, C.c_float), x.shape[0], _ptr(out, C.c_float)))
    return out


def mlp_grad(params: np.ndarray, X: np.ndarray, y: np.ndarray) -> tuple[np.ndarray, float]:
    """Gradient of the mean squared error computed by the backward kernel."""
    p, x, t = _f32(params), _f32(X), _f32(y)
    g = np.zeros(capi.MLP_PARAMS, np.float32)
    loss = C.c_float()
    check(lib().tgs_mlp_grad(_ptr(p, C.c_float), _ptr(x, C.c_float), _ptr(t, C.c_float), x.shape[0],
                             _ptr(g, C.c_float), C.byref(loss)))
    return g, loss.value


def _sim_learned_methods():
    def n_mparts(self) -> int:
        n = C.c_uint32()
        check(lib().tgs_num_mparts(self._h, C.byref(n)))
        return n.value

    def mpart_features(self) -> np.ndarray:
        n = self.n_mparts()
        x = np.zeros((n, 16), np.float32)
        check(lib().tgs_mpart_features(self._h, _ptr(x, C.c_float), n))
        return x

    def profile_mparts(self, cycles: int) -> np.ndarray:
        n = self.n_mparts()
        c = np.zeros(n, np.float32)
        check(lib().tgs_profile_mparts(self._h, int(cycles), _ptr(c, C.c_float), n))
        return c

    def train_cost_model(self, features, cycles, *, epochs=30, batch=1024, lr=2e-3, seed=1, val_frac=0.2) -> dict:
        x, c = _f32(features), _f32(cycles)
        o = capi.TrainOpts(epochs, batch, lr, seed, val_frac)
        r = capi.TrainReport()
        check(lib().tgs_cost_model_train(self._h, _ptr(x, C.c_float), _ptr(c, C.c_float), x.shape[0], C.byref(o),
                                         C.byref(r)))
        return {f: getattr(r, f) for f, _ in capi.TrainReport._fields_ if f != "reserved"}

    def cost_model_state(self) -> np.ndarray:
        s = np.zeros(capi.MLP_PARAMS + 2, np.float32)
        check(lib().tgs_cost_model_state(self._h, _ptr(s, C.c_float), s.size, 0))
        return s

    def set_cost_model_state(self, state) -> None:
        s = _f32(state)
        check(lib().tgs_cost_model_state(self._h, _ptr(s, C.c_float), s.size, 1))

    for f in (n_mparts, mpart_features, profile_mparts, train_cost_model, cost_model_state, set_cost_model_state):
        setattr(Simulator, f.__name__, f)


_sim_learned_methods()
