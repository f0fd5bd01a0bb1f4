"""ctypes binding of the CPU oracle (oracle/toucan_oracle.h).

TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and bench.py's
CPU-baseline leg as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_TOOL = HERE / "_ref" / "ref_tool"
REF_CUBIN = HERE / "_ref" / "ref_simeval.cubin"
_lib = None


class Stim(C.Structure):
    _fields_ = [("base_seed", C.c_uint64), ("n_inputs", C.c_uint32), ("reg", C.POINTER(C.c_uint32)),
                ("bits", C.POINTER(C.c_uint8)), ("toggle", C.POINTER(C.c_uint16))]


class Result(C.Structure):
    _fields_ = [("final_reg_digest", C.POINTER(C.c_uint64)), ("final_mem_digest", C.POINTER(C.c_uint64)),
                ("rolling_digest", C.POINTER(C.c_uint64)), ("cycle_digest", C.POINTER(C.c_uint64)),
                ("cycle_stride", C.c_uint32), ("stop_cycle", C.POINTER(C.c_uint32)),
                ("final_regs", C.POINTER(C.c_uint8)), ("final_mems", C.POINTER(C.c_uint8))]


def reference_dir() -> Path | None:
    """The reference checkout the recipe (oracle/Makefile) builds from, or
    None where it is absent."""
    r = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref-dir"], capture_output=True, text=True)
    d = Path(r.stdout.strip()) if r.returncode == 0 and r.stdout.strip() else None
    return d if d is not None and d.is_dir() else None


def build() -> None:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.orc_load.restype = C.c_void_p
        L.orc_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_size_t]
        L.orc_free.argtypes = [C.c_void_p]
        for f in ("orc_reg_pool_size", "orc_mem_pool_size", "orc_num_parts"):
            getattr(L, f).restype = C.c_uint32
            getattr(L, f).argtypes = [C.c_void_p]
        L.orc_num_lut_ops.restype = C.c_uint64
        L.orc_num_lut_ops.argtypes = [C.c_void_p]
        L.orc_initial_regs.restype = C.POINTER(C.c_uint8)
        L.orc_initial_regs.argtypes = [C.c_void_p]
        L.orc_initial_mems.restype = C.POINTER(C.c_uint8)
        L.orc_initial_mems.argtypes = [C.c_void_p]
        L.orc_run.restype = C.c_int
        L.orc_run.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(Stim), C.POINTER(Result),
                              C.c_int, C.c_char_p, C.c_size_t]
        L.orc_state_new.restype = C.c_void_p
        L.orc_state_new.argtypes = [C.c_void_p]
        L.orc_state_free.argtypes = [C.c_void_p]
        L.orc_state_eval.restype = C.c_int
        L.orc_state_eval.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_int), C.c_char_p, C.c_size_t]
        L.orc_state_set_probes.restype = C.c_int
        L.orc_state_set_probes.argtypes = [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32]
        L.orc_state_probe_values.restype = C.POINTER(C.c_uint8)
        L.orc_state_probe_values.argtypes = [C.c_void_p]
        L.orc_state_regs.restype = C.POINTER(C.c_uint8)
        L.orc_state_regs.argtypes = [C.c_void_p]
        L.orc_state_mems.restype = C.POINTER(C.c_uint8)
        L.orc_state_mems.argtypes = [C.c_void_p]
        L.orc_digest.restype = C.c_uint64
        L.orc_digest.argtypes = [C.POINTER(C.c_uint8), C.c_size_t]
        L.orc_mix64.restype = C.c_uint64
        L.orc_mix64.argtypes = [C.c_uint64]
        _lib = L
    return _lib


def _p(a, t):
    return C.cast(None, C.POINTER(t)) if a is None else a.ctypes.data_as(C.POINTER(t))


def digest(pool: np.ndarray) -> int:
    a = np.ascontiguousarray(pool, np.uint8)
    return int(lib().orc_digest(_p(a, C.c_uint8), a.size))


class OracleDesign:
    def __init__(self, design, symbols=None, randomize=False):
        err = C.create_string_buffer(512)
        sym = str(symbols).encode() if symbols else None
        self._d = lib().orc_load(str(design).encode(), sym, int(randomize), err, 512)
        if not self._d:
            raise RuntimeError(f"oracle load failed: {err.value.decode()}")
        self.reg_pool = lib().orc_reg_pool_size(self._d)
        self.mem_pool = lib().orc_mem_pool_size(self._d)
        self.n_parts = lib().orc_num_parts(self._d)
        self.lut_ops = lib().orc_num_lut_ops(self._d)

    def __del__(self):
        if getattr(self, "_d", None):
            lib().orc_free(self._d)
            self._d = None

    def initial_regs(self) -> np.ndarray:
        return np.ctypeslib.as_array(lib().orc_initial_regs(self._d), (self.reg_pool,)).copy()

    def initial_mems(self) -> np.ndarray:
        if self.mem_pool == 0:
            return np.zeros(0, np.uint8)
        return np.ctypeslib.as_array(lib().orc_initial_mems(self._d), (self.mem_pool,)).copy()

    def run(self, cycles, stim=None, *, threads=0, cycle_digests=False, final_state=False, final_digests=True):
        """final_digests=False skips the final register and memory digests
        (the memory digest reads every stream's whole pool)."""
        cyc = np.ascontiguousarray(cycles, np.uint32)
        n = cyc.size
        out = {k: np.zeros(n, np.uint64) for k in ("final_reg_digest", "final_mem_digest", "rolling_digest")}
        out["stop_cycle"] = np.zeros(n, np.uint32)
        stride = int(cyc.max()) if cycle_digests else 0
        if cycle_digests:
            out["cycle_digest"] = np.zeros((n, stride), np.uint64)
        if final_state:
            out["final_regs"] = np.zeros((n, self.reg_pool), np.uint8)
            out["final_mems"] = np.zeros((n, max(1, self.mem_pool)), np.uint8)
        fin = (lambda a: _p(a, C.c_uint64)) if final_digests else (lambda a: _p(None, C.c_uint64))
        res = Result(fin(out["final_reg_digest"]), fin(out["final_mem_digest"]),
                     _p(out["rolling_digest"], C.c_uint64), _p(out.get("cycle_digest"), C.c_uint64), stride,
                     _p(out["stop_cycle"], C.c_uint32), _p(out.get("final_regs"), C.c_uint8),
                     _p(out.get("final_mems"), C.c_uint8))
        keep = []
        sp = C.cast(None, C.POINTER(Stim))
        if stim is not None:
            reg = np.ascontiguousarray(stim.reg, np.uint32)
            bits = np.ascontiguousarray(stim.bits, np.uint8)
            tog = None if stim.toggle is None else np.ascontiguousarray(stim.toggle, np.uint16)
            keep += [reg, bits, tog]
            s = Stim(stim.base_seed, reg.size, _p(reg, C.c_uint32), _p(bits, C.c_uint8), _p(tog, C.c_uint16))
            keep.append(s)
            sp = C.pointer(s)
        err = C.create_string_buffer(512)
        rc = lib().orc_run(self._d, n, _p(cyc, C.c_uint32), sp, C.byref(res), threads, err, 512)
        if rc != 0:
            raise RuntimeError(f"oracle run failed: {err.value.decode()}")
        return out


class OracleState:
    """Single-stream stepping (the reference's eval() flow)."""

    def __init__(self, design: OracleDesign):
        self.d = design
        self._s = lib().orc_state_new(design._d)

    def __del__(self):
        if getattr(self, "_s", None):
            lib().orc_state_free(self._s)
            self._s = None

    def eval(self, cycles=1) -> bool:
        stop = C.c_int()
        err = C.create_string_buffer(512)
        if lib().orc_state_eval(self._s, cycles, C.byref(stop), err, 512) != 0:
            raise RuntimeError(err.value.decode())
        return bool(stop.value)

    def set_probes(self, parts, slots) -> None:
        """Record value-pool slot slots[i] of partition parts[i] every cycle."""
        self._np = len(parts)
        pa = np.ascontiguousarray(parts, np.uint32)
        sl = np.ascontiguousarray(slots, np.uint32)
        if lib().orc_state_set_probes(self._s, pa.ctypes.data_as(C.POINTER(C.c_uint32)),
                                      sl.ctypes.data_as(C.POINTER(C.c_uint32)), len(pa)) != 0:
            raise RuntimeError("probe beyond the design")

    def probe_values(self) -> np.ndarray:
        return np.ctypeslib.as_array(lib().orc_state_probe_values(self._s), (self._np,)).copy()

    def signal(self, sections) -> int:
        """Value of a signal given as (partition, slot, width) sections, most
        significant section first, from the probes set for exactly these
        sections in this order."""
        v = 0
        vals = self.probe_values()
        for (_, _, w), x in zip(sections, vals):
            v = (v << w) | (int(x) & ((1 << w) - 1))
        return v

    def regs(self) -> np.ndarray:
        return np.ctypeslib.as_array(lib().orc_state_regs(self._s), (self.d.reg_pool,))

    def mems(self) -> np.ndarray:
        if self.d.mem_pool == 0:
            return np.zeros(0, np.uint8)
        return np.ctypeslib.as_array(lib().orc_state_mems(self._s), (self.d.mem_pool,))
