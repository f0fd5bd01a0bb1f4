"""Hand-built designs in the reference's design/symbol file format.

Test infrastructure: the known-answer tests build tiny designs op by op.
Record layouts follow include/ToucanGPUGenDataTypes.h (struct sizes and
field offsets of the reference, padding bytes written as zero) and the
stream grammar of the reference Serializer (src/Serializer.cpp:106-300).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

LUT_SIZE = 4642


def u64(v):
    return struct.pack("<Q", v)


def vec(records: list[bytes]) -> bytes:
    return u64(len(records)) + b"".join(records)


def top(lut, a, b, c):
    return struct.pack("<HHHH", lut, a, b, c)


def mid(lut, a, b, c):
    return struct.pack("<I", (lut << 18) | (a << 12) | (b << 6) | c)


def wb(src, result):
    return struct.pack("<BxH", src, result)


def vec_read(base, length, offset, is_const, idx, out_range, result):
    return struct.pack("<HHH?xHHHHHH", base, length, offset, is_const, *idx, out_range, result)


def vec_op(v1, v2, length, op, cflags, result):
    return struct.pack("<HHHBBH", v1, v2, length, op, cflags, result)


def mem_read(multi, base, en, addr, result):
    return struct.pack("<?7xQHHH2x", multi, base, en, addr, result)


def mem_write(multi, base, addr, dat, en):
    return struct.pack("<?7xQHHH2x", multi, base, addr, dat, en)


def reg_read(reg, result):
    return struct.pack("<IH2x", reg, result)


def copy_op(dst, dat, count):
    return struct.pack("<IHH", dst, dat, count)


@dataclass
class MPart:
    is_lut: bool = True
    top: list = field(default_factory=list)      # bytes from top()
    mids: list = field(default_factory=list)     # list of lists of mid()
    wbs: list = field(default_factory=list)
    vec_reads: list = field(default_factory=list)
    vec_ops: list = field(default_factory=list)
    mem_reads: list = field(default_factory=list)

    def bytes(self) -> bytes:
        if self.is_lut:
            out = b"\x01" + vec(self.top) + u64(len(self.mids))
            for m in self.mids:
                out += vec(m)
            return out + vec(self.wbs)
        return b"\x00" + vec(self.vec_reads) + vec(self.vec_ops) + vec(self.mem_reads)


@dataclass
class Part:
    vp_size: int = 64
    const_vec: bytes = b""
    reg_reads: list = field(default_factory=list)   # (reg, slot)
    exg_reads: list = field(default_factory=list)   # (exchange, slot)
    levels: list = field(default_factory=list)      # list of lists of MPart
    reg_write: tuple = (0, 0, 0)                    # (reg, dat, count)
    mem_writes: list = field(default_factory=list)  # bytes from mem_write()
    prints: list = field(default_factory=list)      # (en, msg)
    stops: list = field(default_factory=list)       # en
    exg_write: tuple = (0, 0, 0)                    # (exchange, dat, count)

    def bytes(self) -> bytes:
        out = vec([]) + struct.pack("<I", self.vp_size) + u64(len(self.const_vec)) + self.const_vec
        out += vec([reg_read(r, s) for r, s in self.reg_reads])
        out += vec([reg_read(e, s) for e, s in self.exg_reads])
        out += u64(len(self.levels))
        for lvl in self.levels:
            out += u64(len(lvl)) + b"".join(m.bytes() for m in lvl)
        out += copy_op(*self.reg_write)
        out += vec(self.mem_writes)
        out += vec([struct.pack("<HH", e, m) for e, m in self.prints])
        out += vec([struct.pack("<H", e) for e in self.stops])
        out += copy_op(*self.exg_write)
        return out


@dataclass
class Design:
    reg_pool: int
    mem_pool: int
    exg_pool: int
    lut: bytes = bytes(LUT_SIZE)
    parts: list = field(default_factory=list)
    regions: list = field(default_factory=lambda: [[], []])
    msgs: list = field(default_factory=list)
    reg_init: bytes = b""   # initial regPool contents (Init() keeps them, SimInit.cpp:16-26)
    mem_init: bytes = b""

    def bytes(self) -> bytes:
        out = struct.pack("<III?", self.reg_pool, self.mem_pool, self.exg_pool, False)
        out += u64(len(self.lut)) + bytes(self.lut)
        out += u64(len(self.reg_init)) + bytes(self.reg_init) + u64(len(self.mem_init)) + bytes(self.mem_init)
        out += u64(len(self.parts)) + b"".join(p.bytes() for p in self.parts)
        out += u64(len(self.regions))
        for r in self.regions:
            out += u64(len(r)) + b"".join(struct.pack("<I", i) for i in r)
        out += u64(len(self.msgs))
        for m in self.msgs:
            b = m.encode()
            out += u64(len(b)) + b
        return out

    def write(self, path):
        with open(path, "wb") as f:
            f.write(self.bytes())


def symbols(regs: dict | None = None, signals: dict | None = None, mems: dict | None = None) -> bytes:
    """regs: name -> [(id, width)...] (most significant first); mems: name -> [(start, bits, depth)]."""
    out = b""
    for m, arity in ((regs or {}, 2), (signals or {}, 3), (mems or {}, 3)):
        out += u64(len(m))
        for name, locs in m.items():
            nb = name.encode()
            out += u64(len(nb)) + nb + u64(len(locs))
            for t in locs:
                out += struct.pack("<" + "I" * arity, *t)
    return out


def write_symbols(path, **kw):
    with open(path, "wb") as f:
        f.write(symbols(**kw))
