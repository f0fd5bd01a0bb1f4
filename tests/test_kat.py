"""Known-answer tests, one per op kind of the reference evaluator.

Each case is a hand-built two-partition design: partition 0 (region 0) reads
input registers 0..15 into slots 16..31, runs the case's micro-partitions
and copies 32 output slots [64, 96) to the exchange pool; partition 1
(region 1) copies them into registers 16..47.  The expected outputs are
derived by hand from the reference source line named in each case, not from
the oracle.  The same designs run on the oracle (CPU) and, marked gpu, on the
GB300 kernels.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import designlib as dl

OUT = 64  # first output slot
IN = 16   # first input slot (register i -> slot 16 + i)


def zero_outputs():
    """Exec level writing immediate 0 to all 32 output slots (write-back
    shuffleId < 32 is an immediate, SimEval.cu:439-442)."""
    return [dl.MPart(top=[], wbs=[dl.wb(0, OUT + i) for i in range(32)])]


def frame(levels, lut=None, mem_pool=4, const_vec=b"", mem_writes=(), prints=(), stops=(), msgs=(),
          p0_reg_write=(0, 0, 0), reg_pool=64):
    p0 = dl.Part(vp_size=160, const_vec=const_vec, reg_reads=[(i, IN + i) for i in range(16)],
                 levels=[zero_outputs()] + levels, exg_write=(0, OUT, 32), reg_write=p0_reg_write)
    p1 = dl.Part(vp_size=64, exg_reads=[(i, 16 + i) for i in range(32)], levels=[], reg_write=(16, 16, 32),
                 mem_writes=list(mem_writes), prints=list(prints), stops=list(stops))
    d = dl.Design(reg_pool=reg_pool, mem_pool=mem_pool, exg_pool=32, lut=lut if lut is not None else bytes(dl.LUT_SIZE),
                  parts=[p0, p1], regions=[[0], [1]], msgs=list(msgs))
    return d


def table(base, fn, rows=16):
    """4642-entry table with fn(a, b, c) at base + (a << 8 | b << 4 | c)."""
    t = bytearray(dl.LUT_SIZE)
    for a in range(rows):
        for b in range(16):
            for c in range(16):
                idx = base + ((a << 8) | (b << 4) | c)
                if idx < dl.LUT_SIZE:
                    t[idx] = fn(a, b, c) & 0xF
    return bytes(t)


# ---- cases: (design, input regs 0..15, expected regs 16..47 or None, extra) --------
def case_top_lookup():
    # SimEval.cu:345-356: operands < 16 immediate, else slot; index lutIndex + (a<<8|b<<4|c)
    lut = table(100, lambda a, b, c: a * 3 + b * 5 + c * 7, rows=16)
    lanes = [dl.top(100, IN + 0, IN + 1, IN + 2), dl.top(100, 3, IN + 1, 9), dl.top(100, 0, 0, IN + 15)]
    m = dl.MPart(top=lanes, wbs=[dl.wb(32 + i, OUT + i) for i in range(3)])
    regs = np.arange(16, dtype=np.uint8)[::-1].copy()  # 15, 14, ..., 0
    exp = np.zeros(32, np.uint8)
    f = lambda a, b, c: (a * 3 + b * 5 + c * 7) & 0xF  # noqa: E731
    exp[0] = f(15, 14, 13)
    exp[1] = f(3, 14, 9)
    exp[2] = f(0, 0, 0)
    return frame([[m]], lut=lut), regs, exp


def case_nop_moves():
    # SimEval.cu:350-352 (top) and 407-408 (middle): lutIndex 0 passes op2
    m = dl.MPart(top=[dl.top(0, 5, 6, IN + 4), dl.top(0, IN + 1, IN + 2, 11)],
                 mids=[[dl.mid(0, 0, 0, 33), dl.mid(0, 0, 0, 32), dl.mid(0, 0, 0, 7)]],
                 wbs=[dl.wb(32, OUT), dl.wb(33, OUT + 1), dl.wb(34, OUT + 2)])
    regs = np.array([1, 2, 3, 4, 9, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 0], np.uint8)
    exp = np.zeros(32, np.uint8)
    exp[0], exp[1], exp[2] = 11, 9, 7  # lane0 <- prev lane1 (11), lane1 <- prev lane0 (reg4 = 9), lane2 <- imm 7
    return frame([[m]]), regs, exp


def case_middle_operands():
    # SimEval.cu:377-404: operand < 32 immediate, 32..63 lane (op - 32); lanes
    # beyond the previous level (and idle lanes) carry 0; idle lanes compute 0.
    lut = table(200, lambda a, b, c: (a ^ (b << 1) ^ (c << 2)), rows=16)
    m = dl.MPart(top=[dl.top(0, 0, 0, IN + 3), dl.top(0, 0, 0, IN + 7)],  # lane0 = r3, lane1 = r7
                 mids=[[dl.mid(200, 32, 33, 5), dl.mid(200, 34, 45, 33), dl.mid(200, 1, 2, 3)],
                       [dl.mid(0, 0, 0, 34), dl.mid(0, 0, 0, 33), dl.mid(0, 0, 0, 32), dl.mid(0, 0, 0, 40)]],
                 wbs=[dl.wb(32, OUT), dl.wb(33, OUT + 1), dl.wb(34, OUT + 2), dl.wb(35, OUT + 3)])
    regs = np.zeros(16, np.uint8)
    regs[3], regs[7] = 6, 13
    f = lambda a, b, c: (a ^ (b << 1) ^ (c << 2)) & 0xF  # noqa: E731
    l0 = f(6, 13, 5)
    l1 = f(0, 0, 13)  # lane 34 -> lane 2 of the top level: idle (0); lane 45 -> lane 13: idle (0)
    l2 = f(1, 2, 3)
    exp = np.zeros(32, np.uint8)
    exp[0], exp[1], exp[2], exp[3] = l2, l1, l0, 0  # second middle level permutes; lane 8 of previous is idle
    return frame([[m]], lut=lut), regs, exp


def case_writeback_immediates():
    # SimEval.cu:436-442: shuffleId < 32 writes the immediate itself; >= 32 reads lane id & 31
    m = dl.MPart(top=[dl.top(0, 0, 0, IN + 9)], wbs=[dl.wb(7, OUT), dl.wb(32, OUT + 1), dl.wb(15, OUT + 2), dl.wb(96, OUT + 3)])
    regs = np.zeros(16, np.uint8)
    regs[9] = 12
    exp = np.zeros(32, np.uint8)
    exp[0], exp[1], exp[2], exp[3] = 7, 12, 15, 12  # 96 mod 32 = lane 0
    return frame([[m]]), regs, exp


def case_vec_read():
    # SimEval.cu:449-480: index nibbles (most significant first) + static
    # offset; in range reads the vector (slots or constVecPool), else outRange
    const = bytes([3, 1, 4, 1, 5, 9, 2, 6])
    ops = [
        dl.vec_read(IN + 8, 8, 1, False, (0, 0, 0, IN + 0), 5, OUT),           # idx r0=2 +1 -> slot 16+8+3 = r11
        dl.vec_read(IN + 8, 8, 0, False, (0, 0, IN + 1, IN + 0), 5, OUT + 1),   # idx (r1<<4|r0) = 0x12 = 18 >= 8 -> imm 5
        dl.vec_read(0, 8, 2, True, (0, 0, 0, IN + 0), IN + 2, OUT + 2),         # const[2 + 2] = 5
        dl.vec_read(0, 8, 7, True, (0, 0, 0, IN + 0), IN + 2, OUT + 3),         # 2 + 7 = 9 >= 8 -> slot r2 = 7
    ]
    m = dl.MPart(is_lut=False, vec_reads=ops)
    regs = np.array([2, 1, 7, 0, 0, 0, 0, 0, 10, 11, 12, 13, 14, 15, 8, 9], np.uint8)
    exp = np.zeros(32, np.uint8)
    exp[0], exp[1], exp[2], exp[3] = 13, 5, 5, 7
    return frame([[m]], const_vec=const), regs, exp


def case_vec_arith():
    # SimEval.cu:482-548: vector nibbles least significant first at the base
    # slot, sign-extended at bit 4*len-1; ADD/SUB/MUL store len nibbles,
    # EQ/LT/LE store 0/1 (signed comparison).
    a = 0x3F  # slots 16,17 = 0xF, 0x3 (2 nibbles): +63 as 8-bit signed
    b = 0xC1  # slots 18,19 = 0x1, 0xC: -63 as 8-bit signed
    regs = np.zeros(16, np.uint8)
    regs[0], regs[1], regs[2], regs[3] = a & 0xF, a >> 4, b & 0xF, b >> 4
    ops = [
        dl.vec_op(IN + 0, IN + 2, 2, 0, 0, OUT + 0),   # ADD -> 0x00
        dl.vec_op(IN + 0, IN + 2, 2, 1, 0, OUT + 2),   # SUB -> 63 - (-63) = 126 = 0x7E
        dl.vec_op(IN + 0, IN + 2, 2, 2, 0, OUT + 4),   # MUL -> -3969 mod 256 = 0x7F
        dl.vec_op(IN + 0, IN + 2, 2, 3, 0, OUT + 6),   # EQ -> 0
        dl.vec_op(IN + 2, IN + 0, 2, 4, 0, OUT + 7),   # LT: -63 < 63 -> 1
        dl.vec_op(IN + 0, IN + 2, 2, 5, 0, OUT + 8),   # LE: 63 <= -63 -> 0
        dl.vec_op(IN + 0, 0, 2, 3, 1, OUT + 9),        # EQ with const vector [0xF, 0x3] -> 1
        dl.vec_op(IN + 0, IN + 2, 2, 7, 0, OUT + 10),  # unknown op -> 0
    ]
    m = dl.MPart(is_lut=False, vec_ops=ops)
    exp = np.zeros(32, np.uint8)
    exp[0:2] = [0x0, 0x0]
    exp[2:4] = [0xE, 0x7]
    exp[4:6] = [0xF, 0x7]
    exp[6], exp[7], exp[8], exp[9], exp[10] = 0, 1, 0, 1, 0
    return frame([[m]], const_vec=bytes([0xF, 0x3])), regs, exp


def case_mem_read():
    # SimEval.cu:550-575: 8 address nibbles least significant first; multiple
    # writers shift the address by 2; en == 0 leaves the slot untouched
    mem = 64
    addr_level = [dl.MPart(top=[dl.top(0, 0, 0, IN + i) for i in range(8)], wbs=[dl.wb(32 + i, 120 + i) for i in range(8)])]
    preset = [dl.MPart(top=[dl.top(0, 0, 0, 9)], wbs=[dl.wb(32, OUT + 2)])]
    reads = dl.MPart(is_lut=False, mem_reads=[dl.mem_read(False, 8, 1, 120, OUT), dl.mem_read(True, 1, 1, 120, OUT + 1),
                                               dl.mem_read(False, 8, 0, 120, OUT + 2)])
    regs = np.zeros(16, np.uint8)
    regs[0] = 3  # address 3: plain reads memPool[8 + 3], multi-writer reads memPool[1 + (3 << 2)]
    d = frame([addr_level + preset, [reads]], mem_pool=mem)
    init = np.arange(mem, dtype=np.uint8) % 16
    exp = np.zeros(32, np.uint8)
    exp[0] = init[8 + 3]
    exp[1] = init[1 + (3 << 2)]
    exp[2] = 9
    return d, regs, exp, init


def case_reg_copy_rounding():
    # SimEval.cu:658-665: (count + 3) / 4 words from (dat & ~3) to (reg & ~3)
    p0 = dl.Part(vp_size=128, reg_reads=[(i, IN + i) for i in range(16)], levels=[zero_outputs()],
                 exg_write=(0, OUT, 32))
    p1 = dl.Part(vp_size=96, exg_reads=[(i, 16 + i) for i in range(32)],
                 levels=[[dl.MPart(top=[dl.top(0, 0, 0, 16 + i) for i in range(8)], wbs=[dl.wb(32 + i, 64 + i) for i in range(8)])]],
                 reg_write=(18, 65, 5))  # copies slots 64..71 to registers 16..23
    d = dl.Design(reg_pool=64, mem_pool=4, exg_pool=32, parts=[p0, p1], regions=[[0], [1]])
    regs = np.zeros(16, np.uint8)  # outputs zero -> exchange zero
    exp = None
    return d, regs, exp


CASES = {
    "top_lookup": case_top_lookup,
    "nop_moves": case_nop_moves,
    "middle_operands": case_middle_operands,
    "writeback_immediates": case_writeback_immediates,
    "vec_read": case_vec_read,
    "vec_arith": case_vec_arith,
    "mem_read": case_mem_read,
}


def _build(tmp_path, name):
    r = CASES[name]()
    d, regs, exp = r[0], r[1], r[2]
    init_mem = r[3] if len(r) > 3 else None
    dp = tmp_path / f"{name}.bin"
    d.write(dp)
    return dp, regs, exp, init_mem


@pytest.mark.parametrize("name", list(CASES))
def test_kat_oracle(tmp_path, built, name):
    from oracle import pyoracle

    dp, regs, exp, init_mem = _build(tmp_path, name)
    od = pyoracle.OracleDesign(dp)
    st = pyoracle.OracleState(od)
    st.regs()[:16] = regs
    if init_mem is not None:
        st.mems()[:] = init_mem
    st.eval(1)
    np.testing.assert_array_equal(st.regs()[16:48], exp)


@pytest.mark.parametrize("name", list(CASES))
def test_kat_validator_accepts(tmp_path, built, name):
    from toucangpurt_gb300 import sim

    dp, *_ = _build(tmp_path, name)
    sim.validate_file(dp)


def test_kat_reg_copy_rounding(tmp_path, built):
    """count 5 from dat 65 copies the 8 slots 64..71 to registers 16..23."""
    from oracle import pyoracle

    d, regs, _ = case_reg_copy_rounding()
    dp = tmp_path / "copy.bin"
    d.write(dp)
    od = pyoracle.OracleDesign(dp)
    st = pyoracle.OracleState(od)
    r = st.regs()
    r[:] = 0
    r[16:24] = 5  # all 8 rewritten although count is 5
    r[24:32] = 7  # beyond the copied words: untouched
    st.eval(1)
    # exchange slots 16..23 hold partition 0's zero outputs; copied to regs 16..23
    np.testing.assert_array_equal(st.regs()[16:24], np.zeros(8, np.uint8))
    np.testing.assert_array_equal(st.regs()[24:32], np.full(8, 7, np.uint8))


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_kat_gpu(tmp_path, built, name):
    from toucangpurt_gb300 import sim

    dp, regs, exp, init_mem = _build(tmp_path, name)
    for streams in (1, 8):
        with sim.Simulator(n_streams=streams) as s:
            s.init(0, dp, None, False, False)
            for k in range(streams):
                pool = s.reg_pool(k)
                pool[:16] = regs
                s.write_reg_pool(pool, k)
                if init_mem is not None:
                    s.write_mem_pool(init_mem, k)
            s.eval()
            for k in range(streams):
                np.testing.assert_array_equal(s.reg_pool(k)[16:48], exp, err_msg=f"{name} stream {k}")


def case_mem_write():
    """SimEval.cu:670-693: region-1 memory writes; dat < 16 is an immediate;
    multiple writers shift the address by 2."""
    lvl = [dl.MPart(top=[dl.top(0, 0, 0, IN + i) for i in range(10)], wbs=[dl.wb(32 + i, OUT + i) for i in range(10)])]
    # partition 1 slots 16.. hold exchange 0.. = partition 0 outputs OUT..
    writes = [dl.mem_write(False, 0, 16, 24, 1),    # mem[0 + addr] = slot 24 (reg 8)
              dl.mem_write(True, 2, 16, 25, 1),     # mem[2 + (addr << 2)] = slot 25 (reg 9)
              dl.mem_write(False, 40, 16, 11, 1),   # mem[40 + addr] = immediate 11
              dl.mem_write(False, 50, 16, 24, 0)]   # disabled
    d = frame([lvl], mem_pool=64, mem_writes=writes)
    regs = np.zeros(16, np.uint8)
    regs[0] = 5   # address 5
    regs[8], regs[9] = 13, 6
    exp = np.zeros(64, np.uint8)
    exp[5], exp[2 + 20], exp[45] = 13, 6, 11
    return d, regs, exp


def case_stop_print():
    """SimEval.cu:696-722: print when enabled and en != 0; stop is sticky."""
    lvl = [dl.MPart(top=[dl.top(0, 0, 0, IN + i) for i in range(2)], wbs=[dl.wb(32 + i, OUT + i) for i in range(2)])]
    d = frame([lvl], prints=[(17, 0), (16, 1)], stops=[17], msgs=["stop-message\n", "never\n"])
    return d


def test_kat_mem_write_oracle(tmp_path, built):
    from oracle import pyoracle

    d, regs, exp = case_mem_write()
    dp = tmp_path / "mw.bin"
    d.write(dp)
    st = pyoracle.OracleState(pyoracle.OracleDesign(dp))
    st.regs()[:16] = regs
    st.eval(1)
    np.testing.assert_array_equal(st.mems(), exp)


def test_kat_stop_oracle(tmp_path, built):
    from oracle import pyoracle

    dp = tmp_path / "stop.bin"
    case_stop_print().write(dp)
    st = pyoracle.OracleState(pyoracle.OracleDesign(dp))
    st.regs()[:16] = 0
    assert not st.eval(1)       # slot 17 = reg 1 = 0
    st.regs()[1] = 4
    assert st.eval(1)           # fires
    st.regs()[1] = 0
    assert st.eval(1)           # sticky


@pytest.mark.gpu
def test_kat_mem_write_gpu(tmp_path, built):
    from toucangpurt_gb300 import sim

    d, regs, exp = case_mem_write()
    dp = tmp_path / "mw.bin"
    d.write(dp)
    for streams in (1, 8):
        with sim.Simulator(n_streams=streams) as s:
            s.init(0, dp, None, False, False)
            for k in range(streams):
                pool = s.reg_pool(k)
                pool[:16] = regs
                s.write_reg_pool(pool, k)
            s.eval()
            for k in range(streams):
                np.testing.assert_array_equal(s.mem_pool(k), exp)


@pytest.mark.gpu
def test_kat_stop_print_gpu(tmp_path, built, capfd):
    from toucangpurt_gb300 import sim

    dp = tmp_path / "stop.bin"
    case_stop_print().write(dp)
    with sim.Simulator() as s:
        s.init(0, dp, None, False, True)
        assert not s.eval()
        pool = s.reg_pool()
        pool[1] = 4
        s.write_reg_pool(pool)
        assert s.eval()
        pool[1] = 0
        s.write_reg_pool(pool)
        assert s.eval()
    out = capfd.readouterr().out
    assert "stop-message" in out and "never" not in out
    assert "Toucan first stop" in out


def kat_design_with_inputs(name: str) -> dl.Design:
    """The case's design with its input registers (and memory) stored as the
    initial regPool / memPool of the design file, for runs without a
    testbench (the reference kernel in the golden fixtures)."""
    if name == "mem_write":
        d, regs, _ = case_mem_write()
    elif name == "reg_copy_rounding":
        d, regs, _ = case_reg_copy_rounding()
        regs = np.zeros(16, np.uint8)
        init = np.zeros(d.reg_pool, np.uint8)
        init[16:24] = 5
        init[24:32] = 7
        d.reg_init = init.tobytes()
        return d
    elif name == "stop_print":
        d = case_stop_print()
        regs = np.zeros(16, np.uint8)
        regs[1] = 4
    else:
        r = CASES[name]()
        d, regs = r[0], r[1]
        if len(r) > 3:
            d.mem_init = np.asarray(r[3], np.uint8).tobytes()
    init = np.zeros(d.reg_pool, np.uint8)
    init[:16] = regs
    d.reg_init = init.tobytes()
    return d
