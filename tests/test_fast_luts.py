"""Word-wide evaluation of palette LUT ops and the regrouping of single-level
micro-partitions by kind (tgs_options.fast_luts, csrc/emit.cpp FastLuts /
regroupLevel, csrc/cycle_kernel.cuh fastTop).

A LUT op reads table entry lutIndex + (a << 8 | b << 4 | c)
(src/SimEval.cu:350-356).  Rows that are a bitwise function of (b, c), and
4,096-entry windows whose rows a = 0 / a = 1 pass c / b (multiplexers), are
recognised at load time and computed word-wide; everything else, and a
multiplexer word whose select nibbles are not all 0 or 1, reads the table.

* Known answers: a hand-built design with AND, OR, XOR and NAND rows, a row
  that differs from AND in one entry (must read the table), a window whose
  row 1 is AND and row 0 is not (the op0 immediate picks the row), a
  multiplexer and a reversed one (select nibbles 0/1 in some stream words,
  above 1 in others), a random window and a move.  Expected values are the
  table entries the reference reads, computed here from the table bytes.
* The regrouped design (tgs_repack_design) is an ordinary design file: the
  CPU oracle checks it against the original on generated palette designs and
  against the reference kernel's golden fixtures.
* On the GPU, the word-wide path runs against the oracle per stream.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle
from tests import designlib as dl
from tests.test_golden import EVAL, _h, _ids, _stim
from tests.test_kat import IN, OUT, frame
from toucangpurt_gb300 import capi, sim, workloads

G = Path(__file__).parent / "golden"

MUX, MUXI = 1, 513          # 4,096-entry windows: rows a = 0, 1 pass c, b (MUX) / b, c (MUXI)
AND, OR, XOR, NAND, NEAR, ROWSEL, RAND = 1100, 1400, 1700, 2000, 2300, 2600, 3200


def fast_table() -> bytes:
    rng = np.random.default_rng(5)
    t = bytearray(rng.integers(0, 16, dl.LUT_SIZE, dtype=np.uint8).tobytes())
    for b in range(16):
        for c in range(16):
            i = (b << 4) | c
            t[MUX + i], t[MUX + 256 + i] = c, b
            t[MUXI + i], t[MUXI + 256 + i] = b, c
            t[AND + i], t[OR + i], t[XOR + i], t[NAND + i] = b & c, b | c, b ^ c, ~(b & c) & 15
            t[NEAR + i] = b & c
            t[ROWSEL + 256 + i] = b & c  # row a = 1 only
    t[NEAR + 0x5A] ^= 1  # one entry off: not a bitwise row
    t[ROWSEL + 0x33] = 7  # row a = 0 is not bitwise (7 = 0b0111 with b = c = 3)
    return bytes(t)


# (lut, op0, op1, op2) per lane, three single-level micro-partitions of one exec level
OPS = [
    [(AND, 0, IN + 0, IN + 1), (NEAR, 0, IN + 0, IN + 1), (MUX, IN + 8, IN + 9, IN + 10), (RAND, 0, IN + 2, IN + 3)],
    [(OR, 0, IN + 2, IN + 3), (XOR, 0, IN + 4, IN + 5), (ROWSEL, 1, IN + 6, IN + 7), (ROWSEL, 0, IN + 6, IN + 7)],
    [(NAND, 0, IN + 6, IN + 7), (MUX, IN + 11, IN + 12, IN + 13), (MUXI, IN + 8, IN + 14, IN + 15),
     (0, 0, 9, IN + 4)],
]
FAST = 8  # LUT ops with a word-wide form (every op but NEAR, ROWSEL with a = 0, RAND and the move)
# 29 more table ops into unobserved slots: 32 table ops in all, so the 9
# word-wide ops (the move included) form their own micro-partition (a partial
# one that fits in the table ops' last micro-partition joins them instead)
FILL = [(RAND, 0, IN + (i % 16), IN + ((5 * i) % 16)) for i in range(29)]


def fast_design() -> dl.Design:
    level, k = [], 0
    for mp in OPS:
        lanes = [dl.top(*op) for op in mp]
        level.append(dl.MPart(top=lanes, wbs=[dl.wb(32 + i, OUT + k + i) for i in range(len(mp))]))
        k += len(mp)
    level.append(dl.MPart(top=[dl.top(*op) for op in FILL], wbs=[dl.wb(32 + i, 100 + i) for i in range(len(FILL))]))
    return frame([level], lut=fast_table())


def inputs(stream: int) -> np.ndarray:
    r = np.array([(3 * i + 5 * stream + 1) & 15 for i in range(16)], np.uint8)
    r[8] = stream & 1                               # selects 0/1 in every stream
    r[11] = stream & 1 if stream >= 16 else stream  # above 1 in the first two words of 8 streams
    return r


def expected(stream: int) -> np.ndarray:
    t, r = fast_table(), inputs(stream)
    val = lambda x: int(r[x - IN]) if x >= 16 else x  # noqa: E731
    out, k = np.zeros(32, np.uint8), 0
    for mp in OPS:
        for lut, a, b, c in mp:
            out[k] = val(c) if lut == 0 else t[lut + ((val(a) << 8) | (val(b) << 4) | val(c))]
            k += 1
    return out


def repack(src, dst, lane_packing=1, fast=1):
    st = capi.RepackStats()
    capi.check(capi.lib().tgs_repack_design(str(src).encode(), str(dst).encode(), lane_packing, fast, C.byref(st)))
    return st


def test_palette_rows_recognised(tmp_path, built):
    dp = tmp_path / "fast.bin"
    fast_design().write(dp)
    st = repack(dp, tmp_path / "r.bin")
    assert st.lut_ops == 11 + len(FILL) and st.fast_lut_ops == FAST
    # the ops are regrouped: word-wide ops (bitwise, then multiplexers) share
    # one micro-partition, the 32 table ops another
    assert (st.mparts_before, st.mparts_after, st.fast_mparts) == (5, 3, 1)
    off = repack(dp, tmp_path / "n.bin", lane_packing=0, fast=0)
    assert off.fast_lut_ops == 0 and off.mparts_after == off.mparts_before


@pytest.mark.parametrize("stream", [0, 1, 5, 16, 17])
def test_fast_kat_oracle(tmp_path, built, stream):
    dp, rp = tmp_path / "fast.bin", tmp_path / "r.bin"
    fast_design().write(dp)
    repack(dp, rp)
    for path in (dp, rp):  # the original and the regrouped design
        st = pyoracle.OracleState(pyoracle.OracleDesign(path))
        st.regs()[:16] = inputs(stream)
        st.eval(1)
        np.testing.assert_array_equal(st.regs()[16:48], expected(stream), err_msg=str(path.name))


PALETTE = {
    "wide3op": dict(seed=12, n_lut=20000, levels=12, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=64,
                    ff_bits=2048, pi_bits=64, n_vec_ops=24, vec_nibbles=8, n_mems=3, mem_depth=4096, mem_width=32,
                    mem_read_ports=2, mem_write_ports=2, mem_multi_writer=1, luts_per_part=2500, mpart_width=32,
                    cone_depth=1),
    "mixed": dict(seed=14, n_lut=40000, levels=64, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=65536,
                  ff_bits=8192, pi_bits=64, n_mems=16, mem_depth=1024, mem_width=64, mem_read_ports=2,
                  mem_write_ports=1, luts_per_part=4000, mpart_width=32, cone_depth=1, mixed=1),
    "cones": dict(seed=18, n_lut=12000, levels=16, operands=3, palette_pct=60, ff_bits=1024, pi_bits=32, n_mems=1,
                  mem_depth=256, mem_width=32, mem_read_ports=1, mem_write_ports=1, luts_per_part=3000,
                  mpart_width=16, cone_depth=3),
}


@pytest.fixture(scope="module")
def palette(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("palette")
    out = {}
    for name, cfg in PALETTE.items():
        dp, sp = d / f"{name}.bin", d / f"{name}.sym"
        out[name] = (dp, sp, sim.generate(dp, sp, **cfg))
    return out


@pytest.mark.parametrize("name", list(PALETTE))
def test_regrouped_design_matches_original(palette, tmp_path, name):
    dp, sp, info = palette[name]
    rp = tmp_path / "r.bin"
    st = repack(dp, rp)
    sim.validate_file(rp, sp)
    if name == "wide3op":  # single-level micro-partitions: about the palette share is word-wide
        assert 0.3 < st.fast_lut_ops / st.lut_ops < 0.6, (st.fast_lut_ops, st.lut_ops)
    else:  # cones: only top levels made of palette ops and moves
        assert st.fast_lut_ops < st.lut_ops / 4
    stim = sim.StimulusSpec(3, info["pi_ids"], info["pi_bits"])
    cyc = np.full(3, 25, np.uint32)
    a = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
    b = pyoracle.OracleDesign(rp, sp).run(cyc, stim, cycle_digests=True)
    for k in ("cycle_digest", "final_reg_digest", "final_mem_digest", "stop_cycle"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("f", EVAL, ids=_ids(EVAL))
def test_regrouped_design_reproduces_reference_kernel(built, tmp_path, f):
    dst = tmp_path / "r.bin"
    repack(G / f"{f['case']}.bin", dst)
    od = pyoracle.OracleDesign(dst, G / f"{f['case']}.sym", randomize=bool(f["randomize"]))
    out = od.run(np.full(f["streams"], f["cycles"], np.uint32), _stim(f), cycle_digests=True)
    for s, r in enumerate(f["results"]):
        np.testing.assert_array_equal(out["cycle_digest"][s], np.array([int(x, 16) for x in r["cycle_digests"]], np.uint64))
        assert out["final_reg_digest"][s] == _h(r["final_reg_digest"])
        assert out["final_mem_digest"][s] == _h(r["final_mem_digest"])


@pytest.mark.gpu
@pytest.mark.parametrize("streams,groups", [(1, 1), (24, 1), (24, 2), (32, 4)])
@pytest.mark.parametrize("fast", [0, 1])
def test_fast_kat_gpu(tmp_path, built, streams, groups, fast):
    dp = tmp_path / "fast.bin"
    fast_design().write(dp)
    with sim.Simulator(n_streams=streams, groups_per_item=groups, fast_luts=fast) as s:
        s.init(0, dp, None, False, False)
        for k in range(streams):
            pool = s.reg_pool(k)
            pool[:16] = inputs(k)
            s.write_reg_pool(pool, k)
        s.eval()
        for k in range(streams):
            np.testing.assert_array_equal(s.reg_pool(k)[16:48], expected(k), err_msg=f"stream {k}")


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(PALETTE))
@pytest.mark.parametrize("fast", [0, 1])
def test_palette_designs_gpu(palette, name, fast):
    dp, sp, info = palette[name]
    stim = sim.StimulusSpec(9, info["pi_ids"], info["pi_bits"])
    cyc = np.full(40, 20, np.uint32)
    with sim.Simulator(n_streams=40, fast_luts=fast) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cyc, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"])
    for k in ("final_reg_digest", "final_mem_digest", "rolling_digest"):
        np.testing.assert_array_equal(getattr(got, k), ref[k], err_msg=k)


def test_partial_wordwide_group_joins_table_ops(tmp_path, built):
    """A level of 9 word-wide and 3 table ops: the word-wide group would be a
    second warp pass, so its ops stay with the table ops (one micro-partition,
    evaluated by lookup) -- and still compute the same values."""
    d = fast_design()
    d.parts[0].levels[1] = d.parts[0].levels[1][:3]  # without the filler ops
    dp = tmp_path / "f.bin"
    d.write(dp)
    st = repack(dp, tmp_path / "r.bin")
    assert (st.mparts_before, st.mparts_after, st.fast_mparts, st.fast_lut_ops) == (4, 2, 0, 0)
    s = pyoracle.OracleState(pyoracle.OracleDesign(tmp_path / "r.bin"))
    s.regs()[:16] = inputs(3)
    s.eval(1)
    np.testing.assert_array_equal(s.regs()[16:48], expected(3))
