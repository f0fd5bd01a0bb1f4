"""Signal capture (readSignal / VCD dump, the reference's unbuilt
unsupport/SimVCD.cpp path): every signal of the symbol file read on the GPU
equals the oracle's value-pool probes, per stream, for both value-pool
numberings; the VCD file holds the same values per time step."""
import re

import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import capi, sim

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sig_design(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("signals")
    dp, sp = d / "d.bin", d / "s.bin"
    cfg = dict(seed=41, n_lut=12000, levels=12, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=64,
               ff_bits=2048, pi_bits=64, n_vec_ops=16, vec_nibbles=8, n_mems=2, mem_depth=1024, mem_width=32,
               mem_read_ports=2, mem_write_ports=1, luts_per_part=2000, mpart_width=32, cone_depth=2, signals=48)
    info = sim.generate(dp, sp, **cfg)
    return dp, sp, info


def _oracle_states(dp, sp, n, regs):
    od = pyoracle.OracleDesign(dp, sp)
    sigs = sim.symbol_signals(sp)
    names = sorted(sigs)
    parts, slots, spans = [], [], {}
    for name in names:
        start = len(parts)
        for (pt, sl, w) in sigs[name]:
            parts.append(pt)
            slots.append(sl)
        spans[name] = (start, len(parts))
    states = []
    for s in range(n):
        st = pyoracle.OracleState(od)
        st.regs()[:] = regs[s]
        st.set_probes(parts, slots)
        states.append(st)
    return sigs, names, spans, states


def _value(sigs, spans, name, probe_vals):
    a, b = spans[name]
    v = 0
    for (pt, sl, w), x in zip(sigs[name], probe_vals[a:b]):
        v = (v << w) | (int(x) & ((1 << w) - 1))
    return v


@pytest.mark.parametrize("value_pool", [0, 1])
def test_signals_match_oracle_per_stream(sig_design, value_pool):
    dp, sp, info = sig_design
    n = 10
    with sim.Simulator(n_streams=n, capture_signals=1, value_pool=value_pool) as s:
        s.init(0, dp, sp, False, False)
        rng = np.random.default_rng(3)
        regs = [rng.integers(0, 16, s.pool_sizes()[0]).astype(np.uint8) for _ in range(n)]
        for q in range(n):
            s.write_reg_pool(regs[q], stream=q)
        sigs, names, spans, states = _oracle_states(dp, sp, n, regs)
        assert len(names) >= 20
        for c in range(4):
            s.eval()
            for q in range(n):
                states[q].eval(1)
                pv = states[q].probe_values()
                for name in names:
                    assert s.read_signal(name, q) == _value(sigs, spans, name, pv), (c, q, name)


def test_vcd_dump_matches_oracle(sig_design, tmp_path):
    dp, sp, info = sig_design
    vcd = tmp_path / "dump.vcd"
    with sim.Simulator() as s:
        s.init(0, dp, sp, True, False)
        s.enable_vcd(vcd)  # turns capture on before the first cycle
        for _ in range(3):
            s.eval()
        s.eval_free_running(5)
    od = pyoracle.OracleDesign(dp, sp, randomize=True)
    sigs = sim.symbol_signals(sp)
    names = sorted(sigs)
    parts, slots, spans = [], [], {}
    for name in names:
        spans[name] = (len(parts), len(parts) + len(sigs[name]))
        for (pt, sl, w) in sigs[name]:
            parts.append(pt)
            slots.append(sl)
    st = pyoracle.OracleState(od)
    st.set_probes(parts, slots)
    expect = {}
    for c in range(8):
        st.eval(1)
        expect[c] = {nm: _value(sigs, spans, nm, st.probe_values()) for nm in names}
    text = vcd.read_text()
    ids, widths = {}, {}
    scope = []
    for line in text.splitlines():
        m = re.match(r"\$scope module (\S+) \$end", line)
        if m:
            scope.append(m.group(1))
        elif line.startswith("$upscope"):
            scope.pop()
        m = re.match(r"\$var wire (\d+) (\S+) (\S+) \$end", line)
        if m:
            full = ".".join(scope + [m.group(3)])
            ids[m.group(2)] = full
            widths[full] = int(m.group(1))
    assert sorted(ids.values()) == names
    for nm in names:
        assert widths[nm] == max(1, sum(w for _, _, w in sigs[nm]))
    cur, steps = {}, {}
    body = text.split("$dumpvars", 1)[1]
    t = None
    for line in body.splitlines():
        if not line:
            continue
        if line.startswith("#"):
            t = int(line[1:])
            steps[t] = dict(cur)
            continue
        if line.startswith("b"):
            bits, ident = line[1:].split()
        else:
            bits, ident = line[0], line[1:]
        cur[ids[ident]] = int(bits, 2)
        steps[t] = dict(cur)
    assert sorted(steps) == [0, 1, 2, 7]
    for t, vals in steps.items():
        assert vals == expect[t], t


def test_signal_capture_errors(sig_design, tmp_path):
    dp, sp, _ = sig_design
    with sim.Simulator() as s:
        s.init(0, dp, sp, False, False)
        name = sorted(sim.symbol_signals(sp))[0]
        with pytest.raises(capi.TgsError):
            s.read_signal(name)
        with pytest.raises(capi.TgsError):
            s.read_signal("no_such_signal")
        s.eval()
        with pytest.raises(capi.TgsError):
            s.enable_vcd(tmp_path / "late.vcd")
