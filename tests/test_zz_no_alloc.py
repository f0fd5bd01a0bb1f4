"""tgs_pool_digests_noalloc: digests of caller-owned device memory for
callers that cannot allocate device memory.  Checked against the existing
entry point (tgs_state_digest) on two calls in a row; the pools live in
device memory the test owns (a torch tensor), as a caller's allocator would
hand them over.  Collected last so a failure here stops a -x run only after
every other test has run."""
import ctypes as C

import numpy as np
import pytest

from toucangpurt_gb300 import capi, sim


@pytest.mark.gpu
def test_noalloc_digests_match_state_digest(small_design):
    torch = pytest.importorskip("torch")
    dp, sp, info = small_design
    n = 16
    with sim.Simulator(n_streams=n) as s:
        s.init(0, dp, sp, True, False)
        stim = sim.StimulusSpec(5, info["pi_ids"], info["pi_bits"])
        s.batch_run(np.full(n, 30, np.uint32), stim)
        mem_bytes = s.pool_sizes()[1]
        stride = (mem_bytes + 255) // 256 * 256
        host = np.zeros((n, stride), np.uint8)
        expect = np.zeros(n, np.uint64)
        for k in range(n):
            host[k, :mem_bytes] = s.mem_pool(k)
            expect[k] = s.digest(k)[1]
    dev = torch.from_numpy(host).to("cuda:0")
    torch.cuda.synchronize()
    for call in range(2):
        got = np.zeros(n, np.uint64)
        capi.check(capi.lib().tgs_pool_digests_noalloc(C.c_void_p(dev.data_ptr()), stride, mem_bytes, n,
                                                       got.ctypes.data_as(capi.u64p)))
        np.testing.assert_array_equal(got, expect, err_msg=f"call {call}")
    # a shorter second use of the shared array must not see the first call's sums
    got = np.zeros(3, np.uint64)
    capi.check(capi.lib().tgs_pool_digests_noalloc(C.c_void_p(dev.data_ptr()), stride, mem_bytes, 3,
                                                   got.ctypes.data_as(capi.u64p)))
    np.testing.assert_array_equal(got, expect[:3])
    with pytest.raises(capi.TgsError) as e:
        capi.check(capi.lib().tgs_pool_digests_noalloc(C.c_void_p(dev.data_ptr()), stride, mem_bytes, 4097,
                                                       got.ctypes.data_as(capi.u64p)))
    assert e.value.code == capi.ERR_RANGE


_RESET_CHILD = r"""
import ctypes as C, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from toucangpurt_gb300 import capi, sim
dp, sp, pi_ids, pi_bits = sys.argv[2], sys.argv[3], json.loads(sys.argv[4]), json.loads(sys.argv[5])
lib = capi.lib()
n = 4
with sim.Simulator(n_streams=n) as s:
    s.init(0, dp, sp, True, False)
    s.batch_run(np.full(n, 30, np.uint32), sim.StimulusSpec(5, np.array(pi_ids), np.array(pi_bits)))
    mem_bytes = s.pool_sizes()[1]
    stride = (mem_bytes + 255) // 256 * 256
    host = np.zeros((n, stride), np.uint8)
    expect = np.zeros(n, np.uint64)
    for k in range(n):
        host[k, :mem_bytes] = s.mem_pool(k)
        expect[k] = s.digest(k)[1]


def noalloc():
    # the pools in page-locked host memory, which kernels read directly
    buf = C.c_void_p()
    capi.check(lib.tgs_host_alloc(host.nbytes, C.byref(buf)))
    C.memmove(buf, host.ctypes.data, host.nbytes)
    got = np.zeros(n, np.uint64)
    capi.check(lib.tgs_pool_digests_noalloc(buf, stride, mem_bytes, n, got.ctypes.data_as(capi.u64p)))
    capi.check(lib.tgs_host_free(buf))
    return got


before = noalloc()
capi.check(lib.tgs_device_reset(0))
after = noalloc()
assert (before == expect).all(), (before, expect)
assert (after == expect).all(), (after, expect)
print("noalloc across reset ok")
"""


@pytest.mark.gpu
def test_noalloc_across_device_reset(small_design):
    """The accumulator array's device address is looked up on every call, so
    the entry point stays right after the device's context is destroyed and
    re-created (tgs_device_reset) and the array moves.  A child process: the
    reset destroys every allocation the process holds on the device."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    dp, sp, info = small_design
    root = str(Path(__file__).resolve().parent.parent)
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, root, str(dp), str(sp),
                        json.dumps([int(x) for x in info["pi_ids"]]), json.dumps([int(x) for x in info["pi_bits"]])],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "noalloc across reset ok" in r.stdout
