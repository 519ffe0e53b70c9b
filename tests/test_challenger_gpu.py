"""Device challengers against a restatement of the reference's DuplexChallenger
(cuda/challenger.cuh:37-222) over the oracle's Poseidon2 permutation (pinned to the reference's
own permutation code)."""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
P = O.P


class Duplex:
    def __init__(self):
        self.sponge = [0] * 8
        self.inp, self.out = [], []

    def duplex(self):
        st = np.array([self.inp[i] if i < len(self.inp) else 0 for i in range(4)] + self.sponge[4:], np.uint64)
        self.inp = []
        st = [int(x) % P for x in O.poseidon2_permute(st)]
        self.sponge = st
        self.out = list(reversed(st[:4]))  # popped from the end: st[0] first

    def observe(self, v):
        self.out = []
        self.inp.append(int(v) % P)
        if len(self.inp) == 4:
            self.duplex()

    def sample(self):
        if not self.out:
            self.duplex()
        return self.out.pop()

    def state_bytes(self):
        words = self.sponge + self.inp + [0] * (4 - len(self.inp))
        # the output buffer keeps its last duplex's contents; only the count marks what is pending
        return words, len(self.inp), len(self.out)


def test_challenger_batch_matches_restatement(gpu_lib):
    from morpheus_gb300 import _native as N
    from morpheus_gb300.memory import DeviceBuffer
    L = N.lib()
    assert L.challenger_state_size() == 136
    n = 37
    st = ctypes.c_void_p()
    assert L.challenger_alloc_states(ctypes.byref(st), n) == 0
    try:
        assert L.challenger_init_states(st, n) == 0
        ref = [Duplex() for _ in range(n)]
        rng = np.random.default_rng(3)
        ops = ["obs", "slice3", "s", "obs_e2", "arr5", "s_e2", "slice6", "s_e5", "s", "s", "obs", "arr2"]
        for op in ops:
            if op.startswith("obs") or op.startswith("slice"):
                cnt = {"obs": 1, "obs_e2": 2, "slice3": 3, "slice6": 6}[op]
                vals = rng.integers(0, 1 << 64, size=n * cnt, dtype=np.uint64)  # non-canonical values too
                d = DeviceBuffer.from_numpy(vals)
                if op == "obs":
                    rc = L.challenger_observe_ffi(st, d.ptr, n)
                elif op == "obs_e2":
                    rc = L.challenger_observe_ext2_ffi(st, d.ptr, n)
                else:
                    rc = L.challenger_observe_slice_ffi(st, d.ptr, cnt, n)
                assert rc == 0
                for i in range(n):
                    for v in vals[i * cnt:(i + 1) * cnt]:
                        ref[i].observe(v)
            else:
                cnt = {"s": 1, "s_e2": 2, "s_e5": 5, "arr5": 5, "arr2": 2}[op]
                d = DeviceBuffer(n * cnt)
                if op == "s":
                    rc = L.challenger_sample_ffi(st, d.ptr, n)
                elif op == "s_e2":
                    rc = L.challenger_sample_ext2_ffi(st, d.ptr, n)
                elif op == "s_e5":
                    rc = L.challenger_sample_ext5_ffi(st, d.ptr, n)
                else:
                    rc = L.challenger_sample_array_ffi(st, d.ptr, cnt, n)
                assert rc == 0
                got = d.to_numpy().reshape(n, cnt)
                for i in range(n):
                    assert [int(x) for x in got[i]] == [ref[i].sample() for _ in range(cnt)]
        # one state through the host and back
        buf = ctypes.create_string_buffer(136)
        one = ctypes.c_void_p(st.value + 5 * 136)
        assert L.challenger_copy_state_to_host(buf, one) == 0
        words = np.frombuffer(buf.raw[:128], np.uint64)
        counts = np.frombuffer(buf.raw[128:], np.int32)
        w, ic, oc = ref[5].state_bytes()
        assert [int(x) for x in words[:8]] == w[:8] and int(counts[0]) == ic and int(counts[1]) == oc
        assert L.challenger_copy_state_to_device(ctypes.c_void_p(st.value + 6 * 136), buf) == 0
        d = DeviceBuffer(2 * 2)
        two = ctypes.c_void_p(st.value + 5 * 136)
        assert L.challenger_sample_ffi(two, d.ptr, 2) == 0  # states 5 and 6 are now identical
        a, b = d.to_numpy()[:2]
        assert a == b == ref[5].sample()
    finally:
        L.cuda_free(st)
