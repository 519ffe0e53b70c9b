"""Element-wise batch field operations through the C ABI (goldilocks-cuda-rs ffi.rs:105-280, :633;
almost-goldilocks-cuda-rs ffi.rs:95-140) against plain big-integer arithmetic: base fields,
Ext2 (X^2 - 7 over p, X^2 - 3 over q) and Ext5 (X^5 - 3 over p, cuda/extension.cuh), with zeros
and non-canonical inputs.  Inverses of zero are zero."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
P, Q = O.P, O.Q_AGL
N = 67


def ext_mul(a, b, mod, nr):
    d = len(a)
    out = [0] * d
    for i in range(d):
        for j in range(d):
            k = i + j
            if k < d:
                out[k] += a[i] * b[j]
            else:
                out[k - d] += nr * a[i] * b[j]
    return [x % mod for x in out]


def ext_pow(a, e, mod, nr):
    r = [1] + [0] * (len(a) - 1)
    b = list(a)
    while e:
        if e & 1:
            r = ext_mul(r, b, mod, nr)
        b = ext_mul(b, b, mod, nr)
        e >>= 1
    return r


def ext_inv(a, mod, nr):
    d = len(a)
    if not any(x % mod for x in a):
        return [0] * d
    # a^(mod^d - 2) in F_{mod^d}
    return ext_pow(a, mod ** d - 2, mod, nr)


def call(L, name, ins, scalar=None, exp=None, out_words=0, acc=None):
    from morpheus_gb300.memory import DeviceBuffer
    bufs = [DeviceBuffer.from_numpy(np.ascontiguousarray(x, np.uint64)) for x in ins]
    out = DeviceBuffer.from_numpy(np.ascontiguousarray(acc, np.uint64)) if acc is not None else DeviceBuffer(out_words)
    fn = getattr(L, name)
    if scalar is not None and isinstance(scalar, tuple):
        rc = fn(scalar[0], scalar[1], bufs[0].ptr, out.ptr, N)
    elif scalar is not None:
        rc = fn(scalar, bufs[0].ptr, out.ptr, N)
    elif exp is not None:
        rc = fn(bufs[0].ptr, exp, out.ptr, N)
    else:
        rc = fn(*[b.ptr for b in bufs], out.ptr, N)
    assert rc == 0, name
    L.cuda_sync_mine()
    return out.to_numpy()


CASES = [("gl", P, 1, 0, "gl_batch_{}"), ("gl2", P, 2, 7, "ext2_batch_{}_ffi"), ("gl5", P, 5, 3, "ext5_batch_{}_ffi"),
         ("agl", Q, 1, 0, "agl_batch_{}_ffi"), ("agl2", Q, 2, 3, "aext2_batch_{}_ffi")]


def rand_elems(rng, n, d, mod):
    x = rng.integers(0, 2**64 - 1, size=(n, d), dtype=np.uint64)  # non-canonical words too
    x[0] = 0
    x[1] = [1] + [0] * (d - 1)
    x[2] = [mod - 1] * d
    return x


@pytest.mark.parametrize("tag,mod,d,nr,pat", CASES)
def test_elementwise_ops(gpu_lib, tag, mod, d, nr, pat):
    from morpheus_gb300 import _native as N_
    L = N_.lib()
    rng = np.random.default_rng(d * 7 + nr)
    a, b = rand_elems(rng, N, d, mod), rand_elems(rng, N, d, mod)[::-1].copy()
    A = [[int(v) % mod for v in row] for row in a]
    B = [[int(v) % mod for v in row] for row in b]
    s = int(rng.integers(0, mod, dtype=np.uint64))
    e = 0x1234_5678_9ABC
    ops = {
        "div": (lambda x, y: ext_mul(x, ext_inv(y, mod, nr), mod, nr) if d > 1 else [x[0] * (pow(y[0], mod - 2, mod)) % mod], 2),
        "neg": (lambda x, y: [(-v) % mod for v in x], 1),
        "square": (lambda x, y: ext_mul(x, x, mod, nr) if d > 1 else [x[0] * x[0] % mod], 1),
        "mul_scalar": (lambda x, y: [v * s % mod for v in x], "s"),
        "exp": (lambda x, y: ext_pow(x, e, mod, nr) if d > 1 else [pow(x[0], e, mod)], "e"),
        "inverse": (lambda x, y: ext_inv(x, mod, nr) if d > 1 else [pow(x[0], mod - 2, mod)], 1),
        "add": (lambda x, y: [(u + v) % mod for u, v in zip(x, y)], 2),
        "sub": (lambda x, y: [(u - v) % mod for u, v in zip(x, y)], 2),
        "mul": (lambda x, y: ext_mul(x, y, mod, nr) if d > 1 else [x[0] * y[0] % mod], 2),
        "double": (lambda x, y: [2 * v % mod for v in x], 1),
    }
    present = {"gl": ["div", "neg", "square", "mul_scalar", "exp", "double"],
               "gl2": ["inverse", "neg", "square", "mul_scalar", "exp"],
               "gl5": ["add", "sub", "mul", "inverse", "neg", "square", "mul_scalar", "exp"],
               "agl": ["add", "sub", "mul", "div", "inverse", "neg", "square", "mul_scalar", "exp", "double"],
               "agl2": ["add", "sub", "mul", "inverse", "neg", "square", "mul_scalar", "exp"]}[tag]
    for op in present:
        f, kind = ops[op]
        name = pat.format(op)
        if kind == "s":
            got = call(L, name, [a], scalar=s, out_words=N * d)
        elif kind == "e":
            got = call(L, name, [a], exp=e, out_words=N * d)
        elif kind == 2:
            got = call(L, name, [a, b], out_words=N * d)
        else:
            got = call(L, name, [a], out_words=N * d)
        want = [f(x, y) for x, y in zip(A, B)]
        assert [[int(v) for v in row] for row in got.reshape(N, d)] == want, name
    if d >= 2:
        # Frobenius a -> a^mod; conjugate (quadratic) the same map
        for op in (["frobenius", "conjugate"] if d == 2 else ["frobenius"]):
            got = call(L, pat.format(op), [a], out_words=N * d)
            want = [ext_pow(x, mod, mod, nr) for x in A[:12]]
            assert [[int(v) for v in row] for row in got.reshape(N, d)[:12]] == want, op


def test_scale_accumulate_conversions_and_zero(gpu_lib):
    from morpheus_gb300 import _native as N_
    from morpheus_gb300.memory import DeviceBuffer
    L = N_.lib()
    rng = np.random.default_rng(3)
    for mod, nr, name in [(P, 7, "ext2_scale_accumulate_ffi"), (Q, 3, "aext2_scale_accumulate_ffi")]:
        src = rng.integers(0, mod, size=(N, 2), dtype=np.uint64)
        acc = rng.integers(0, mod, size=(N, 2), dtype=np.uint64)
        sc = (int(rng.integers(0, mod, dtype=np.uint64)), int(rng.integers(0, mod, dtype=np.uint64)))
        got = call(L, name, [src], scalar=sc, acc=acc).reshape(N, 2)
        for i in range(N):
            t = ext_mul(list(sc), [int(src[i, 0]), int(src[i, 1])], mod, nr)
            assert [int(got[i, 0]), int(got[i, 1])] == [(int(acc[i, 0]) + t[0]) % mod, (int(acc[i, 1]) + t[1]) % mod]
    x = rng.integers(0, 2**64 - 1, size=N, dtype=np.uint64)
    for up, down, w, mod in [("gl_to_ext2_batch_ffi", "ext2_to_gl_batch_ffi", 2, P),
                             ("gl_to_ext5_batch_ffi", "ext5_to_gl_batch_ffi", 5, P),
                             ("agl_to_aext2_batch_ffi", "aext2_to_agl_batch_ffi", 2, Q)]:
        lifted = call(L, up, [x], out_words=N * w).reshape(N, w)
        assert [int(v) for v in lifted[:, 0]] == [int(v) % mod for v in x] and not lifted[:, 1:].any()
        back = call(L, down, [lifted.reshape(-1)], out_words=N)
        assert [int(v) for v in back] == [int(v) % mod for v in x]
    buf = DeviceBuffer.from_numpy(np.full(100, 7, np.uint64))
    assert L.gl_memset_zero(buf.ptr, 60) == 0 and L.gl_zero_buffer(buf.ptr, 0) == 0
    L.cuda_sync_mine()
    v = buf.to_numpy()
    assert not v[:60].any() and (v[60:] == 7).all()
    assert L.agl_zero_buffer_ffi(buf.ptr, 100) == 0
    L.cuda_sync_mine()
    assert not buf.to_numpy().any()
    assert L.gl_batch_neg(buf.ptr, buf.ptr, -1) == -2


def test_runtime_helpers(gpu_lib):
    """Peer copies on one device, NVTX ranges, the i64/i32 helpers and the stream toggle."""
    from morpheus_gb300 import _native as N_
    from morpheus_gb300.memory import DeviceBuffer
    L = N_.lib()
    src = DeviceBuffer.from_numpy(np.arange(100, dtype=np.uint64))
    dst = DeviceBuffer(100)
    assert L.cuda_memcpy_peer(dst.ptr, 0, src.ptr, 0, 800) == 0
    assert (dst.to_numpy() == np.arange(100)).all()
    assert L.cuda_enable_peer_access(0) == -1  # a device is not its own peer
    L.agl_nvtx_push(b"range")
    L.agl_nvtx_pop()
    s = DeviceBuffer.from_numpy(np.array([1, -2, 2**40 + 5, -(2**33)], np.int64))
    d = DeviceBuffer(4, np.int32)
    assert L.agl_i64_to_i32(s.ptr, d.ptr, 4) == 0
    assert d.to_numpy().tolist() == [1, -2, 5, 0]
    assert L.agl_add_i32_i64(s.ptr, d.ptr, 4) == 0
    assert s.to_numpy().tolist() == [2, -4, 2**40 + 10, -(2**33)]
    assert L.agl_gauss_low_priority(1) == 0 and L.agl_gauss_low_priority(0) == 0
