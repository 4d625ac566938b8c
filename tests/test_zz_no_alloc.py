"""PSReduceNoAlloc: the reduction for callers that cannot allocate GPU memory.

Some callers of this library may not call cudaMalloc: latency-bound loops
that cannot afford the device-wide synchronisation an allocation implies, and
processes whose device memory belongs to another allocator (a caching pool
that has reserved the free memory).  PSReduceNoAlloc reduces a grid the
caller already holds in device memory and writes the 8-byte result to device
memory the caller passes, using only a static device array as scratch.
These tests check that it agrees with the allocating entry point (PSReduce
through a grid handle) on two calls in a row, and that it rejects bad
arguments before touching a GPU.

This file is collected last on purpose (tests/test_zz_*): if it fails, a
run that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import physis_gb300 as ps
from physis_gb300 import synth


@pytest.fixture(scope="module")
def lib():
    ps.build()
    return ps.lib()


def _call(L, data, pitch, dims, typ, op, result, stream=None):
    nz, ny, nx = dims
    return L.PSReduceNoAlloc(data, pitch, nx, ny, nz, typ, op, result, stream)


def test_rejects_bad_arguments_before_using_a_gpu(lib):
    ps.clear_error()
    fake = ctypes.c_void_p(4096)  # never dereferenced: arguments fail first
    assert _call(lib, None, 512, (4, 4, 4), ps.PS_FLOAT, ps.PS_SUM, fake) == \
        ps.PS_ERR_INVALID_ARGUMENT
    assert _call(lib, fake, 8, (4, 4, 4), ps.PS_FLOAT, ps.PS_SUM, fake) == \
        ps.PS_ERR_INVALID_ARGUMENT  # pitch shorter than a row
    assert _call(lib, fake, 512, (4, 4, 4), 9, ps.PS_SUM, fake) == \
        ps.PS_ERR_INVALID_ARGUMENT  # unknown element type
    assert _call(lib, fake, 512, (4, 4, 4), ps.PS_FLOAT, 7, fake) == \
        ps.PS_ERR_INVALID_ARGUMENT  # unknown op
    assert _call(lib, fake, 512, (0, 4, 4), ps.PS_FLOAT, ps.PS_SUM, fake) == \
        ps.PS_ERR_INVALID_ARGUMENT
    code, msg = ps.last_error()
    assert code == ps.PS_ERR_INVALID_ARGUMENT and "PSReduceNoAlloc" in msg
    ps.clear_error()


CASES = [
    (np.float32, ps.PS_SUM, (64, 96, 130)),
    (np.float32, ps.PS_MAX, (9, 17, 33)),
    (np.float64, ps.PS_SUM, (16, 40, 77)),
    (np.int32, ps.PS_SUM, (20, 20, 20)),
    (np.int64, ps.PS_MIN, (3, 5, 1000)),
]


def _data(shape, dtype, seed):
    if np.issubdtype(dtype, np.integer):
        return np.random.default_rng(seed).integers(-1000, 1000, shape).astype(dtype)
    return synth.uniform(shape, seed).astype(dtype)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,op,shape", CASES)
def test_matches_allocating_entry_point_on_two_calls(lib, dtype, op, shape):
    ps.init()
    stream = lib.PSGetStream()
    is_int = np.issubdtype(dtype, np.integer)
    slot = ps.Grid((1,), np.int64 if is_int else np.float64)  # 8-byte result
    for call, seed in enumerate((21, 22)):  # two calls in a row, new data each
        data = _data(shape, dtype, seed)
        g = ps.Grid(shape, dtype)
        g.copyin(data)
        expect = ps.reduce(g, op) if is_int else ps.reduce_f64(g, op)
        slot.copyin(np.array([-12345], dtype=slot.dtype))  # no stale pass
        rc = _call(lib, g.dev_ptr, g.pitch, shape, ps.TYPE_OF[np.dtype(dtype)], op,
                   slot.dev_ptr, stream)
        assert rc == ps.PS_OK, ps.last_error()
        ps.synchronize()
        got = slot.copyout()[0]
        if is_int:
            assert int(got) == int(expect), (call, got, expect)
        else:
            # the tolerance the float reductions are held to everywhere
            assert abs(float(got) - expect) <= 1e-6 * abs(expect), (call, got, expect)
        g.free()
    slot.free()
