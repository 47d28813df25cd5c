"""The allocation-free evaluation entry (hp_cuda_v1_mle_evaluate_noalloc).

Callers that own all device memory through their own arena cannot let the
library allocate; this entry keeps its intermediates in a fixed device array.  The test calls it through
the C ABI and checks its result against the allocating entry
hp_cuda_v1_mle_evaluate on the same inputs, twice in a row (the shared array
keeps the previous call's contents, which must not matter).  This file is
collected last so that a failing run with -x has already run every other test.
"""
import ctypes
import random

import pytest

from hyperplonk_gb300 import _native
from hyperplonk_gb300.backend import encode_frs
from hyperplonk_gb300.errors import InvalidParameters, check_status

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def _bind(lib):
    fn = lib.hp_cuda_v1_mle_evaluate_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_uint8),
                   ctypes.c_void_p]
    fn.restype = _native.Status
    return fn


def _evaluate_allocating(gpu, mle, point_bytes):
    out = (ctypes.c_uint8 * 32)()
    check_status(gpu.lib.hp_cuda_v1_mle_evaluate(gpu.ctx.raw, ctypes.c_void_p(mle.address), mle.num_vars,
                                                 _native.buf(point_bytes), out), "mle_evaluate")
    return bytes(out)


def _evaluate_noalloc(gpu, fn, mle, point_bytes):
    out = (ctypes.c_uint8 * 32)()
    check_status(fn(ctypes.c_void_p(mle.address), mle.num_vars, _native.buf(point_bytes), out,
                    ctypes.c_void_p(gpu.ctx.stream())), "mle_evaluate_noalloc")
    return bytes(out)


def test_noalloc_evaluate_matches_allocating_entry_twice(gpu, oracle):
    fn = _bind(gpu.lib)
    rng = random.Random(2024)
    # two calls in a row with different sizes and inputs, then the first again
    cases = [(20, 31), (13, 32), (20, 31)]
    tables = {}
    for nv, seed in cases:
        if (nv, seed) not in tables:
            tables[(nv, seed)] = gpu.mle_from_evaluations(nv, oracle.random_fr(seed, 1 << nv))
    for nv, seed in cases:
        mle = tables[(nv, seed)]
        pt = encode_frs([rng.randrange(R) for _ in range(nv)])
        expect = _evaluate_allocating(gpu, mle, pt)
        assert _evaluate_noalloc(gpu, fn, mle, pt) == expect
        assert _evaluate_noalloc(gpu, fn, mle, pt) == expect


@pytest.mark.parametrize("nv", [0, 1, 9, 10, 11, 24])
def test_noalloc_evaluate_sizes(gpu, oracle, nv):
    fn = _bind(gpu.lib)
    mle = gpu.mle_from_evaluations(nv, oracle.random_fr(50 + nv, 1 << nv))
    rng = random.Random(nv)
    pt = encode_frs([rng.randrange(R) for _ in range(nv)]) if nv else None
    assert _evaluate_noalloc(gpu, fn, mle, pt) == _evaluate_allocating(gpu, mle, pt)


def test_noalloc_rejects_tables_above_the_limit(gpu, oracle):
    fn = _bind(gpu.lib)
    mle = gpu.mle_from_evaluations(2, oracle.random_fr(1, 4))
    pt = encode_frs([1] * 25)
    out = (ctypes.c_uint8 * 32)()
    with pytest.raises(InvalidParameters):
        check_status(fn(ctypes.c_void_p(mle.address), 25, _native.buf(pt), out, None), "mle_evaluate_noalloc")


def test_noalloc_rejects_a_host_pointer(gpu):
    """A table that is not memory of the current device is refused before any
    kernel runs."""
    fn = _bind(gpu.lib)
    host_table = (ctypes.c_uint8 * (32 * 4))()
    pt = encode_frs([3, 5])
    out = (ctypes.c_uint8 * 32)()
    with pytest.raises(InvalidParameters):
        check_status(fn(ctypes.cast(host_table, ctypes.c_void_p), 2, _native.buf(pt), out, None),
                     "mle_evaluate_noalloc")
