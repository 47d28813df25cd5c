"""GPU parity of the MSM and multilinear-KZG entries.

MSM: every case of the reference's golden MSM vectors (generate_golden.py:
uniform, zero/one scalars, identity bases, cancellations, hot buckets,
exceptional additions).  KZG: commit / multi_commit / open against the oracle
over the testing SRS, as backend/src/ascend910b3/integration_tests.rs
(commit_matches_cpu_and_independent_msm, open_matches_cpu_with_exact_quotients_and_evaluations)."""
import ctypes
import random

import pytest

from hyperplonk_gb300 import _native
from hyperplonk_gb300.backend import decode_g1
from hyperplonk_gb300.errors import InvalidParameters, InvalidState, check_status

from test_oracle_golden import msm_case, msm_keys

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def gpu_msm(gpu, bases_affine: bytes, scalars: bytes):
    import oracle as orc
    n = len(scalars) // 32
    packets = orc.affine_to_packets(bases_affine) if n else b""
    out = (ctypes.c_uint8 * 97)()
    check_status(gpu.lib.hp_cuda_v1_msm(gpu.ctx.raw, _native.buf(packets) if n else None,
                                        _native.buf(scalars) if n else None, n, out), "msm")
    return decode_g1(bytes(out))


def test_msm_matches_golden(gpu, oracle, golden):
    keys = msm_keys(golden.msm)
    for key in keys:
        bases, scalars, expected = msm_case(oracle, golden.msm, key)
        assert gpu_msm(gpu, bases, scalars) == oracle.affine_to_point(expected), key


def test_msm_hot_bucket(gpu, oracle):
    n = 4097
    gen = oracle.g1_generator()
    bases = oracle.g1_op(3, gen * n, k=list(range(1, n + 1)))
    scalars = (1).to_bytes(32, "little") * n
    assert gpu_msm(gpu, bases, scalars) == oracle.affine_to_point(oracle.msm(bases, scalars))


@pytest.mark.parametrize("n", [1, 3, 64, 1000, 1 << 13])
def test_msm_random(gpu, oracle, n):
    layers = oracle.srs_layers(13, 77)
    bases = layers[0][:96 * n]
    scalars = bytearray(oracle.random_fr(30 + n, n))
    scalars[0:32] = (R - 1).to_bytes(32, "little")
    scalars = bytes(scalars)
    assert gpu_msm(gpu, bases, scalars) == oracle.affine_to_point(oracle.msm(bases, scalars))


@pytest.fixture(scope="module")
def srs(oracle):
    nv = 10
    layers = oracle.srs_layers(nv, 5)
    return nv, layers


@pytest.fixture(scope="module")
def params(gpu, cpu, srs, oracle):
    nv, layers = srs
    return (gpu.prepare_prover_param(nv, [oracle.affine_to_packets(l) for l in layers]),
            cpu.prepare_prover_param(nv, layers))


def test_commit_every_dimension(gpu, cpu, oracle, params):
    pg, pc = params
    for nv in range(0, 11):
        t = oracle.random_fr(40 + nv, 1 << nv)
        assert gpu.commit(pg, gpu.mle_from_evaluations(nv, t)) == cpu.commit(pc, cpu.mle_from_evaluations(nv, t)), nv


def test_commit_equals_independent_msm(gpu, oracle, params, srs):
    """Commit = sum base * scalar over layer (pp_nv - nv) (pcs/multilinear_kzg/mod.rs:285-340)."""
    pg, _ = params
    nv_pp, layers = srs
    nv = 7
    t = oracle.random_fr(99, 1 << nv)
    direct = oracle.affine_to_point(oracle.msm(layers[nv_pp - nv], t))
    assert gpu.commit(pg, gpu.mle_from_evaluations(nv, t)) == direct


def test_multi_commit_mixed_dimensions_and_duplicates(gpu, cpu, oracle, params):
    pg, pc = params
    dims = [3, 10, 0, 7, 3]
    tables = [oracle.random_fr(60 + i, 1 << d) for i, d in enumerate(dims)]
    gm = [gpu.mle_from_evaluations(d, t) for d, t in zip(dims, tables)]
    cm = [cpu.mle_from_evaluations(d, t) for d, t in zip(dims, tables)]
    gm.append(gm[1])
    cm.append(cm[1])
    assert gpu.multi_commit(pg, gm) == cpu.multi_commit(pc, cm)
    assert gpu.multi_commit(pg, []) == []


@pytest.mark.parametrize("nv", [0, 1, 2, 5, 10])
def test_open(gpu, cpu, oracle, params, nv):
    pg, pc = params
    t = oracle.random_fr(80 + nv, 1 << nv)
    rng = random.Random(nv)
    pt = [rng.randrange(R) for _ in range(nv)]
    qg, eg = gpu.open(pg, gpu.mle_from_evaluations(nv, t), pt)
    qc, ec = cpu.open(pc, cpu.mle_from_evaluations(nv, t), pt)
    assert eg == ec
    assert qg == qc
    assert eg == cpu.evaluate_mle(cpu.mle_from_evaluations(nv, t), pt)


def test_kzg_errors(gpu, oracle, params):
    pg, _ = params
    big = gpu.mle_from_evaluations(11, oracle.random_fr(1, 1 << 11))
    with pytest.raises(InvalidParameters):
        gpu.commit(pg, big)
    with pytest.raises(InvalidParameters):
        gpu.open(pg, big, [1] * 11)
    small = gpu.mle_from_evaluations(2, oracle.random_fr(1, 4))
    with pytest.raises(InvalidParameters):
        gpu.open(pg, small, [1])
    with pytest.raises(InvalidParameters):
        gpu.prepare_prover_param(2, [b"\x00" * 97 * 4, b"\x00" * 97 * 2])
    bad = bytearray(oracle.affine_to_packets(oracle.srs_layers(1, 3)[0]))
    bad[0] = 7
    with pytest.raises(InvalidParameters):
        gpu.prepare_prover_param(1, [bytes(bad), oracle.affine_to_packets(oracle.g1_generator())])


@pytest.mark.parametrize("nv", [1, 3, 8])
def test_srs_generate_matches_oracle(gpu, oracle, nv):
    total = (1 << (nv + 1)) - 1
    out = (ctypes.c_uint8 * (97 * total))()
    check_status(gpu.lib.hp_cuda_v1_srs_generate(gpu.ctx.raw, nv, 21, out, total), "srs_generate")
    expect = b"".join(oracle.affine_to_packets(l) for l in oracle.srs_layers(nv, 21))
    assert bytes(out) == expect


def test_fixture_rng_matches_oracle(native_lib, oracle):
    out = (ctypes.c_uint8 * (32 * 5000))()
    check_status(native_lib.hp_cuda_v1_fixture_random_fr(3, 7, 5000, out), "fixture_random_fr")
    assert bytes(out) == oracle.random_fr(3, 5000, first=7)
