"""MSMs whose scalars are all 0 or 1 (the product-check tables frac and prod
of a circuit whose permutation is the identity) take the sum-of-bases path
(msm_binary_tasks / msm_run_binary in csrc/msm.cu); every result must equal
the oracle's, with the path taken only when every scalar is 0 or 1, and the
same results with the path switched off (HP_MSM_BINARY=0)."""
import ctypes
import random

import pytest

from hyperplonk_gb300.errors import check_status

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
ONE = (1).to_bytes(32, "little")
ZERO = bytes(32)


def binary_table(pattern: str, nv: int, seed: int) -> bytes:
    n = 1 << nv
    rng = random.Random(seed)
    if pattern == "ones":
        bits = [1] * n
    elif pattern == "zeros":
        bits = [0] * n
    elif pattern == "last":
        bits = [0] * (n - 1) + [1]
    elif pattern == "prod":  # a product table of the identity permutation: ones, then 0 in the last slot
        bits = [1] * (n - 1) + [0]
    elif pattern == "mostly":  # about 90% ones: the layer's base sum minus the zeros' bases
        bits = [int(rng.random() < 0.9) for _ in range(n)]
    else:
        bits = [rng.randrange(2) for _ in range(n)]
    return b"".join(ONE if b else ZERO for b in bits)


class Profile:
    """Launch counts of the library's named phases on the backend's context."""

    def __init__(self, gpu):
        self.gpu = gpu

    def __enter__(self):
        check_status(self.gpu.lib.hp_cuda_v1_context_profile(self.gpu.ctx.raw, 1), "context_profile")
        return self

    def launches(self, name: bytes) -> int:
        ms, n = ctypes.c_double(), ctypes.c_uint64()
        check_status(self.gpu.lib.hp_cuda_v1_context_profile_read(self.gpu.ctx.raw, name, ctypes.byref(ms),
                                                                 ctypes.byref(n)), "context_profile_read")
        return int(n.value)

    def __exit__(self, *exc):
        check_status(self.gpu.lib.hp_cuda_v1_context_profile(self.gpu.ctx.raw, 0), "context_profile")


@pytest.fixture(scope="module")
def srs(oracle):
    nv = 11
    return nv, oracle.srs_layers(nv, 61)


@pytest.fixture(scope="module")
def params(gpu, cpu, srs, oracle):
    nv, layers = srs
    return (gpu.prepare_prover_param(nv, [oracle.affine_to_packets(l) for l in layers]),
            cpu.prepare_prover_param(nv, layers))


# "ones", "prod" and "mostly" (more ones than zeros over a whole layer) are
# formed as the layer's precomputed base sum minus the bases of the zeros
@pytest.mark.parametrize("pattern", ["ones", "zeros", "last", "prod", "mostly", "bits"])
def test_binary_commits_match_oracle_and_take_the_sum_path(gpu, cpu, params, pattern):
    pg, pc = params
    for nv in range(0, 12):
        t = binary_table(pattern, nv, 100 + nv)
        with Profile(gpu) as prof:
            got = gpu.commit(pg, gpu.mle_from_evaluations(nv, t))
            assert prof.launches(b"msm_binary") == 1 and prof.launches(b"msm") == 0, (pattern, nv)
        assert got == cpu.commit(pc, cpu.mle_from_evaluations(nv, t)), (pattern, nv)


def test_one_large_scalar_keeps_the_full_path(gpu, cpu, params):
    pg, pc = params
    nv = 9
    for value in (2, R - 1):
        t = bytearray(binary_table("bits", nv, 7))
        t[32 * 300:32 * 301] = value.to_bytes(32, "little")
        with Profile(gpu) as prof:
            got = gpu.commit(pg, gpu.mle_from_evaluations(nv, bytes(t)))
            assert prof.launches(b"msm_binary") == 0 and prof.launches(b"msm") == 1
        assert got == cpu.commit(pc, cpu.mle_from_evaluations(nv, bytes(t)))


def test_multi_commit_mixes_binary_and_full_msms(gpu, cpu, params, oracle):
    pg, pc = params
    tables = [(11, binary_table("ones", 11, 1)), (11, oracle.random_fr(71, 1 << 11)),
              (10, binary_table("prod", 10, 2)), (6, binary_table("bits", 6, 3)),
              (8, oracle.random_fr(72, 1 << 8)), (0, ONE), (11, binary_table("zeros", 11, 4))]
    gm = [gpu.mle_from_evaluations(nv, t) for nv, t in tables]
    cm = [cpu.mle_from_evaluations(nv, t) for nv, t in tables]
    with Profile(gpu) as prof:
        got = gpu.multi_commit(pg, gm)
        assert prof.launches(b"msm_binary") == 5
    assert got == cpu.multi_commit(pc, cm)


def test_batch_msm_binary_prefixes(gpu, oracle, params, srs):
    pg, _ = params
    _, layers = srs
    dims = [3, 7, 9, 11, 5]
    tables = [binary_table("bits", d, 20 + d) for d in dims]
    got = gpu.batch_msm(pg, 0, [gpu.mle_from_evaluations(d, t) for d, t in zip(dims, tables)])
    for d, t, g in zip(dims, tables, got):
        assert g == oracle.affine_to_point(oracle.msm(layers[0][:96 * (1 << d)], t)), d


def test_switched_off_gives_the_same_points(gpu, cpu, params, monkeypatch):
    pg, pc = params
    t = binary_table("prod", 11, 5)
    on = gpu.commit(pg, gpu.mle_from_evaluations(11, t))
    monkeypatch.setenv("HP_MSM_BINARY", "0")
    with Profile(gpu) as prof:
        off = gpu.commit(pg, gpu.mle_from_evaluations(11, t))
        assert prof.launches(b"msm_binary") == 0 and prof.launches(b"msm") == 1
    assert on == off == cpu.commit(pc, cpu.mle_from_evaluations(11, t))
