"""GPU parity of the eq-factored zero-check rounds against the oracle.

A prover state whose products all contain one factor exactly once, that
factor an eq table built by build_eq_x_r (the reference's zero-check,
poly_iop/zero_check/mod.rs: f_hat = f * eq(x, r) before the sumcheck),
takes k_sumcheck_round_eq for its large rounds: the round polynomial is
eq1(t; r_i) Q(t) with Q read off the folded eq table.  Every message must
equal the oracle's, which runs the generic sumcheck on the same products."""
import ctypes
import random

import pytest

from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
ALPHA = 0x1234567890ABCDEF1234567890ABCDEF

# (coefficient, factor indices); index "e" is the eq table
SHAPES = {
    # the vanilla gate (q_L w1 + q_R w2 + q_O w3 + q_M w1 w2 + q_C) times eq: degree 4
    "gate": [(1, [0, 5, "e"]), (1, [1, 6, "e"]), (1, [2, 7, "e"]), (1, [3, 5, 6, "e"]), (1, [4, "e"])],
    # the product check's Q = prod - p1 p2 + alpha g1 g2 g3 frac - alpha f1 f2 f3, times eq: degree 5
    "prodcheck": [(1, [0, "e"]), (R - 1, [1, 2, "e"]), (ALPHA, [3, 4, 5, 6, "e"]), (R - ALPHA, [7, 3, 4, "e"])],
    # degree 2, and a product that is the eq table alone
    "degree2": [(5, [0, "e"]), (R - 3, [1, "e"]), (7, ["e"])],
}
N_MLES = {"gate": 8, "prodcheck": 8, "degree2": 2}


def build(gpu, cpu, oracle, nv, shape, seed, eq_twice=False, eq_plain=False):
    rng = random.Random(seed)
    r = [rng.randrange(R) for _ in range(nv)]
    tables = [oracle.random_fr(seed, 1 << nv, first=j << nv) for j in range(N_MLES[shape])]
    gm = [gpu.mle_from_evaluations(nv, t) for t in tables]
    cm = [cpu.mle_from_evaluations(nv, t) for t in tables]
    ce = cpu.build_eq_x_r(r)
    ge = gpu.mle_from_evaluations(nv, ce.evaluations) if eq_plain else gpu.build_eq_x_r(r)
    vg, vc = VirtualPolynomial(nv), VirtualPolynomial(nv)
    for k, (coef, ix) in enumerate(SHAPES[shape]):
        ix = list(ix) + (["e"] if eq_twice and k == 0 else [])
        vg.add_mle_list([ge if i == "e" else gm[i] for i in ix], coef)
        vc.add_mle_list([ce if i == "e" else cm[i] for i in ix], coef)
    return vg, vc


def eq_rounds(gpu):
    ms, n = ctypes.c_double(), ctypes.c_uint64()
    assert gpu.lib.hp_cuda_v1_context_profile_read(gpu.ctx.raw, b"sumcheck_round_eq", ctypes.byref(ms),
                                                   ctypes.byref(n)).kind == 0
    return n.value


def run_rounds(gpu, cpu, vg, vc, seed):
    rng = random.Random(seed)
    sg, sc = gpu.prover_init(vg), cpu.prover_init(vc)
    ch = None
    for _ in range(vg.aux_info.num_variables):
        assert gpu.prove_round_and_update_state(sg, ch) == cpu.prove_round_and_update_state(sc, ch)
        ch = rng.randrange(R)
    assert gpu.final_evaluations(sg, ch) == cpu.final_evaluations(sc, ch)


@pytest.fixture
def profiled(gpu, monkeypatch):
    monkeypatch.delenv("HP_SUMCHECK_EQ", raising=False)  # these tests count eq launches
    gpu.lib.hp_cuda_v1_context_profile(gpu.ctx.raw, 1)
    yield gpu
    gpu.lib.hp_cuda_v1_context_profile(gpu.ctx.raw, 0)


@pytest.mark.parametrize("shape", sorted(SHAPES))
@pytest.mark.parametrize("nv,min_pairs", [(3, "1"), (9, "1"), (15, None)])
def test_eq_rounds_match_the_oracle(profiled, cpu, oracle, monkeypatch, shape, nv, min_pairs):
    """min_pairs 1: every round through the eq kernel (1 to 2^(nv-1) pairs,
    round 1 without a claim, the others with Q(0) from it); nv = 15: the
    built-in threshold (rounds of >= 2^13 pairs)."""
    gpu = profiled
    if min_pairs is not None:
        monkeypatch.setenv("HP_SUMCHECK_EQ_MIN_PAIRS", min_pairs)
    vg, vc = build(gpu, cpu, oracle, nv, shape, 100 + nv)
    run_rounds(gpu, cpu, vg, vc, nv)
    assert eq_rounds(gpu) == (nv if min_pairs else 2)


def test_eq_round_with_r_equal_one(profiled, cpu, oracle, monkeypatch):
    """r_2 = 1: round 2's Q(0) cannot come from the claim (1 - r_2 = 0) and
    the kernel evaluates it; the other rounds take the claim."""
    gpu = profiled
    monkeypatch.setenv("HP_SUMCHECK_EQ_MIN_PAIRS", "1")
    nv = 8
    rng = random.Random(77)
    r = [rng.randrange(R) for _ in range(nv)]
    r[1] = 1
    tables = [oracle.random_fr(300 + j, 1 << nv) for j in range(N_MLES["gate"])]
    gm = [gpu.mle_from_evaluations(nv, t) for t in tables]
    cm = [cpu.mle_from_evaluations(nv, t) for t in tables]
    ge, ce = gpu.build_eq_x_r(r), cpu.build_eq_x_r(r)
    vg, vc = VirtualPolynomial(nv), VirtualPolynomial(nv)
    for coef, ix in SHAPES["gate"]:
        vg.add_mle_list([ge if i == "e" else gm[i] for i in ix], coef)
        vc.add_mle_list([ce if i == "e" else cm[i] for i in ix], coef)
    run_rounds(gpu, cpu, vg, vc, 8)
    assert eq_rounds(gpu) == nv


@pytest.mark.parametrize("variant", ["eq_twice", "eq_plain"])
def test_other_eq_uses_stay_generic(profiled, cpu, oracle, monkeypatch, variant):
    """eq twice in one product, or an eq table uploaded as a plain table (no
    recorded point): the generic rounds, the same messages."""
    gpu = profiled
    monkeypatch.setenv("HP_SUMCHECK_EQ_MIN_PAIRS", "1")
    vg, vc = build(gpu, cpu, oracle, 10, "gate", 7, **{variant: True})
    run_rounds(gpu, cpu, vg, vc, 10)
    assert eq_rounds(gpu) == 0


@pytest.mark.parametrize("shape", ["gate", "prodcheck"])
def test_zerocheck_prove_nv18_matches_the_oracle(gpu, cpu, oracle, shape):
    """protocol.zerocheck_prove through prove_rounds (native transcript): the
    eq rounds (2^17 .. 2^15 pairs here), then the resident launch over the
    tables they folded; the oracle runs the generic sumcheck round by round."""
    import transcript_ref as tref
    from hyperplonk_gb300 import protocol
    from hyperplonk_gb300.transcript import IOPTranscript
    nv = 18
    tables = [oracle.random_fr(200 + j, 1 << nv) for j in range(N_MLES[shape])]
    gm = [gpu.mle_from_evaluations(nv, t) for t in tables]
    cm = [cpu.mle_from_evaluations(nv, t) for t in tables]
    vg, vc = VirtualPolynomial(nv), VirtualPolynomial(nv)
    for coef, ix in SHAPES[shape]:
        if "e" in ix and len(ix) == 1:
            continue
        vg.add_mle_list([gm[i] for i in ix if i != "e"], coef)
        vc.add_mle_list([cm[i] for i in ix if i != "e"], coef)
    tg, tc = IOPTranscript(b"eq rounds"), tref.OracleIOPTranscript(b"eq rounds")
    for t in (tg, tc):
        t.append_message(b"circuit", b"zero-check test")
    pg = protocol.zerocheck_prove(gpu, vg, tg)
    pc = protocol.zerocheck_prove(cpu, vc, tc)
    assert pg.proofs == pc.proofs
    assert pg.point == pc.point
