"""GPU parity of the sumcheck prover state against the oracle, every round.

Mirrors backend/src/ascend910b3/integration_tests.rs
(sumcheck_round_messages_match_cpu_for_mixed_products,
sumcheck_repeated_factors_mixed_arity_max_degree_34_are_independent) and the
CPU KAT of backend/src/cpu/sum_check.rs:224-253."""
import random

import pytest

from hyperplonk_gb300.errors import InvalidParameters, InvalidState
from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def build_pair(gpu, cpu, oracle, nv, n_mles, products, seed):
    """products: list of (coef, [mle indices]) -> (gpu VP, cpu VP)."""
    tables = [oracle.random_fr(seed, 1 << nv, first=j << nv) for j in range(n_mles)]
    gm = [gpu.mle_from_evaluations(nv, t) for t in tables]
    cm = [cpu.mle_from_evaluations(nv, t) for t in tables]
    vg, vc = VirtualPolynomial(nv), VirtualPolynomial(nv)
    for coef, ix in products:
        vg.add_mle_list([gm[i] for i in ix], coef)
        vc.add_mle_list([cm[i] for i in ix], coef)
    return vg, vc, gm, cm


def run_both(gpu, cpu, vg, vc, seed):
    rng = random.Random(seed)
    sg, sc = gpu.prover_init(vg), cpu.prover_init(vc)
    ch = None
    for _ in range(vg.aux_info.num_variables):
        a = gpu.prove_round_and_update_state(sg, ch)
        b = cpu.prove_round_and_update_state(sc, ch)
        assert a == b
        ch = rng.randrange(R)
    assert gpu.final_evaluations(sg, ch) == cpu.final_evaluations(sc, ch)
    return sg, ch


def test_round_kat_and_ordering(gpu):
    mle = gpu.mle_from_evaluations(2, [2, 3, 5, 7])
    poly = VirtualPolynomial.new_from_mle(mle, 2)
    poly.add_mle_list([mle, mle], 3)
    st = gpu.prover_init(poly)
    with pytest.raises(InvalidState):
        gpu.prove_round_and_update_state(st, 2)
    assert gpu.prove_round_and_update_state(st, None) == [101, 194, 317]
    with pytest.raises(InvalidState):
        gpu.prove_round_and_update_state(st, None)
    assert gpu.prove_round_and_update_state(st, 2) == [56, 261, 616]
    with pytest.raises(InvalidState):
        gpu.prove_round_and_update_state(st, 2)
    assert gpu.download(mle) == b"".join(v.to_bytes(32, "little") for v in (2, 3, 5, 7))


# nv <= 14: every round in the wide (slot, pair) kernel, from unfolded inputs
# on; nv = 16: the first two rounds in the grid kernel, whose folded tables
# the wide kernel then reads
@pytest.mark.parametrize("nv", [1, 2, 3, 10, 14, 16])
def test_degree2_four_products_over_six_mles(gpu, cpu, oracle, nv):
    rng = random.Random(nv)
    prods = [(rng.randrange(R), [0, 1]), (rng.randrange(R), [2, 3]), (rng.randrange(R), [4, 5]),
             (rng.randrange(R), [0, 3])]
    vg, vc, _, _ = build_pair(gpu, cpu, oracle, nv, 6, prods, 1)
    run_both(gpu, cpu, vg, vc, nv)


def test_mixed_products(gpu, cpu, oracle):
    nv = 9
    prods = [(5, [0, 1, 2]), (7, [3]), (R - 1, [1, 1]), (11, [4, 0, 2, 3]), (0, [2, 4])]
    vg, vc, _, _ = build_pair(gpu, cpu, oracle, nv, 5, prods, 2)
    run_both(gpu, cpu, vg, vc, 9)


def test_mixed_arity_large_rounds(gpu, cpu, oracle):
    """Arity 1..5 products at nv = 15: the first rounds run the fold kernel
    and the (slot, pair) kernel over the folded tables (arity-1 slots take
    the shifted accumulator, arity 5 the <6> instantiation), the later ones
    the fused and one-block kernels."""
    nv = 15
    prods = [(3, [0]), (R - 2, [1, 2]), (5, [2, 3, 4]), (7, [0, 5, 1, 6]), (11, [6, 5, 4, 3, 2]), (13, [1])]
    vg, vc, _, _ = build_pair(gpu, cpu, oracle, nv, 7, prods, 7)
    run_both(gpu, cpu, vg, vc, 15)


# Rounds after the first take p(0) from the previous round's claim, and
# products whose arity equals the degree drop their t = 0 slot.  nv = 18
# reaches the (product, pair) kernel (>= 2^16 pairs): arity 3 everywhere takes
# its reduced form, arity 2 next to arity 3 keeps the full layout there and
# per-product first nodes in the resident grid; the native transcript runs
# prove_rounds (resident from 2^15 pairs), the oracle one round at a time.
REDUCED_SHAPES = {
    "arity3": [(3, [0, 1, 2]), (5, [3, 4, 5]), (R - 7, [0, 3, 5])],
    "mixed23": [(3, [0, 1, 2]), (5, [3, 4]), (R - 7, [1, 5]), (11, [2, 4, 5])],
}


@pytest.mark.parametrize("shape", sorted(REDUCED_SHAPES))
def test_reduced_layout_rounds_nv18(gpu, cpu, oracle, shape):
    vg, vc, _, _ = build_pair(gpu, cpu, oracle, 18, 6, REDUCED_SHAPES[shape], 91)
    run_both(gpu, cpu, vg, vc, 18)


@pytest.mark.parametrize("shape", sorted(REDUCED_SHAPES))
def test_prove_rounds_reduced_layout_nv18(gpu, cpu, oracle, shape):
    import transcript_ref as tref
    from hyperplonk_gb300 import protocol
    from hyperplonk_gb300.transcript import IOPTranscript
    vg, vc, _, _ = build_pair(gpu, cpu, oracle, 18, 6, REDUCED_SHAPES[shape], 92)
    fg, fc = [], []
    pg = protocol.sumcheck_prove(gpu, vg, IOPTranscript(b"reduced layout"), fg)
    pc = protocol.sumcheck_prove(cpu, vc, tref.OracleIOPTranscript(b"reduced layout"), fc)
    assert pg.proofs == pc.proofs
    assert pg.point == pc.point
    assert fg == fc


def test_repeated_factors_max_degree_34(gpu, cpu, oracle):
    nv = 6
    prods = [(3, [0] * 34), (5, [1, 0, 1]), (R - 7, [2] * 17 + [1] * 10), (9, [2])]
    vg, vc, _, _ = build_pair(gpu, cpu, oracle, nv, 3, prods, 3)
    assert vg.aux_info.max_degree == 34
    run_both(gpu, cpu, vg, vc, 34)


@pytest.mark.parametrize("nv", [11, 15])
def test_zerocheck_shape_degree4(gpu, cpu, oracle, nv):
    """Gate polynomial times eq: q_L w1 + q_R w2 + q_O w3 + q_M w1 w2 + q_C, x eq."""
    # 0..4 selectors, 5..7 witnesses, 8 eq
    prods = [(1, [0, 5, 8]), (1, [1, 6, 8]), (1, [2, 7, 8]), (1, [3, 5, 6, 8]), (1, [4, 8])]
    vg, vc, _, _ = build_pair(gpu, cpu, oracle, nv, 9, prods, 4)
    run_both(gpu, cpu, vg, vc, 4)


def test_empty_sum_and_state_independence(gpu, cpu, oracle):
    nv = 4
    vg = VirtualPolynomial(nv)
    vg.aux_info.max_degree = 2
    st = gpu.prover_init(vg)
    assert gpu.prove_round_and_update_state(st, None) == [0, 0, 0]
    # two states over the same factors advance independently
    prods = [(1, [0, 1])]
    vg, vc, gm, _ = build_pair(gpu, cpu, oracle, 6, 2, prods, 5)
    s1, s2 = gpu.prover_init(vg), gpu.prover_init(vg)
    a = gpu.prove_round_and_update_state(s1, None)
    gpu.prove_round_and_update_state(s1, 3)
    b = gpu.prove_round_and_update_state(s2, None)
    assert a == b


def test_state_outlives_retired_inputs(gpu, cpu, oracle):
    nv = 8
    prods = [(2, [0, 1]), (3, [1])]
    vg, vc, gm, cm = build_pair(gpu, cpu, oracle, nv, 2, prods, 6)
    sg, sc = gpu.prover_init(vg), cpu.prover_init(vc)
    del vg, gm  # drop every Python handle: the buffers are retired
    import gc
    gc.collect()
    ch = None
    rng = random.Random(1)
    for _ in range(nv):
        assert gpu.prove_round_and_update_state(sg, ch) == cpu.prove_round_and_update_state(sc, ch)
        ch = rng.randrange(R)


def test_invalid_descriptions(gpu, oracle):
    vg = VirtualPolynomial(0)
    vg.aux_info.max_degree = 1
    with pytest.raises(InvalidParameters):
        gpu.prover_init(vg)
    m = gpu.mle_from_evaluations(2, oracle.random_fr(1, 4))
    vg = VirtualPolynomial.new_from_mle(m, 1)
    vg.aux_info.max_degree = 0
    with pytest.raises(InvalidParameters):
        gpu.prover_init(vg)
