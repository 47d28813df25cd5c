"""CPU check of the identity behind the eq-factored zero-check rounds
(k_sumcheck_round_eq): with the previous challenges folded into every table,
a zero-check round polynomial is

    p(t) = eq1(t; r_i) * Q(t),  Q(t) = sum_b w_b g_b(t),  w_b = eq[2b] + eq[2b+1],

g the polynomial without its eq factor, Q of degree d - 1 (d nodes), and from
round 2 on Q(0) = (claim - r_i Q(1)) / (1 - r_i).  A plain-Python restatement
of those steps at small sizes must give the oracle's generic round messages
(poly_iop/zero_check/mod.rs builds f_hat = f * eq(x, r) before the sumcheck;
the oracle runs that generic sumcheck)."""
import random

import pytest

from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001

SHAPES = {
    "gate": [(1, [0, 5]), (1, [1, 6]), (1, [2, 7]), (1, [3, 5, 6]), (1, [4])],
    "prodcheck": [(1, [0]), (R - 1, [1, 2]), (0x1234567, [3, 4, 5, 6]), (R - 0x1234567, [7, 3, 4])],
    "degree2": [(5, [0]), (R - 3, [1]), (7, [])],
}


def lagrange_at(values, x):
    """The polynomial through (k, values[k]), k = 0..len-1, at x (mod R)."""
    n = len(values)
    acc = 0
    for j in range(n):
        num, den = 1, 1
        for m in range(n):
            if m != j:
                num = num * (x - m) % R
                den = den * (j - m) % R
        acc = (acc + values[j] * num * pow(den, R - 2, R)) % R
    return acc


def eq_round_messages(tables, eq, products, r, challenges, degree):
    """Round messages by the eq-factored identity; tables/eq: lists of ints."""
    tabs = [list(t) for t in tables]
    e = list(eq)
    msgs, claim = [], None
    for i, ch in enumerate(challenges):
        if i > 0:
            fold = lambda t: [(t[2 * b] + ch * (t[2 * b + 1] - t[2 * b])) % R for b in range(len(t) // 2)]
            tabs = [fold(t) for t in tabs]
            e = fold(e)
        pairs = len(e) // 2
        w = [(e[2 * b] + e[2 * b + 1]) % R for b in range(pairs)]

        def g(b, k):
            s = 0
            for c, ix in products:
                v = 1
                for f in ix:
                    lo, hi = tabs[f][2 * b], tabs[f][2 * b + 1]
                    v = v * (lo + k * (hi - lo)) % R
                s = (s + c * v) % R
            return s

        ri = r[i]
        use_claim = claim is not None and (1 - ri) % R != 0
        q = [None] * degree
        for k in range(1 if use_claim else 0, degree):
            q[k] = sum(w[b] * g(b, k) for b in range(pairs)) % R
        if use_claim:
            q[0] = (claim - ri * q[1]) * pow((1 - ri) % R, R - 2, R) % R
        msg = [((1 - ri) + x * (2 * ri - 1)) * lagrange_at(q, x) % R for x in range(degree + 1)]
        msgs.append(msg)
        nxt = challenges[i + 1] if i + 1 < len(challenges) else None
        claim = lagrange_at(msg, nxt) if nxt is not None else None
    return msgs


@pytest.mark.parametrize("shape", sorted(SHAPES))
@pytest.mark.parametrize("nv", [1, 2, 5])
def test_eq_identity_gives_the_generic_messages(oracle, cpu, shape, nv):
    rng = random.Random(nv * 7 + len(shape))
    n_mles = 8 if shape != "degree2" else 2
    raw = [oracle.random_fr(900 + j, 1 << nv) for j in range(n_mles)]
    tables = [oracle.frs_ints(t) for t in raw]
    r = [rng.randrange(R) for _ in range(nv)]
    if nv >= 2:
        r[1] = 1  # a round whose Q(0) cannot come from the claim
    ce = cpu.build_eq_x_r(r)
    eq = oracle.frs_ints(ce.evaluations)
    cm = [cpu.mle_from_evaluations(nv, t) for t in raw]
    vc = VirtualPolynomial(nv)
    for c, ix in SHAPES[shape]:
        vc.add_mle_list([cm[i] for i in ix] + [ce], c)
    degree = vc.aux_info.max_degree
    challenges = [None] + [rng.randrange(R) for _ in range(nv - 1)]
    sc = cpu.prover_init(vc)
    want = [cpu.prove_round_and_update_state(sc, ch) for ch in challenges]
    assert eq_round_messages(tables, eq, SHAPES[shape], r, challenges, degree) == want
