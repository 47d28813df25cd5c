"""Pins the oracle (oracle/hp_oracle.c) against the reference's golden vectors
(backend/src/ascend910b3/native/tests/generate_golden.py output, packed by
tests/golden/make_golden.py) and against the reference's own known-answer
tests.  CPU only."""
import hashlib
import random

import numpy as np
import pytest

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
Q = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB

OPS = {"add": 0, "sub": 1, "mul": 2, "neg": 3, "square": 4}


def _cases(npz):
    return sorted({k.split("/")[0] for k in npz.files})


@pytest.mark.parametrize("field", ["fr", "fq"])
def test_field_ops_match_golden(oracle, golden, field):
    npz = getattr(golden, field)
    width = 32 if field == "fr" else 48
    fid = 0 if field == "fr" else 1
    checked = 0
    for case in _cases(npz):
        lhs = npz[f"{case}/lhs"].tobytes()
        rhs = npz[f"{case}/rhs"].tobytes()
        n = len(lhs) // width
        for name, op in OPS.items():
            got = oracle.field_op(fid, op, lhs, rhs, n)
            assert got == npz[f"{case}/{name}"].tobytes(), (field, case, name)
            checked += n
        if f"{case}/inverse" in npz.files:
            inp = npz[f"{case}/inverse_input"].tobytes()
            got = oracle.field_op(fid, 5, inp, None, len(inp) // width)
            assert got == npz[f"{case}/inverse"].tobytes(), (field, case, "inverse")
    assert checked > 1000


def test_wide_reduction_matches_golden(oracle, golden):
    # 64-byte inputs of the Fr fixture are from_le_bytes_mod_order inputs
    wide = golden.wide["fr/wide_input"].tobytes()
    expect = golden.wide["fr/wide_result"].tobytes()
    width_in = len(wide) // 512
    assert width_in == 68  # 2*32 + 4 byte values; reduce the low 64 bytes only when the top is zero
    ins, outs = [], []
    for i in range(512):
        v = wide[width_in * i:width_in * (i + 1)]
        if any(v[64:]):
            continue
        ins.append(v[:64])
        outs.append(expect[32 * i:32 * i + 32])
    got = oracle.fr_from_wide(b"".join(ins))
    assert got == b"".join(outs)
    assert len(ins) >= 4


def test_from_le_bytes_mod_order_random(oracle):
    rng = random.Random(7)
    vals = [rng.getrandbits(512) for _ in range(300)] + [0, R, 2 * R, (1 << 512) - 1, R - 1]
    got = oracle.fr_from_wide(b"".join(v.to_bytes(64, "little") for v in vals))
    assert [int.from_bytes(got[32 * i:32 * i + 32], "little") for i in range(len(vals))] == [v % R for v in vals]


def test_g1_ops_match_golden(oracle, golden):
    g = golden.g1
    assert oracle.g1_generator() == g["generator"].tobytes()
    cases = sorted({k.split("/")[0] for k in g.files if k.startswith("case-")})
    assert len(cases) >= 10
    for case in cases:
        a = g[f"{case}/affine_a"].tobytes()
        b = g[f"{case}/affine_b"].tobytes()
        if not a:
            continue
        assert oracle.g1_op(0, a, b) == g[f"{case}/add"].tobytes(), case
        assert oracle.g1_op(1, a) == g[f"{case}/double"].tobytes(), case
        assert oracle.g1_op(2, a) == g[f"{case}/neg"].tobytes(), case
        k = np.frombuffer(g[f"{case}/mul_u64"].tobytes(), dtype=np.uint64).tolist()
        assert oracle.g1_op(3, a, k=k) == g[f"{case}/mul"].tobytes(), case


def test_g1_chain_msm_match_golden(oracle, golden):
    g = golden.g1
    chains = sorted({k.split("/")[1] for k in g.files if k.startswith("chain/")})
    assert len(chains) == 8
    for c in chains:
        bases = g[f"chain/{c}/bases"].tobytes()
        scalars = g[f"chain/{c}/scalars"].tobytes()
        assert oracle.msm(bases, scalars) == g[f"chain/{c}/expected"].tobytes(), c


def consecutive_bases(oracle, n):
    gen = oracle.g1_generator()
    return oracle.g1_op(3, gen * n, k=list(range(1, n + 1)))


def msm_case(oracle, msm_npz, key):
    """(bases, scalars, expected) of one MSM golden case, rebuilding large
    inputs and checking their digests."""
    files = msm_npz.files
    if f"{key}/bases" in files:
        bases = msm_npz[f"{key}/bases"].tobytes()
    else:
        n = int(msm_npz[f"{key}/bases_consecutive"][0])
        bases = consecutive_bases(oracle, n)
        assert hashlib.sha256(bases).digest() == msm_npz[f"{key}/bases_sha256"].tobytes()
    if f"{key}/scalars" in files:
        scalars = msm_npz[f"{key}/scalars"].tobytes()
    else:
        n = len(bases) // 96
        if f"{key}/scalars_ones" in files:
            vals = [1] * n
        else:
            rng = random.Random(int(msm_npz[f"{key}/scalars_pyrandom_seed"][0]))
            vals = [rng.randrange(R) for _ in range(n)]
        scalars = b"".join(v.to_bytes(32, "little") for v in vals)
        assert hashlib.sha256(scalars).digest() == msm_npz[f"{key}/scalars_sha256"].tobytes()
    return bases, scalars, msm_npz[f"{key}/expected"].tobytes()


def msm_keys(msm_npz):
    return sorted({"/".join(k.split("/")[:2]) for k in msm_npz.files})


def test_msm_matches_golden(oracle, golden):
    keys = msm_keys(golden.msm)
    assert len(keys) == 40
    for key in keys:
        bases, scalars, expected = msm_case(oracle, golden.msm, key)
        assert oracle.msm(bases, scalars) == expected, key


# ---------------------------------------------------------------------------
# Known-answer tests restated from the reference's CPU backend tests
# ---------------------------------------------------------------------------

def test_sumcheck_round_kat(cpu):
    """backend/src/cpu/sum_check.rs:224-253: MLE [2,3,5,7], 2f + 3f^2."""
    from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial
    mle = cpu.mle_from_evaluations(2, [2, 3, 5, 7])
    poly = VirtualPolynomial.new_from_mle(mle, 2)
    poly.add_mle_list([mle, mle], 3)
    st = cpu.prover_init(poly)
    with pytest.raises(Exception):
        cpu.prove_round_and_update_state(st, 2)
    assert cpu.prove_round_and_update_state(st, None) == [101, 194, 317]
    with pytest.raises(Exception):
        cpu.prove_round_and_update_state(st, None)
    assert cpu.prove_round_and_update_state(st, 2) == [56, 261, 616]
    with pytest.raises(Exception):
        cpu.prove_round_and_update_state(st, 2)


def test_mle_kats(cpu):
    """backend/src/cpu/multilinear_polynomial.rs:278-593."""
    p = cpu.mle_from_evaluations(2, [2, 3, 5, 7])
    q = cpu.mle_from_evaluations(2, [11, 13, 17, 19])
    assert cpu.evaluate_mle(p, [2, 3]) == 19
    comb = cpu.linear_combination([p, q, p], [2, 3, R - 2])
    assert cpu.evaluate_mle(comb, [2, 3]) == 99
    assert cpu.evaluate_mle(q, [2, 3]) == 33
    for nv, vals, expect in [(1, [2, 3], [6, 0]), (2, [2, 3, 5, 7], [6, 35, 210, 0]),
                             (3, [2, 3, 5, 7, 11, 13, 17, 19], [6, 35, 143, 323, 210, 46189, 9699690, 0])]:
        frac = cpu.mle_from_evaluations(nv, vals)
        prod = cpu.compute_product_poly(frac)
        from oracle import frs_ints
        assert frs_ints(prod.evaluations) == expect
    frac = cpu.mle_from_evaluations(2, [2, 3, 5, 7])
    prod = cpu.mle_from_evaluations(2, [11, 13, 17, 19])
    p1, p2 = cpu.compute_product_factors(frac, prod)
    from oracle import frs_ints
    assert frs_ints(p1.evaluations) == [2, 5, 11, 17]
    assert frs_ints(p2.evaluations) == [3, 7, 13, 19]
    fxs = [cpu.mle_from_evaluations(0, [v]) for v in (2, 3, 5)]
    gxs = [cpu.mle_from_evaluations(0, [v]) for v in (7, 11, 13)]
    perms = [cpu.mle_from_evaluations(0, [v]) for v in (2, 0, 1)]
    nums, dens = cpu.compute_nums_and_denoms(2, 3, fxs, gxs, perms)
    assert [frs_ints(n.evaluations)[0] for n in nums] == [5, 8, 12]
    assert [frs_ints(d.evaluations)[0] for d in dens] == [14, 14, 18]


def test_nums_denoms_column_offsets(cpu):
    """multilinear_polynomial.rs:438-491: identity term beta*(4*column + row)."""
    from oracle import frs_ints
    fxs = [cpu.mle_from_evaluations(2, [2 + i, 3 + i, 5 + i, 7 + i]) for i in range(3)]
    gxs = [cpu.mle_from_evaluations(2, [0, 11 + i, 13 + i, 17 + i]) for i in range(3)]
    perms = [cpu.mle_from_evaluations(2, [11 - 4 * i, 10 - 4 * i, 9 - 4 * i, 8 - 4 * i]) for i in range(3)]
    for beta, gamma in [(2, 5), (0, 5), (R - 2, 0), (0, 0)]:
        nums, dens = cpu.compute_nums_and_denoms(beta, gamma, fxs, gxs, perms)
        for c in range(3):
            f = frs_ints(fxs[c].evaluations)
            g = frs_ints(gxs[c].evaluations)
            pm = frs_ints(perms[c].evaluations)
            assert frs_ints(nums[c].evaluations) == [(f[r] + beta * (4 * c + r) + gamma) % R for r in range(4)]
            assert frs_ints(dens[c].evaluations) == [(g[r] + beta * pm[r] + gamma) % R for r in range(4)]


def test_frac_kat_and_zero_denominator(cpu):
    from oracle import OracleInvalidParameters, frs_ints
    f = cpu.mle_from_evaluations(2, [2, 3, 5, 7])
    g = cpu.mle_from_evaluations(2, [1, 3, 10, 14])
    frac = cpu.compute_frac_poly([f], [g])
    got = frs_ints(frac.evaluations)
    assert got == [2, 1, (5 * pow(10, -1, R)) % R, (7 * pow(14, -1, R)) % R]
    z = cpu.mle_from_evaluations(2, [1, 0, 3, 4])
    with pytest.raises(OracleInvalidParameters):
        cpu.compute_frac_poly([f], [z])


def test_eq_table_matches_naive(cpu):
    """common/eq.rs:105-151: eq(x, r) = prod (x_i r_i + (1-x_i)(1-r_i)), r[0] <-> bit 0."""
    from oracle import frs_ints
    rng = random.Random(11)
    for nv in range(1, 8):
        r = [rng.randrange(R) for _ in range(nv)]
        eq = frs_ints(cpu.build_eq_x_r(r).evaluations)
        for x in range(1 << nv):
            v = 1
            for i in range(nv):
                v = v * (r[i] if (x >> i) & 1 else (1 - r[i])) % R
            assert eq[x] == v


def test_evaluate_is_multilinear_extension(cpu):
    from oracle import frs_bytes
    rng = random.Random(3)
    for nv in (1, 3, 6):
        vals = [rng.randrange(R) for _ in range(1 << nv)]
        pt = [rng.randrange(R) for _ in range(nv)]
        mle = cpu.mle_from_evaluations(nv, frs_bytes(vals))
        # sum_x f(x) eq(x, pt)
        expect = 0
        for x in range(1 << nv):
            w = 1
            for i in range(nv):
                w = w * (pt[i] if (x >> i) & 1 else (1 - pt[i])) % R
            expect = (expect + vals[x] * w) % R
        assert cpu.evaluate_mle(mle, pt) == expect


def test_sumcheck_messages_are_consistent(cpu):
    """Round messages satisfy s_k(0) + s_k(1) = s_{k-1}(r_{k-1}) (checked by
    direct Lagrange evaluation here, independent of the oracle's extrapolation)."""
    from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial
    from oracle import frs_bytes
    rng = random.Random(5)
    nv = 5
    mles = [cpu.mle_from_evaluations(nv, frs_bytes([rng.randrange(R) for _ in range(1 << nv)])) for _ in range(4)]
    vp = VirtualPolynomial(nv)
    vp.add_mle_list([mles[0], mles[1], mles[2]], 7)
    vp.add_mle_list([mles[3]], 5)
    vp.add_mle_list([mles[1], mles[1]], 3)
    st = cpu.prover_init(vp)
    d = vp.aux_info.max_degree

    def lagrange(vals, x):
        tot = 0
        for j, v in enumerate(vals):
            num, den = 1, 1
            for i in range(len(vals)):
                if i != j:
                    num = num * (x - i) % R
                    den = den * (j - i) % R
            tot = (tot + v * num * pow(den, -1, R)) % R
        return tot

    claim = None
    ch = None
    for _ in range(nv):
        msg = cpu.prove_round_and_update_state(st, ch)
        assert len(msg) == d + 1
        if claim is not None:
            assert (msg[0] + msg[1]) % R == claim
        ch = rng.randrange(R)
        claim = lagrange(msg, ch)
    finals = cpu.final_evaluations(st, ch)
    # the final claim equals the VP evaluated at the final folded factor values
    f = finals
    expect = (7 * f[0] * f[1] * f[2] + 5 * f[3] + 3 * f[1] * f[1]) % R
    assert claim == expect


def test_srs_layers_are_eq_structured(oracle):
    """Layer i of the testing SRS is g * eq(t[i..], x): the first point of each
    layer is g * prod(1 - t_j); layer nv is [g] (srs.rs:158-235)."""
    from oracle import frs_ints
    nv = 4
    layers = oracle.srs_layers(nv, 9)
    assert [len(l) // 96 for l in layers] == [16, 8, 4, 2, 1]
    blocks = [oracle.chacha20_block(9, i) for i in range(nv + 1)]
    t = [int.from_bytes(b, "little") % R for b in blocks]
    g = layers[nv]
    for i in range(nv):
        s = 1
        for j in range(i, nv):
            s = s * (1 - t[j]) % R
        # g * s via the oracle's MSM of one point
        assert oracle.msm(g, s.to_bytes(32, "little")) == layers[i][:96]
    # every point of layer 0 matches g * eq(t, x)
    eq = frs_ints(oracle.CpuBackend().build_eq_x_r(t[:nv]).evaluations)
    for x in range(16):
        assert oracle.msm(g, eq[x].to_bytes(32, "little")) == layers[0][96 * x:96 * x + 96]
