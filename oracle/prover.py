"""TEST INFRASTRUCTURE ONLY -- the oracle's own HyperPlonk prover.

An independent restatement of the reference's prover-side protocol over the
oracle's CPU backend (oracle.py / hp_oracle.c) and the oracle's pure-Python
Merlin transcript (transcript_ref.py).  It imports nothing from the product
package, so a parity test that compares the GB300 prover's bytes with this
prover's bytes compares two separately written drivers, and the CPU reference
timing runs no product code.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU legs use it.

Follows:
- VirtualPolynomial add_mle_list / mul_by_mle:  backend/src/virtual_polynomial.rs:126-234
- SumCheck prove:       subroutines/src/poly_iop/sum_check/mod.rs:130-169
- ZeroCheck prove:      subroutines/src/poly_iop/zero_check/mod.rs:70-92
- ProductCheck prove:   subroutines/src/poly_iop/prod_check/mod.rs:150-212, util.rs:24-65
- PermutationCheck:     subroutines/src/poly_iop/perm_check/mod.rs:105-158
- batch opening:        subroutines/src/pcs/multilinear_kzg/batching.rs:33-194
- HyperPlonk prove:     hyperplonk/src/snark.rs:156-341, utils.rs:16-86, 179-227
- vanilla gate:         hyperplonk/src/custom_gate.rs:86-96

Proof bytes: every HyperPlonkProof field in declaration order
(hyperplonk/src/structs.rs:21-38) in ark-serialize's compressed conventions
(u64 LE lengths, Fr 32-byte LE, G1 48-byte big-endian x with flag bits 0x80
compressed / 0x40 infinity / 0x20 larger y); the reference's proof structs
carry no serialization of their own.
"""
from __future__ import annotations

import numpy as np

import oracle as orc
import transcript_ref as tref

R = orc.R
Q = orc.Q

# (coefficient, selector index or None, witness indices): custom_gate.rs:86-96
VANILLA_GATE = [(1, 0, [0]), (1, 1, [1]), (1, 2, [2]), (1, 3, [0, 1]), (1, 4, [])]


# ---------------------------------------------------------------------------
# serialization
# ---------------------------------------------------------------------------

def usize(n: int) -> bytes:
    return int(n).to_bytes(8, "little")


def fr(x: int) -> bytes:
    return (x % R).to_bytes(32, "little")


def vec_fr(xs) -> bytes:
    xs = list(xs)
    return usize(len(xs)) + b"".join(fr(x) for x in xs)


def g1_compressed(p) -> bytes:
    """ark-bls12-381 compressed G1: 48-byte big-endian x, flags in byte 0."""
    if p is None:
        return bytes([0xC0]) + bytes(47)
    x, y = p
    b = bytearray(x.to_bytes(48, "big"))
    b[0] |= 0x80
    if 2 * y > Q - 1:  # y is the lexicographically larger of the two roots
        b[0] |= 0x20
    return bytes(b)


def vec_g1(ps) -> bytes:
    ps = list(ps)
    return usize(len(ps)) + b"".join(g1_compressed(p) for p in ps)


def iop_proof_bytes(point, msgs) -> bytes:
    return vec_fr(point) + usize(len(msgs)) + b"".join(vec_fr(m) for m in msgs)


# ---------------------------------------------------------------------------
# virtual polynomial (products over identity-deduplicated factors)
# ---------------------------------------------------------------------------

class _Aux:
    def __init__(self, num_variables: int):
        self.max_degree = 0
        self.num_variables = num_variables


class VP:
    """Sum of coefficient * product of MLEs; factors deduplicated by object
    identity in first-insertion order (virtual_polynomial.rs:154-234)."""

    def __init__(self, num_vars: int):
        self.aux_info = _Aux(num_vars)
        self.products: list = []
        self._flat: list = []
        self._lookup: dict = {}

    def flattened_ml_extensions(self) -> list:
        return self._flat

    def _index(self, mle) -> int:
        k = id(mle)
        if k not in self._lookup:
            self._lookup[k] = len(self._flat)
            self._flat.append(mle)
        return self._lookup[k]

    def add_mle_list(self, mles, coefficient: int) -> None:
        mles = list(mles)
        if not mles:
            raise ValueError("input mle_list is empty")
        if any(m.num_vars != self.aux_info.num_variables for m in mles):
            raise ValueError("product has a multiplicand with wrong number of variables")
        self.aux_info.max_degree = max(self.aux_info.max_degree, len(mles))
        self.products.append((coefficient % R, [self._index(m) for m in mles]))

    def mul_by_mle(self, mle, coefficient: int) -> None:
        if mle.num_vars != self.aux_info.num_variables:
            raise ValueError("product has a multiplicand with wrong number of variables")
        idx = self._index(mle)
        self.products = [(c * coefficient % R, ix + [idx]) for c, ix in self.products]
        self.aux_info.max_degree += 1

    def copy(self) -> "VP":
        out = VP(self.aux_info.num_variables)
        out.aux_info.max_degree = self.aux_info.max_degree
        out.products = [(c, list(ix)) for c, ix in self.products]
        out._flat = list(self._flat)
        out._lookup = dict(self._lookup)
        return out


# ---------------------------------------------------------------------------
# PolyIOP
# ---------------------------------------------------------------------------

def sumcheck_prove(cpu, vp: VP, tr, final_evaluations: list | None = None):
    """Returns (point, messages).  With `final_evaluations` a list, the
    factor values at the final point are appended to it (one extra fold of
    the last challenge, as callers obtain them with evaluate_mle)."""
    nv, d = vp.aux_info.num_variables, vp.aux_info.max_degree
    if nv == 0 or d == 0:
        raise ValueError("SumCheck requires positive variable count and degree.")
    tr.append_serializable_element(b"aux info", usize(d) + usize(nv))
    state = cpu.prover_init(vp)
    challenge, point, msgs = None, [], []
    for _ in range(nv):
        msg = cpu.prove_round_and_update_state(state, challenge)
        tr.append_serializable_element(b"prover msg", vec_fr(msg))
        msgs.append(msg)
        challenge = tr.get_and_append_challenge(b"Internal round")
        point.append(challenge)
    if final_evaluations is not None:
        final_evaluations.extend(cpu.final_evaluations(state, challenge))
    return point, msgs


def zerocheck_prove(cpu, vp: VP, tr):
    r = tr.get_and_append_challenge_vectors(b"0check r", vp.aux_info.num_variables)
    f_hat = vp.copy()
    f_hat.mul_by_mle(cpu.build_eq_x_r(r), 1)
    return sumcheck_prove(cpu, f_hat, tr)


def prodcheck_prove(cpu, pp, fxs, gxs, tr):
    frac = cpu.compute_frac_poly(fxs, gxs)
    prod = cpu.compute_product_poly(frac)
    frac_comm = cpu.commit(pp, frac)
    prod_comm = cpu.commit(pp, prod)
    tr.append_serializable_element(b"frac(x)", g1_compressed(frac_comm))
    tr.append_serializable_element(b"prod(x)", g1_compressed(prod_comm))
    alpha = tr.get_and_append_challenge(b"alpha")
    p1, p2 = cpu.compute_product_factors(frac, prod)
    q = VP(frac.num_vars)
    q.add_mle_list([prod], 1)  # new_from_mle(prod, 1)
    q.add_mle_list([p1, p2], R - 1)
    q.add_mle_list(list(gxs) + [frac], alpha)
    q.add_mle_list(list(fxs), R - alpha)
    point, msgs = zerocheck_prove(cpu, q, tr)
    return (point, msgs, prod_comm, frac_comm), prod, frac


def permcheck_prove(cpu, pp, fxs, gxs, perms, tr):
    beta = tr.get_and_append_challenge(b"beta")
    gamma = tr.get_and_append_challenge(b"gamma")
    nums, dens = cpu.compute_nums_and_denoms(beta, gamma, fxs, gxs, perms)
    return prodcheck_prove(cpu, pp, nums, dens, tr)


# ---------------------------------------------------------------------------
# batch opening
# ---------------------------------------------------------------------------

def _log2_ceil(k: int) -> int:
    return 0 if k <= 1 else (k - 1).bit_length()


def _eq_eval(x, y) -> int:
    out = 1
    for a, b in zip(x, y):
        out = out * ((2 * a * b - a - b + 1) % R) % R
    return out


def _batch_weights(t) -> list:
    if not t:
        return [1]
    tab = orc.frs_ints(orc.CpuBackend().build_eq_x_r(t).evaluations)
    return tab


def multi_open(cpu, pp, polys, points, evals, tr):
    k = len(polys)
    nv = polys[0].num_vars
    for pt in points:
        tr.append_serializable_element(b"eval_point", vec_fr(pt))
    for e in evals:
        tr.append_field_element(b"eval", e)
    t = tr.get_and_append_challenge_vectors(b"t", _log2_ceil(k))
    w = _batch_weights(t)
    first: dict = {}
    for pt in points:
        first.setdefault(tuple(pt), len(first))
    deduped = sorted(first, key=first.get)
    groups = [[] for _ in deduped]
    for i, pt in enumerate(points):
        groups[first[tuple(pt)]].append(i)
    merged = [cpu.linear_combination([polys[i] for i in g], [w[i] for i in g]) for g in groups]
    vp = VP(nv)
    for g, pt in zip(merged, deduped):
        vp.add_mle_list([g, cpu.build_eq_x_r(list(pt))], 1)
    point, msgs = sumcheck_prove(cpu, vp, tr)
    g_prime = cpu.linear_combination(merged, [_eq_eval(point, pt) for pt in deduped])
    quotients, _ = cpu.open(pp, g_prime, point)
    return point, msgs, list(evals), quotients


# ---------------------------------------------------------------------------
# HyperPlonk
# ---------------------------------------------------------------------------

class ProvingKey:
    def __init__(self, cpu, num_vars, num_pub_input, selectors, permutation, srs_layers, gate=VANILLA_GATE):
        self.num_vars, self.num_pub_input, self.gate = num_vars, num_pub_input, gate
        self.pp = cpu.prepare_prover_param(num_vars, srs_layers)
        self.selectors = [cpu.mle_from_evaluations(num_vars, s) for s in selectors]
        self.perms = [cpu.mle_from_evaluations(num_vars, p) for p in permutation]


def prove(cpu, pk: ProvingKey, pub_input, witnesses) -> bytes:
    """snark.rs:156-341; returns the serialized proof."""
    tr = tref.OracleIOPTranscript(b"hyperplonk")
    nv = pk.num_vars
    ell = _log2_ceil(pk.num_pub_input)
    wmles = [cpu.mle_from_evaluations(nv, w) for w in witnesses]
    commits = [cpu.commit(pk.pp, m) for m in wmles]
    for c in commits:
        tr.append_serializable_element(b"w", g1_compressed(c))
    fx = VP(nv)
    for coef, sel, wit in pk.gate:
        fx.add_mle_list(([pk.selectors[sel]] if sel is not None else []) + [wmles[j] for j in wit], coef)
    zc_point, zc_msgs = zerocheck_prove(cpu, fx, tr)
    (pc_point, pc_msgs, prod_comm, frac_comm), prod, frac = permcheck_prove(cpu, pk.pp, wmles, wmles, pk.perms, tr)
    acc_polys, acc_points = [], []

    def insert(m, pt):
        acc_polys.append(m)
        acc_points.append(list(pt))

    p0 = [0] + pc_point[:nv - 1]
    p1 = [1] + pc_point[:nv - 1]
    for pt in (pc_point, p0, p1, [0] + [1] * (nv - 1)):
        insert(prod, pt)
    for pt in (pc_point, p0, p1):
        insert(frac, pt)
    for m in pk.perms:
        insert(m, pc_point)
    for m in wmles:
        insert(m, pc_point)
    for m in wmles:
        insert(m, zc_point)
    for m in pk.selectors:
        insert(m, zc_point)
    r_pi = tr.get_and_append_challenge_vectors(b"r_pi", ell)
    insert(wmles[0], r_pi + [0] * (nv - ell))
    evals = [cpu.evaluate_mle(m, pt) for m, pt in zip(acc_polys, acc_points)]
    b_point, b_msgs, b_evals, b_quotients = multi_open(cpu, pk.pp, acc_polys, acc_points, evals, tr)
    return (vec_g1(commits)
            + iop_proof_bytes(b_point, b_msgs) + vec_fr(b_evals) + vec_g1(b_quotients)
            + iop_proof_bytes(zc_point, zc_msgs)
            + iop_proof_bytes(pc_point, pc_msgs) + g1_compressed(prod_comm) + g1_compressed(frac_comm))


# ---------------------------------------------------------------------------
# fixtures
# ---------------------------------------------------------------------------

def vanilla_fixture(num_vars: int, seed: int, wired: bool = False, num_pub_input: int = 16,
                    witness_seed: int | None = None):
    """Selectors, witnesses and permutation tables of the vanilla-plonk
    circuit (hp_oracle.c or_fixture_vanilla_plonk) as lists of canonical
    table bytes, and the public inputs w1[0..num_pub_input].  `witness_seed`
    (default `seed`) draws another satisfying witness of the same circuit."""
    import ctypes
    lib = orc.load()
    if not hasattr(lib, "_fixture_bound"):
        lib.or_fixture_vanilla_plonk.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_uint8),
                                                 ctypes.POINTER(ctypes.c_uint8)]
        lib.or_fixture_vanilla_plonk.restype = ctypes.c_int
        lib._fixture_bound = True
    n = 1 << num_vars
    sel = np.empty((5, 32 * n), dtype=np.uint8)
    wit = np.empty((3, 32 * n), dtype=np.uint8)
    perm = np.empty((3, 32 * n), dtype=np.uint8)
    u8 = ctypes.POINTER(ctypes.c_uint8)
    ws = seed if witness_seed is None else witness_seed
    if lib.or_fixture_vanilla_plonk(seed, ws, num_vars, 1 if wired else 0, sel.ctypes.data_as(u8),
                                    wit.ctypes.data_as(u8), perm.ctypes.data_as(u8)):
        raise ValueError("fixture num_vars out of range")
    pub = orc.frs_ints(wit[0, :32 * min(num_pub_input, n)].tobytes())
    return ([s.tobytes() for s in sel], [w.tobytes() for w in wit], [p.tobytes() for p in perm], pub)


def prove_fixture(num_vars: int, seed: int, srs_seed: int = 0, wired: bool = False, srs_layers=None,
                  witness_seed: int | None = None) -> bytes:
    """The whole oracle path of the full-prove workload: the fixture, the
    testing SRS (or `srs_layers`: the num_vars + 1 layers of the trimmed
    parameters, 96-byte affine), preprocessing and one proof."""
    cpu = orc.CpuBackend()
    sel, wit, perm, pub = vanilla_fixture(num_vars, seed, wired, witness_seed=witness_seed)
    layers = srs_layers if srs_layers is not None else orc.srs_layers(num_vars, srs_seed)
    pk = ProvingKey(cpu, num_vars, min(16, 1 << num_vars), sel, perm, layers)
    return prove(cpu, pk, pub, wit)


# ---------------------------------------------------------------------------
# the other measured workloads, restated on the oracle
# ---------------------------------------------------------------------------

SUMCHECK_PAIRS = [(0, 1), (2, 3), (4, 5), (0, 3)]
SUMCHECK_LABEL = b"Initializing SumCheck transcript"


def sumcheck_instance(nv: int, seed: int):
    """The degree-2 sumcheck instance: 6 tables of 2^nv Fr (stream `seed`,
    table j = elements [j 2^nv, (j+1) 2^nv)) and 4 arity-2 products over the
    factor pairs SUMCHECK_PAIRS with coefficients = stream 10 + seed,
    elements 0..3.  Returns (tables, coefficients)."""
    n = 1 << nv
    tables = [orc.random_fr(seed, n, first=j * n) for j in range(6)]
    coefs = orc.frs_ints(orc.random_fr(10 + seed, len(SUMCHECK_PAIRS)))
    return tables, coefs


def sumcheck_prove_instance(nv: int, seed: int, instance=None):
    """PolyIOP SumCheck prove of the instance under the transcript
    `SUMCHECK_LABEL`: (point, messages, final folded values of the 6 tables).
    `instance` = sumcheck_instance(nv, seed) when already built."""
    cpu = orc.CpuBackend()
    tables, coefs = instance if instance is not None else sumcheck_instance(nv, seed)
    mles = [cpu.mle_from_evaluations(nv, t) for t in tables]
    vp = VP(nv)
    for c, (a, b) in zip(coefs, SUMCHECK_PAIRS):
        vp.add_mle_list([mles[a], mles[b]], c)
    finals: list = []
    point, msgs = sumcheck_prove(cpu, vp, tref.OracleIOPTranscript(SUMCHECK_LABEL), finals)
    return point, msgs, finals


def sumcheck_digest(point, msgs, finals) -> str:
    """SHA-256 of a sumcheck result: the IOPProof bytes, then the final values."""
    import hashlib
    return hashlib.sha256(iop_proof_bytes(point, msgs) + vec_fr(finals)).hexdigest()


def batch_plan(seed: int = 3, msm_count: int = 64, msm_k=(12, 22), sumcheck_count: int = 32, sumcheck_nv=(14, 22)):
    """The batch workload's sizes: MSM log sizes k uniform in msm_k, then
    sumcheck num_vars uniform in sumcheck_nv, drawn by random.Random(seed).
    MSM i takes stream `seed` elements [sum_{j<i} 2^k_j, ...) as scalars over
    the first 2^k_i bases of SRS layer 0; sumcheck instance i is
    sumcheck_instance(nv_i, 100 + seed + i)."""
    import random
    rng = random.Random(seed)
    ks = [rng.randint(*msm_k) for _ in range(msm_count)]
    nvs = [rng.randint(*sumcheck_nv) for _ in range(sumcheck_count)]
    return ks, nvs


def batch_msm_scalars(ks, seed: int = 3) -> list:
    out, first = [], 0
    for k in ks:
        out.append(orc.random_fr(seed, 1 << k, first=first))
        first += 1 << k
    return out


def serve_requests(count: int, nv_lo: int, nv_hi: int, seed: int = 4):
    """Serving stream requests: num_vars uniform in [nv_lo, nv_hi] drawn by
    random.Random(seed); request i proves the circuit of fixture seed 2 with
    the witness of stream (seed << 32) | i."""
    import random
    rng = random.Random(seed)
    return [(rng.randint(nv_lo, nv_hi), (seed << 32) | i) for i in range(count)]
