"""GPU parity of the MLE ABI entries against the oracle, byte for byte.

Mirrors backend/src/ascend910b3/integration_tests.rs (device vs CpuBackend on
the same inputs) with sizes chosen around the kernels' tile edges."""
import random

import numpy as np

import pytest

from hyperplonk_gb300.errors import InvalidParameters

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def table(oracle, nv, seed, edges=True):
    b = bytearray(oracle.random_fr(seed, 1 << nv))
    if edges and nv >= 2:
        b[0:32] = (0).to_bytes(32, "little")
        b[-32:] = (R - 1).to_bytes(32, "little")
    return bytes(b)


def pair(gpu, cpu, oracle, nv, seed):
    t = table(oracle, nv, seed)
    return gpu.mle_from_evaluations(nv, t), cpu.mle_from_evaluations(nv, t)


@pytest.mark.parametrize("nv", [0, 1, 2, 5, 10, 13])
def test_upload_download_roundtrip(gpu, oracle, nv):
    t = table(oracle, nv, 100 + nv)
    m = gpu.mle_from_evaluations(nv, t)
    assert gpu.download(m) == t


def test_upload_rejects_noncanonical_and_bad_shape(gpu, oracle):
    t = bytearray(table(oracle, 3, 1))
    t[32 * 5:32 * 6] = R.to_bytes(32, "little")
    with pytest.raises(InvalidParameters):
        gpu.mle_from_evaluations(3, bytes(t))
    with pytest.raises(InvalidParameters):
        gpu.mle_from_evaluations(3, bytes(32 * 7))


@pytest.mark.parametrize("nv,count", [(0, 2), (1, 1), (4, 3), (11, 5), (9, 40)])
def test_linear_combination(gpu, cpu, oracle, nv, count):
    rng = random.Random(nv * 100 + count)
    gs, cs = [], []
    for j in range(count):
        g, c = pair(gpu, cpu, oracle, nv, 200 + j)
        gs.append(g)
        cs.append(c)
    coefs = [rng.randrange(R) for _ in range(count)]
    if count > 2:
        coefs[1] = 0
    got = gpu.download(gpu.linear_combination(gs, coefs))
    assert got == cpu.linear_combination(cs, coefs).evaluations
    zero = gpu.linear_combination(gs[:1], [0])
    assert gpu.download(zero) == bytes(32 << nv)
    assert zero.num_vars == nv


@pytest.mark.parametrize("nv", [0, 1, 5, 10, 11, 12, 16])
def test_evaluate(gpu, cpu, oracle, nv):
    g, c = pair(gpu, cpu, oracle, nv, 300 + nv)
    rng = random.Random(nv)
    pt = [rng.randrange(R) for _ in range(nv)]
    assert gpu.evaluate_mle(g, pt) == cpu.evaluate_mle(c, pt)
    with pytest.raises(InvalidParameters):
        gpu.evaluate_mle(g, pt + [1])


@pytest.mark.parametrize("nv", [1, 2, 11, 14])
def test_evaluate_with_boolean_last_coordinates(gpu, cpu, oracle, nv):
    """Points whose last coordinates are 0 or 1 (the proof's (0, 1, .., 1) and
    (r_pi, 0, .., 0) openings) start the fold at a sub-table: same values."""
    g, c = pair(gpu, cpu, oracle, nv, 320 + nv)
    rng = random.Random(1000 + nv)
    points = [[0] + [1] * (nv - 1), [1] * nv, [0] * nv,
              [rng.randrange(R) for _ in range(min(4, nv))] + [0] * max(0, nv - 4),
              [rng.randrange(R) for _ in range(nv // 2)] + [rng.randrange(2) for _ in range(nv - nv // 2)],
              [rng.randrange(2) for _ in range(nv - 1)] + [rng.randrange(R)]]
    for pt in points:
        assert gpu.evaluate_mle(g, pt) == cpu.evaluate_mle(c, pt), pt
    many = gpu.evaluate_many([g] * len(points), points)
    assert many == [cpu.evaluate_mle(c, pt) for pt in points]


@pytest.mark.parametrize("nv", [1, 2, 5, 12, 13, 17])
def test_build_eq_x_r(gpu, cpu, nv):
    rng = random.Random(40 + nv)
    r = [rng.randrange(R) for _ in range(nv)]
    r[0] = 0
    assert gpu.download(gpu.build_eq_x_r(r)) == cpu.build_eq_x_r(r).evaluations
    with pytest.raises(InvalidParameters):
        gpu.build_eq_x_r([])


@pytest.mark.parametrize("nv,count", [(0, 1), (1, 1), (3, 3), (11, 1), (12, 3), (16, 2)])
def test_frac(gpu, cpu, oracle, nv, count):
    fs = [pair(gpu, cpu, oracle, nv, 500 + j) for j in range(count)]
    gs = []
    for j in range(count):
        t = bytearray(oracle.random_fr(600 + j, 1 << nv))
        gs.append((gpu.mle_from_evaluations(nv, bytes(t)), cpu.mle_from_evaluations(nv, bytes(t))))
    got = gpu.download(gpu.compute_frac_poly([f[0] for f in fs], [g[0] for g in gs]))
    assert got == cpu.compute_frac_poly([f[1] for f in fs], [g[1] for g in gs]).evaluations


def test_frac_zero_denominator_is_invalid_parameters(gpu, oracle):
    nv = 10
    f = gpu.mle_from_evaluations(nv, oracle.random_fr(1, 1 << nv))
    t = bytearray(oracle.random_fr(2, 1 << nv))
    t[32 * 777:32 * 778] = bytes(32)
    g = gpu.mle_from_evaluations(nv, bytes(t))
    with pytest.raises(InvalidParameters):
        gpu.compute_frac_poly([f], [g])
    # 0/0 too
    z = gpu.mle_from_evaluations(1, bytes(64))
    with pytest.raises(InvalidParameters):
        gpu.compute_frac_poly([z], [z])


@pytest.mark.parametrize("nv", [1, 2, 3, 9, 10, 11, 16])
def test_product_poly_and_factors(gpu, cpu, oracle, nv):
    f, c = pair(gpu, cpu, oracle, nv, 700 + nv)
    pg, pc = gpu.compute_product_poly(f), cpu.compute_product_poly(c)
    assert gpu.download(pg) == pc.evaluations
    a, b = gpu.compute_product_factors(f, pg)
    ea, eb = cpu.compute_product_factors(c, pc)
    assert gpu.download(a) == ea.evaluations
    assert gpu.download(b) == eb.evaluations


def test_product_poly_kat(gpu):
    from oracle import frs_ints
    frac = gpu.mle_from_evaluations(3, [2, 3, 5, 7, 11, 13, 17, 19])
    assert frs_ints(gpu.download(gpu.compute_product_poly(frac))) == [6, 35, 143, 323, 210, 46189, 9699690, 0]
    with pytest.raises(InvalidParameters):
        gpu.compute_product_poly(gpu.mle_from_evaluations(0, [2]))


@pytest.mark.parametrize("nv", [0, 2, 10, 15])
def test_nums_and_denoms(gpu, cpu, oracle, nv):
    cols = 3
    fx = [pair(gpu, cpu, oracle, nv, 800 + j) for j in range(cols)]
    gx = [pair(gpu, cpu, oracle, nv, 810 + j) for j in range(cols)]
    pm = [pair(gpu, cpu, oracle, nv, 820 + j) for j in range(cols)]
    rng = random.Random(nv)
    for beta, gamma in [(rng.randrange(R), rng.randrange(R)), (0, 5), (R - 2, 0)]:
        ng, dg = gpu.compute_nums_and_denoms(beta, gamma, [x[0] for x in fx], [x[0] for x in gx], [x[0] for x in pm])
        nc, dc = cpu.compute_nums_and_denoms(beta, gamma, [x[1] for x in fx], [x[1] for x in gx], [x[1] for x in pm])
        for j in range(cols):
            assert gpu.download(ng[j]) == nc[j].evaluations
            assert gpu.download(dg[j]) == dc[j].evaluations


def test_inputs_stay_immutable(gpu, oracle):
    nv = 8
    t = table(oracle, nv, 900)
    m = gpu.mle_from_evaluations(nv, t)
    gpu.linear_combination([m, m], [3, 4])
    gpu.compute_product_poly(m)
    gpu.compute_frac_poly([m], [gpu.mle_from_evaluations(nv, oracle.random_fr(901, 1 << nv))])
    gpu.evaluate_mle(m, list(range(nv)))
    assert gpu.download(m) == t


def test_evaluate_many_matches_single_evaluations(gpu, oracle):
    import random
    rng = random.Random(21)
    R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
    nvs = [0, 1, 5, 10, 11, 13, 21, 3]
    mles = [gpu.mle_from_evaluations(nv, oracle.random_fr(500 + i, 1 << nv)) for i, nv in enumerate(nvs)]
    points = [[rng.randrange(R) for _ in range(nv)] for nv in nvs]
    many = gpu.evaluate_many(mles, points)
    assert many == [gpu.evaluate_mle(m, p) for m, p in zip(mles, points)]
    cpu = oracle.CpuBackend()
    for i, (nv, p) in enumerate(zip(nvs[:6], points[:6])):
        assert many[i] == cpu.evaluate_mle(cpu.mle_from_evaluations(nv, oracle.random_fr(500 + i, 1 << nv)), p)
    assert gpu.evaluate_many([], []) == []


def test_evaluate_many_shared_points_use_eq_dot_products(gpu, oracle):
    """Polynomials of >= 2^12 entries sharing a point are evaluated as dot
    products with one eq table; values equal the single evaluations and the
    oracle's."""
    import random
    rng = random.Random(22)
    R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
    nv = 13
    p1 = [rng.randrange(R) for _ in range(nv)]
    p2 = [rng.randrange(R) for _ in range(nv)]
    tables = [oracle.random_fr(600 + i, 1 << nv) for i in range(5)]
    mles = [gpu.mle_from_evaluations(nv, t) for t in tables]
    points = [p1, p2, p1, p1, p2]
    many = gpu.evaluate_many(mles, points)
    assert many == [gpu.evaluate_mle(m, p) for m, p in zip(mles, points)]
    cpu = oracle.CpuBackend()
    assert many == [cpu.evaluate_mle(cpu.mle_from_evaluations(nv, t), p) for t, p in zip(tables, points)]


@pytest.mark.parametrize("nv", [12, 13, 17])
def test_evaluate_many_large_shared_point_group(gpu, oracle, nv):
    """A point shared by more polynomials than one dot-product launch takes
    (32): the group is split over launches, every value where it belongs.
    From nv = 13 on the dot products take eq's two half tables instead of
    the full table (nv = 17: the grid's stride spans many rows)."""
    import random
    rng = random.Random(23 + nv)
    p1 = [rng.randrange(R) for _ in range(nv)]
    p2 = [rng.randrange(R) for _ in range(nv)]
    tables = [oracle.random_fr(700 + i, 1 << nv) for i in range(40)]
    mles = [gpu.mle_from_evaluations(nv, t) for t in tables]
    points = [p2 if i in (3, 17, 38) else p1 for i in range(40)]
    many = gpu.evaluate_many(mles, points)
    cpu = oracle.CpuBackend()
    assert many == [cpu.evaluate_mle(cpu.mle_from_evaluations(nv, t), p) for t, p in zip(tables, points)]


def test_upload_many_equals_single_uploads(gpu, oracle):
    from hyperplonk_gb300.errors import InvalidParameters
    nv = 9
    tables = [oracle.random_fr(40 + k, 1 << nv) for k in range(4)]
    many = gpu.mle_from_evaluations_many(nv, tables)
    for t, m in zip(tables, many):
        assert gpu.download(m) == t
        assert gpu.evaluate_mle(m, [3] * nv) == gpu.evaluate_mle(gpu.mle_from_evaluations(nv, t), [3] * nv)
    assert gpu.mle_from_evaluations_many(nv, []) == []
    bad = bytearray(tables[2])
    bad[32 * 17:32 * 18] = (0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001).to_bytes(32, "little")
    with pytest.raises(InvalidParameters):
        gpu.mle_from_evaluations_many(nv, [tables[0], bytes(bad), tables[1]])
    with pytest.raises(InvalidParameters):
        gpu.mle_from_evaluations_many(nv, [tables[0], tables[1][:-32]])


# ---------------------------------------------------------------------------
# asynchronous upload (ingress stream): hp_cuda_v1_mle_upload_async / _wait
# ---------------------------------------------------------------------------

def _pinned(table):
    import torch
    t = torch.empty(len(table), dtype=torch.uint8, pin_memory=True)
    t.numpy()[:] = np.frombuffer(table, dtype=np.uint8)
    return t


@pytest.mark.gpu
def test_async_upload_is_waited_for_on_the_device(gpu, cpu, oracle):
    nv = 14
    tables = [oracle.random_fr(90 + j, 1 << nv) for j in range(3)]
    pinned = [_pinned(t) for t in tables]
    up = gpu.mle_upload_async(nv, [p.numpy() for p in pinned])
    # queued before the wait: the linear combination waits for the copies on the device
    lc = gpu.linear_combination(up.mles, [3, 5, 7])
    mles = up.wait()
    assert gpu.download(lc) == cpu.linear_combination([cpu.mle_from_evaluations(nv, t) for t in tables],
                                                      [3, 5, 7]).evaluations
    assert [gpu.download(m) for m in mles] == tables
    assert up.wait() is mles  # a second wait is a no-op


@pytest.mark.gpu
def test_async_upload_rejects_non_canonical_at_wait(gpu, oracle):
    from hyperplonk_gb300.errors import InvalidParameters
    nv = 6
    good = oracle.random_fr(95, 1 << nv)
    bad = bytearray(good)
    bad[32 * 7 + 31] = 0xff  # >= r
    up = gpu.mle_upload_async(nv, [_pinned(good).numpy(), _pinned(bytes(bad)).numpy()])
    with pytest.raises(InvalidParameters):
        up.wait()
    assert up.mles == []
    # the context keeps working, and a later upload call is independent
    ok = gpu.mle_upload_async(nv, [_pinned(good).numpy()]).wait()
    assert gpu.download(ok[0]) == good


@pytest.mark.gpu
def test_pipelined_proofs_equal_proofs_from_blocking_uploads(gpu, oracle):
    """Proof i+1's witness upload queued before proof i runs: every proof
    equals the proof of the same witnesses uploaded the blocking way."""
    from hyperplonk_gb300 import snark
    nv = 9
    layers = [oracle.affine_to_packets(l) for l in oracle.srs_layers(nv, 96)]
    sel, wit, perm, pub = snark.vanilla_fixture(nv, 2)
    pk = snark.preprocess(gpu, nv, 16, sel, perm, layers, commit=False)
    witness_sets = [snark.vanilla_witness(nv, 2, (6 << 32) | i) for i in range(3)]
    pubs = [[int.from_bytes(w[0][32 * j:32 * j + 32].tobytes(), "little") for j in range(16)] for w in witness_sets]
    pinned = [[_pinned(t.tobytes()).numpy() for t in w] for w in witness_sets]
    expect = [snark.prove(gpu, pk, p, w).to_bytes() for p, w in zip(pubs, witness_sets)]
    got = []
    nxt = gpu.mle_upload_async(nv, pinned[0])
    for i in range(3):
        cur = nxt
        if i + 1 < 3:
            nxt = gpu.mle_upload_async(nv, pinned[i + 1])
        got.append(snark.prove(gpu, pk, pubs[i], None, witness_mles=cur.wait()).to_bytes())
    assert got == expect
