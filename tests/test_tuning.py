"""MSM autotuner (csrc/tune.cu, hyperplonk_gb300/tuning.py).

CPU: the tuning table's host logic -- the size rules a query reports with no
entry (checked against a restatement here), the text file round trip, the
rejection of malformed or foreign files, the precedence environment override >
tuned entry > size rule, and a tuned segment / chunk applying only with the
window width it was measured with.  GPU: the tuner's entries (alone and
shared launch), the re-prepared parameter layers and arbitrary geometries all
give the oracle's points."""
import os
import pathlib
import random
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def windows(c):
    return (256 + c - 1) // c


def window_fits(n, c):
    if windows(c) * n >= 1 << 31:
        return False
    top_bits = 255 - c * (windows(c) - 1)
    top_buckets = 1 << (top_bits - 1) if top_bits >= 2 else 1
    return c == 4 or n / top_buckets <= 2048


def model_c(n):
    best, best_cost = 4, float("inf")
    for c in range(4, 21):
        if not window_fits(n, c):
            continue
        cost = windows(c) * 10 * n + 28 * (1 << (c - 1))
        if cost < best_cost:
            best, best_cost = c, cost
    return best


def default_seg(c):
    b = 1 << (c - 1)
    seg = min(16, max(1, b >> 13))
    while b // seg > 64 * 1024:
        seg *= 2
    return seg


def default_chunk(records):
    return 8 if records < 1 << 21 else 32


@pytest.fixture
def tuning(native_lib, tmp_path):
    """An empty table for the test; the process's table is put back after."""
    from hyperplonk_gb300 import tuning as t
    saved = tmp_path / "saved_table.txt"
    t.save(saved)
    t.clear()
    yield t
    t.clear()
    t.load(saved)


def _write(path, lines):
    path.write_text("\n".join(lines) + "\n")
    return path


def test_query_without_entries_is_the_size_rule(tuning):
    for k in range(0, 25):
        n = 1 << k
        c = model_c(n)
        assert tuning.query(tuning.ALONE, n) == (c, default_seg(c), default_chunk(windows(c) * n)), k
    for records in (1, 5000, (1 << 21) - 1, 1 << 21, 1 << 26):
        assert tuning.query(tuning.SHARED, records) == (0, 0, default_chunk(records))
    assert model_c(1 << 20) == 20 and default_seg(20) == 16  # the 2^20 commit geometry


def test_file_round_trip(tuning, tmp_path):
    src = _write(tmp_path / "a.txt", ["hp_cuda msm tuning 1", "device NVIDIA_GB300", "alone 20 16 8 16 7.5000",
                                      "alone 12 11 2 4 0.3000", "many 24 16 3.2500"])
    tuning.load(src)
    assert tuning.query(tuning.ALONE, 1 << 20) == (16, 8, 16)
    assert tuning.query(tuning.ALONE, (1 << 19) + 1) == (16, 8, 16)  # keyed by ceil(log2 n)
    assert tuning.query(tuning.ALONE, 1 << 12) == (11, 2, 4)
    assert tuning.query(tuning.SHARED, 1 << 24) == (0, 0, 16)
    assert tuning.query(tuning.SHARED, 1 << 25) == (0, 0, 32)  # no entry: size rule
    out = tmp_path / "b.txt"
    tuning.save(out)
    assert out.read_text().splitlines() == ["hp_cuda msm tuning 1", "device NVIDIA_GB300", "alone 12 11 2 4 0.3000",
                                            "alone 20 16 8 16 7.5000", "many 24 16 3.2500"]
    tuning.clear()
    assert tuning.query(tuning.ALONE, 1 << 20) == (20, 16, 32)
    tuning.load(out, device="NVIDIA GB300")
    assert tuning.query(tuning.ALONE, 1 << 20) == (16, 8, 16)


@pytest.mark.parametrize("lines", [
    ["hp_cuda msm tuning 2", "alone 20 19 8 16 1.0"],         # unknown version
    ["hp_cuda msm tuning 1", "alone 20 23 8 16 1.0"],         # window width out of range
    ["hp_cuda msm tuning 1", "alone 20 19 12 16 1.0"],        # segment not a power of two
    ["hp_cuda msm tuning 1", "alone 20 19 8 1 1.0"],          # chunk below 2
    ["hp_cuda msm tuning 1", "alone 20 19 8 16"],             # missing field
    ["hp_cuda msm tuning 1", "alone 20 19 8 16 1.0 extra"],   # trailing token
    ["hp_cuda msm tuning 1", "many 24 16 nan"],               # not a time
    ["hp_cuda msm tuning 1", "window 20 19"],                 # unknown entry
])
def test_malformed_files_are_rejected_and_change_nothing(tuning, tmp_path, lines):
    from hyperplonk_gb300.errors import InvalidParameters
    before = tuning.query(tuning.ALONE, 1 << 20)
    with pytest.raises(InvalidParameters):
        tuning.load(_write(tmp_path / "bad.txt", lines))
    assert tuning.query(tuning.ALONE, 1 << 20) == before
    with pytest.raises(InvalidParameters):
        tuning.load(tmp_path / "missing.txt")


def test_foreign_device_is_rejected(tuning, tmp_path):
    from hyperplonk_gb300.errors import InvalidParameters
    f = _write(tmp_path / "t.txt", ["hp_cuda msm tuning 1", "device NVIDIA_B200", "alone 20 16 8 16 1.0"])
    with pytest.raises(InvalidParameters):
        tuning.load(f, device="NVIDIA GB300")
    assert tuning.query(tuning.ALONE, 1 << 20) == (20, 16, 32)
    tuning.load(f)  # no device given: accepted
    assert tuning.query(tuning.ALONE, 1 << 20) == (16, 8, 16)
    anyf = _write(tmp_path / "any.txt", ["hp_cuda msm tuning 1", "alone 16 13 4 8 1.0"])
    tuning.load(anyf, device="NVIDIA GB300")  # no device line: any device
    assert tuning.query(tuning.ALONE, 1 << 16) == (13, 4, 8)


def _query_in_child(env, n):
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from hyperplonk_gb300 import tuning\n"
            "print(*tuning.query(tuning.ALONE, %d))\n") % (str(ROOT), n)
    full = dict(os.environ)
    for k in ("HP_CUDA_MSM_TUNING", "HP_MSM_WINDOW_BITS", "HP_MSM_SEG", "HP_ACC_CHUNK"):
        full.pop(k, None)
    full.update(env)
    res = subprocess.run([sys.executable, "-c", code], env=full, capture_output=True, text=True, timeout=120,
                         check=True)
    return tuple(int(x) for x in res.stdout.split())


def test_environment_file_and_override_precedence(native_lib, tmp_path):
    f = _write(tmp_path / "env.txt", ["hp_cuda msm tuning 1", "alone 20 16 4 64 1.0"])
    assert _query_in_child({"HP_CUDA_MSM_TUNING": str(f)}, 1 << 20) == (16, 4, 64)
    # an unreadable file is ignored; "off" is the size rules
    assert _query_in_child({"HP_CUDA_MSM_TUNING": str(tmp_path / "none.txt")}, 1 << 20) == (20, 16, 32)
    assert _query_in_child({"HP_CUDA_MSM_TUNING": "off"}, 1 << 20) == (20, 16, 32)
    # the geometry overrides beat the table
    assert _query_in_child({"HP_CUDA_MSM_TUNING": str(f), "HP_ACC_CHUNK": "24"}, 1 << 20) == (16, 4, 24)
    assert _query_in_child({"HP_CUDA_MSM_TUNING": str(f), "HP_MSM_SEG": "32"}, 1 << 20) == (16, 32, 64)
    # a forced window width drops the entry's segment and chunk (measured with another width)
    assert _query_in_child({"HP_CUDA_MSM_TUNING": str(f), "HP_MSM_WINDOW_BITS": "17"}, 1 << 20) == (
        17, default_seg(17), default_chunk(windows(17) << 20))


def test_entry_whose_width_does_not_fit_is_ignored(tuning, tmp_path):
    # c = 19 at 2^20 leaves 8 bits in the top window: 8192 records per bucket
    assert not window_fits(1 << 20, 19) and window_fits(1 << 20, 16)
    tuning.load(_write(tmp_path / "w.txt", ["hp_cuda msm tuning 1", "alone 20 19 8 16 1.0"]))
    assert tuning.query(tuning.ALONE, 1 << 20) == (20, 16, 32)


def _builtin_table_text():
    inc = (ROOT / "hyperplonk_gb300" / "csrc" / "msm_tuning_gb300.inc").read_text()
    return inc.split('R"HPTUNE(', 1)[1].split(')HPTUNE"', 1)[0]


def test_builtin_gb300_table_parses(tuning, tmp_path):
    text = _builtin_table_text()
    assert text.splitlines()[:2] == ["hp_cuda msm tuning 1", "device NVIDIA_GB300"]
    tuning.load(_write(tmp_path / "b.txt", text.strip().splitlines()), device="NVIDIA GB300")
    for line in text.splitlines()[2:]:
        f = line.split()
        if f[0] == "alone":
            n = 1 << int(f[1])
            c, seg, chunk = int(f[2]), int(f[3]), int(f[4])
            assert window_fits(n, c)
            assert tuning.query(tuning.ALONE, n) == (c, seg, chunk), line
        elif f[0] == "many":
            assert tuning.query(tuning.SHARED, 1 << int(f[1]))[2] == int(f[2]), line
        else:
            k, arity, slots, fold, kernel, per_sm = (int(x) for x in f[1:7])
            assert tuning.route(1 << k, arity, slots, fold=bool(fold)) == (kernel, per_sm), line
    # the headline sizes keep the size rule's geometry
    assert tuning.query(tuning.ALONE, 1 << 20) == (20, 16, 32)


def test_unusable_segment_falls_back(tuning, tmp_path):
    # 2^21 buckets (c = 22) need at least 32-bucket segments for the subset sums
    tuning.load(_write(tmp_path / "s.txt", ["hp_cuda msm tuning 1", "alone 22 22 8 32 1.0"]))
    assert tuning.query(tuning.ALONE, 1 << 22) == (22, 32, 32)


# ---------------------------------------------------------------------------
# GPU


def _prefix_points(oracle, layer0, n, scalars):
    return oracle.affine_to_point(oracle.msm(layer0[:96 * n], scalars))


@pytest.mark.gpu
def test_autotune_alone_keeps_results(gpu, oracle, tuning):
    nv_srs = 12
    layers = oracle.srs_layers(nv_srs, 43)
    pg = gpu.prepare_prover_param(nv_srs, [oracle.affine_to_packets(l) for l in layers])
    res = tuning.autotune(gpu, pg, [8, 10, 12])
    assert [r.size for r in res] == [1 << 8, 1 << 10, 1 << 12]
    for r in res:
        assert r.mode == tuning.ALONE and 4 <= r.window_bits <= 22 and r.chunk >= 2
        assert r.segment & (r.segment - 1) == 0
        assert 0 < r.tuned_ms <= r.model_ms * 1.0001
        assert tuning.query(tuning.ALONE, r.size) == (r.window_bits, r.segment, r.chunk)
    # the parameter object's layers were re-prepared with the entries: commits still match
    for nv in (12, 10, 7):
        t = oracle.random_fr(500 + nv, 1 << nv)
        got = gpu.commit(pg, gpu.mle_from_evaluations(nv, t))
        assert got == oracle.affine_to_point(oracle.msm(layers[nv_srs - nv], t)), nv
    mles = [gpu.mle_from_evaluations(nv, oracle.random_fr(600 + nv, 1 << nv)) for nv in (8, 10, 12, 5)]
    got = gpu.batch_msm(pg, 0, mles)
    for m, g in zip(mles, got):
        n = 1 << m.num_vars
        assert g == _prefix_points(oracle, layers[0], n, gpu.download(m)), m.num_vars


@pytest.mark.gpu
def test_autotune_shared_launch_keeps_results(gpu, oracle, tuning):
    nv_srs = 12
    layers = oracle.srs_layers(nv_srs, 44)
    pg = gpu.prepare_prover_param(nv_srs, [oracle.affine_to_packets(l) for l in layers])
    mix = [4, 6, 8, 9, 10, 11]
    (r,) = tuning.autotune(gpu, pg, mix, mode=tuning.SHARED)
    assert r.mode == tuning.SHARED and r.chunk in (4, 8, 16, 32, 64)
    assert tuning.query(tuning.SHARED, r.size)[2] == r.chunk
    mles = [gpu.mle_from_evaluations(nv, oracle.random_fr(700 + i, 1 << nv)) for i, nv in enumerate(mix)]
    for m, g in zip(mles, gpu.batch_msm(pg, 0, mles)):
        assert g == _prefix_points(oracle, layers[0], 1 << m.num_vars, gpu.download(m))


@pytest.mark.gpu
@pytest.mark.parametrize("entry", [
    "alone 11 6 1 2 1.0",     # narrow windows (43 of them), no segments, 2-record chunks
    "alone 11 13 64 64 1.0",  # 4096 buckets for 2^11 points, one long segment, long chunks
    "alone 11 9 2 5 1.0",     # odd chunk length
])
def test_any_tuned_geometry_gives_the_oracle_point(gpu, oracle, tuning, tmp_path, entry):
    tuning.load(_write(tmp_path / "g.txt", ["hp_cuda msm tuning 1", entry, "many 17 4 1.0", "many 18 64 1.0"]))
    nv_srs = 11
    layers = oracle.srs_layers(nv_srs, 45)
    pg = gpu.prepare_prover_param(nv_srs, [oracle.affine_to_packets(l) for l in layers])
    c = int(entry.split()[2])
    assert tuning.query(tuning.ALONE, 1 << 11)[0] == c
    t = oracle.random_fr(800, 1 << 11)
    assert gpu.commit(pg, gpu.mle_from_evaluations(11, t)) == oracle.affine_to_point(oracle.msm(layers[0], t))
    rng = random.Random(c)
    dims = [rng.randint(3, 10) for _ in range(10)]
    mles = [gpu.mle_from_evaluations(d, oracle.random_fr(900 + i, 1 << d)) for i, d in enumerate(dims)]
    for m, g in zip(mles, gpu.batch_msm(pg, 0, mles)):
        assert g == _prefix_points(oracle, layers[0], 1 << m.num_vars, gpu.download(m))


@pytest.mark.gpu
def test_builtin_table_is_the_default_on_gb300(native_lib):
    import torch
    if torch.cuda.get_device_name(0) != "NVIDIA GB300":
        pytest.skip("the built-in table is for NVIDIA GB300")
    # a fresh process: the built-in entries, e.g. 2^10 points with 13-bit windows
    assert _query_in_child({}, 1 << 10) == (13, 1, 8)
    c = model_c(1 << 10)
    assert c != 13
    assert _query_in_child({"HP_CUDA_MSM_TUNING": "off"}, 1 << 10) == (c, default_seg(c), default_chunk(windows(c) << 10))


@pytest.mark.gpu
def test_autotune_refuses_geometry_overrides(gpu, oracle, tuning, monkeypatch):
    from hyperplonk_gb300.errors import InvalidState
    layers = oracle.srs_layers(6, 46)
    pg = gpu.prepare_prover_param(6, [oracle.affine_to_packets(l) for l in layers])
    monkeypatch.setenv("HP_MSM_SEG", "4")
    with pytest.raises(InvalidState):
        tuning.autotune(gpu, pg, [6])


# ---------------------------------------------------------------------------
# sumcheck round routes (csrc/sumcheck.cu, same table and file)
# ---------------------------------------------------------------------------

ONE_BLOCK, PER_PAIR, SLOT, SLOT_FUSED, PP, PP_FUSED = 1, 2, 3, 4, 5, 6


def test_round_routes_without_entries_are_the_built_in_rules(tuning):
    # degree-2 products of arity 2, 12 slots (the sumcheck workload's shape)
    assert tuning.route(1 << 19, 2, 12) == (PP, 4)
    assert tuning.route(1 << 16, 2, 12) == (PP, 4)
    assert tuning.route(1 << 15, 2, 12) == (SLOT, 16)
    assert tuning.route(1 << 13, 2, 12) == (SLOT_FUSED, 0)
    assert tuning.route(65, 2, 12) == (SLOT_FUSED, 0)
    assert tuning.route(64, 2, 12) == (ONE_BLOCK, 0)
    # arity 4 and 5 (the zero-checks): separate fold in the middle rounds
    assert tuning.route(1 << 19, 5, 18) == (SLOT, 16)
    assert tuning.route(1 << 10, 4, 20) == (SLOT, 0)
    # products of arity above 8 keep the (slot, pair) kernel even when small
    assert tuning.route(8, 34, 35) == (SLOT, 0)


def test_round_route_file_round_trip_and_validity(tuning, tmp_path):
    f = _write(tmp_path / "t.txt", ["hp_cuda msm tuning 1", "device any",
                                    "round 19 2 12 1 3 8 120.5",
                                    "round 10 2 12 1 2 0 30.0",
                                    "round 12 5 18 1 5 3 40.0"])  # (product, pair) cannot run arity 5
    tuning.load(f)
    assert tuning.route(1 << 19, 2, 12) == (SLOT, 8)
    assert tuning.route((1 << 18) + 1, 2, 12) == (SLOT, 8)  # ceil(log2 pairs) = 19
    assert tuning.route(1 << 10, 2, 12) == (PER_PAIR, 0)
    assert tuning.route(1 << 12, 5, 18) == (SLOT, 0)  # invalid entry: the built-in rule
    assert tuning.route(1 << 10, 2, 13) == (SLOT_FUSED, 0)  # other key
    assert tuning.route(1 << 19, 2, 12, fold=False) == (PP, 4)  # the first round is another key
    out = tmp_path / "out.txt"
    tuning.save(out)
    lines = out.read_text().splitlines()
    assert "round 19 2 12 1 3 8 120.50" in lines and "round 10 2 12 1 2 0 30.00" in lines
    tuning.clear()
    assert tuning.route(1 << 19, 2, 12) == (PP, 4)
    tuning.load(out)
    assert tuning.route(1 << 19, 2, 12) == (SLOT, 8)


@pytest.mark.parametrize("bad", ["round 19 2 12 1 9 8 1.0", "round 19 2 12 1 0 8 1.0", "round 19 2 12 1 3 99 1.0",
                                 "round 19 0 12 1 3 8 1.0", "round 19 2 12 2 3 8 1.0", "round 19 2 12 1 3 8",
                                 "round 19 2 12 1 3 8 1.0 x"])
def test_malformed_round_lines_are_rejected(tuning, tmp_path, bad):
    from hyperplonk_gb300.errors import InvalidParameters
    f = _write(tmp_path / "bad.txt", ["hp_cuda msm tuning 1", "device any", bad])
    with pytest.raises(InvalidParameters):
        tuning.load(f)
    assert tuning.route(1 << 19, 2, 12) == (PP, 4)


@pytest.mark.gpu
@pytest.mark.parametrize("arities,nv", [((2, 2, 2, 2), 13), ((3, 4, 5, 2), 11)])
def test_sumcheck_autotune_then_rounds_equal_oracle(gpu, cpu, oracle, tuning, arities, nv):
    """Tune the routes of a shape on one state, then prove another state of
    the same shape round by round: every message equals the oracle's, and the
    rounds took the stored routes."""
    from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial
    R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
    rng = random.Random(sum(arities) + nv)
    nf = 6
    tables = [oracle.random_fr(400 + nv, 1 << nv, first=j << nv) for j in range(nf)]
    products = [(rng.randrange(1, R), [rng.randrange(nf) for _ in range(m)]) for m in arities]

    def vp_for(be, mles):
        vp = VirtualPolynomial(nv)
        for c, ix in products:
            vp.add_mle_list([mles[i] for i in ix], c)
        return vp

    gm = [gpu.mle_from_evaluations(nv, t) for t in tables]
    cm = [cpu.mle_from_evaluations(nv, t) for t in tables]
    records = tuning.autotune_sumcheck(gpu, vp_for(gpu, gm))
    assert [r.pairs for r in records] == [1 << (nv - 1 - k) for k in range(nv)]
    vg = vp_for(gpu, gm)
    slots = sum(len(ix) + 1 for _, ix in vg.products)
    max_arity = max(len(ix) for _, ix in vg.products)
    for k, r in enumerate(records):
        assert r.tuned_us <= r.default_us
        assert tuning.route(r.pairs, max_arity, slots, fold=k > 0) == (r.kernel, r.blocks_per_sm)
    sg, sc = gpu.prover_init(vg), cpu.prover_init(vp_for(cpu, cm))
    ch = None
    for k in range(nv):
        assert gpu.prove_round_and_update_state(sg, ch) == cpu.prove_round_and_update_state(sc, ch), k
        ch = rng.randrange(R)
    assert gpu.final_evaluations(sg, ch) == cpu.final_evaluations(sc, ch)


def test_route_kernel_names_cover_every_route_code():
    """tuning.ROUTE_KERNELS names every route code csrc/sumcheck.cuh defines
    (1 .. kRouteKinds - 1), so tuner records always print a kernel name."""
    import re
    from hyperplonk_gb300 import tuning as tn
    text = (pathlib.Path(__file__).resolve().parent.parent / "hyperplonk_gb300" / "csrc" / "sumcheck.cuh").read_text()
    kinds = int(re.search(r"kRouteKinds\s*=\s*(\d+)", text).group(1))
    assert sorted(tn.ROUTE_KERNELS) == list(range(1, kinds))
