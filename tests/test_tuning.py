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
        else:
            assert tuning.query(tuning.SHARED, 1 << int(f[1]))[2] == int(f[2]), line
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
