"""Host-side workload logic (no GPU): fixture streams of the measured
workloads against the oracle's generator, and the lockstep batch sumcheck
driver against one-at-a-time proofs on the oracle backend."""
from hyperplonk_gb300 import protocol, workloads


def test_fixture_stream_matches_oracle(native_lib, oracle):
    for seed, n, first in [(1, 16, 0), (1, 16, 32), (3, 5, 1000), (11, 4, 0)]:
        assert workloads.fixture_fr(seed, n, first).tobytes() == oracle.random_fr(seed, n, first=first)


def test_sumcheck_instance_matches_config2_fixture(native_lib, oracle):
    tables = workloads.sumcheck_tables(4, 1)
    assert [t.tobytes() for t in tables] == [oracle.random_fr(1, 16, first=j << 4) for j in range(6)]
    assert workloads.sumcheck_coefficients(1) == [
        int.from_bytes(oracle.random_fr(11, 4)[32 * i:32 * i + 32], "little") for i in range(4)]


def test_batch_plan_is_seeded():
    ks, nvs = workloads.batch_plan(3)
    assert (len(ks), len(nvs)) == (64, 32)
    assert all(12 <= k <= 22 for k in ks) and all(14 <= nv <= 22 for nv in nvs)
    assert workloads.batch_plan(3) == (ks, nvs)


def test_lockstep_sumcheck_equals_sequential(native_lib, cpu):
    import transcript_ref as tref
    nvs = [3, 6, 1, 5]
    finals_b, finals_s = [], []
    wb = workloads.BatchWorkload(cpu, None, [], nvs)
    batched = protocol.batch_sumcheck_prove(
        cpu, wb.polynomials(), [tref.OracleIOPTranscript(workloads.SUMCHECK_LABEL) for _ in nvs], finals_b)
    ws = workloads.BatchWorkload(cpu, None, [], nvs)
    seq = []
    for vp in ws.polynomials():
        f = []
        seq.append(protocol.sumcheck_prove(cpu, vp, tref.OracleIOPTranscript(workloads.SUMCHECK_LABEL), f))
        finals_s.append(f)
    assert batched == seq
    assert finals_b == finals_s
