"""Prove server scheduling (host logic, no GPU): requests of several sizes
submitted together to lanes over the oracle backend finish, and each proof
equals the same request proven alone."""
from hyperplonk_gb300 import serve, snark


def test_served_proofs_equal_alone_on_oracle(native_lib, oracle):
    import transcript_ref as tref
    nv_max = 6
    layers = oracle.srs_layers(nv_max, 9)
    srv = serve.ProofServer(nv_max=nv_max, lanes=2, hbm_budget_bytes=1 << 40, slots_per_lane=3,
                            srs_layers=layers, backend_factory=oracle.CpuBackend,
                            transcript_cls=tref.OracleIOPTranscript)
    reqs = [(nv, (4 << 32) | i) for i, nv in enumerate([3, 5, 4, 6, 3, 5, 2])]
    tickets = []
    for nv, ws in reqs:
        wit = snark.vanilla_witness(nv, 2, ws)
        pub = [int.from_bytes(wit[0][32 * i:32 * i + 32].tobytes(), "little") for i in range(min(16, 1 << nv))]
        tickets.append((srv.submit(nv, wit, pub), nv, wit, pub))
    got = [srv.wait(t, timeout=600) for t, _, _, _ in tickets]
    srv.close()
    lane = srv.lanes[0]
    cpu = oracle.CpuBackend()
    param = cpu.prepare_prover_param(nv_max, layers)
    for (t, nv, wit, pub), g in zip(tickets, got):
        sel, _, perm, _ = snark.vanilla_fixture(nv, 2)
        pk = snark.ProvingKey(nv, min(16, 1 << nv), snark.VANILLA_GATE, param,
                              [cpu.mle_from_evaluations(nv, s) for s in sel],
                              [cpu.mle_from_evaluations(nv, p) for p in perm])
        alone = snark.prove(cpu, pk, pub, wit, transcript_cls=tref.OracleIOPTranscript).to_bytes()
        assert g == alone, nv
    assert sum(l.flushes for l in srv.lanes) > 0
    assert max(l.coalesced_calls / max(1, l.flushes) for l in srv.lanes) > 1  # calls were batched
    assert all(l.running == 0 and not l.pending for l in srv.lanes)
    assert lane.inflight == 0 and srv.in_use == 0
