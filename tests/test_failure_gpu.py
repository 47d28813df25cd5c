"""Failure paths and the runtime audit, on the GPU, with every failure made
on the host (no GPU fault, trap or hang is ever provoked):

- an injected pool-allocation failure (hp_cuda_v1_debug_inject_failure, the
  library's own link-time wrapper of cudaMallocFromPoolAsync) makes the call
  return InvalidState with its output slots nulled, and the context keeps
  working (bridge.h:22-27 of the reference: on failure, partial resources
  are cleaned and output slots nulled);
- an injected execution failure (a synchronisation that completes but
  reports cudaErrorLaunchFailure) poisons the sumcheck prover state: every
  later round and the final evaluations are InvalidState, while a new state
  on the same context proves correctly (bridge.h:26-27: an execution
  failure poisons the state);
- a handle destructor that fails aborts the process, as the reference's
  backend does (ascend910b3/mod.rs:46-47);
- the runtime audit: one proof step with resident witnesses makes no device
  or host allocation outside the context's stream-ordered pool and moves no
  table-sized buffer across PCIe/C2C (the reference's runtime audit,
  native/CMakeLists.txt:106-116)."""
import ctypes
import os
import subprocess
import sys
import textwrap

import pytest

from hyperplonk_gb300 import _native, snark
from hyperplonk_gb300.errors import InvalidState
from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial

pytestmark = pytest.mark.gpu

ALLOC, SYNC, NONE = _native.INJECT_POOL_ALLOCATION, _native.INJECT_SYNCHRONIZE, _native.INJECT_NONE
MEMORY_ALLOCATION, LAUNCH_FAILURE = 2, 719  # cudaErrorMemoryAllocation, cudaErrorLaunchFailure


@pytest.fixture(autouse=True)
def disarm():
    _native.inject_failure(NONE, 0)
    yield
    _native.inject_failure(NONE, 0)


def _tables(oracle, nv, seed, k=2):
    return [oracle.random_fr(seed, 1 << nv, first=j << nv) for j in range(k)]


def test_allocation_failure_nulls_output_and_context_recovers(gpu, cpu, oracle):
    nv = 10
    tabs = _tables(oracle, nv, 61)
    gm = [gpu.mle_from_evaluations(nv, t) for t in tabs]
    addrs = (ctypes.c_void_p * 2)(gm[0].address, gm[1].address)
    coefs = b"".join(c.to_bytes(32, "little") for c in (3, 5))
    out = ctypes.c_void_p(0x1234)
    before = _native.runtime_counters()["injected_failures"]
    _native.inject_failure(ALLOC, 1)
    st = gpu.lib.hp_cuda_v1_mle_linear_combination(gpu.ctx.raw, nv, addrs, _native.buf(coefs), 2,
                                                   ctypes.byref(out))
    assert (st.kind, st.native_code) == (2, MEMORY_ALLOCATION)
    assert not out.value
    assert _native.runtime_counters()["injected_failures"] == before + 1
    # the same call succeeds afterwards and equals the oracle
    got = gpu.download(gpu.linear_combination(gm, [3, 5]))
    cm = [cpu.mle_from_evaluations(nv, t) for t in tabs]
    assert got == cpu.linear_combination(cm, [3, 5]).evaluations


@pytest.mark.parametrize("nth", [1, 2, 3])
def test_allocation_failure_in_state_create(gpu, cpu, oracle, nth):
    nv = 8
    tabs = _tables(oracle, nv, 62, 4)
    gm = [gpu.mle_from_evaluations(nv, t) for t in tabs]
    vp = VirtualPolynomial(nv)
    vp.add_mle_list([gm[0], gm[1]], 7)
    vp.add_mle_list([gm[2], gm[3], gm[0]], 9)
    _native.inject_failure(ALLOC, nth)
    try:
        gpu.prover_init(vp)
        armed_left = True  # the create made fewer than nth allocations
    except InvalidState as e:
        assert f"native_code={MEMORY_ALLOCATION}" in str(e)
        armed_left = False
    _native.inject_failure(NONE, 0)
    if armed_left:
        pytest.skip(f"prover state creation makes fewer than {nth} pool allocations")
    # a fresh state on the same context agrees with the oracle round for round
    cvp = VirtualPolynomial(nv)
    cm = [cpu.mle_from_evaluations(nv, t) for t in tabs]
    cvp.add_mle_list([cm[0], cm[1]], 7)
    cvp.add_mle_list([cm[2], cm[3], cm[0]], 9)
    sg, sc = gpu.prover_init(vp), cpu.prover_init(cvp)
    ch = None
    for k in range(nv):
        assert gpu.prove_round_and_update_state(sg, ch) == cpu.prove_round_and_update_state(sc, ch)
        ch = 1000 + k


def test_allocation_failure_in_commit(gpu, cpu, oracle):
    nv = 9
    layers = oracle.srs_layers(nv, 63)
    pg = gpu.prepare_prover_param(nv, [oracle.affine_to_packets(l) for l in layers])
    t = oracle.random_fr(64, 1 << nv)
    m = gpu.mle_from_evaluations(nv, t)
    _native.inject_failure(ALLOC, 1)
    with pytest.raises(InvalidState):
        gpu.commit(pg, m)
    _native.inject_failure(NONE, 0)
    pc = cpu.prepare_prover_param(nv, layers)
    assert gpu.commit(pg, m) == cpu.commit(pc, cpu.mle_from_evaluations(nv, t))


def _degree2(be, mles):
    vp = VirtualPolynomial(mles[0].num_vars)
    vp.add_mle_list([mles[0], mles[1]], 11)
    vp.add_mle_list([mles[1]], 13)
    return vp


def test_execution_failure_poisons_the_round_state(gpu, cpu, oracle):
    nv = 9
    tabs = _tables(oracle, nv, 65)
    gm = [gpu.mle_from_evaluations(nv, t) for t in tabs]
    cm = [cpu.mle_from_evaluations(nv, t) for t in tabs]
    warm = gpu.prover_init(_degree2(gpu, gm))  # grows the context's result mailbox first
    gpu.prove_round_and_update_state(warm, None)
    s = gpu.prover_init(_degree2(gpu, gm))
    assert gpu.prove_round_and_update_state(s, None)
    _native.inject_failure(SYNC, 1)
    with pytest.raises(InvalidState) as e:
        gpu.prove_round_and_update_state(s, 5)
    assert f"native_code={LAUNCH_FAILURE}" in str(e.value)
    _native.inject_failure(NONE, 0)
    # poisoned: correct requests now fail too, without advancing anything
    for _ in range(2):
        with pytest.raises(InvalidState):
            gpu.prove_round_and_update_state(s, 5)
    with pytest.raises(InvalidState):
        gpu.final_evaluations(s, 5)
    del s  # destroying a poisoned state succeeds (a failure would abort)
    # the context is healthy: a new state matches the oracle in every round
    sg, sc = gpu.prover_init(_degree2(gpu, gm)), cpu.prover_init(_degree2(cpu, cm))
    ch = None
    for k in range(nv):
        assert gpu.prove_round_and_update_state(sg, ch) == cpu.prove_round_and_update_state(sc, ch)
        ch = 77 + k
    assert gpu.final_evaluations(sg, ch) == cpu.final_evaluations(sc, ch)


@pytest.mark.parametrize("nth", [2, 3])
def test_execution_failure_poisons_prove_rounds(gpu, oracle, nth):
    """nv = 20, a degree-2 shape with 5 slots: rounds 1 and 2 (2^19, 2^18
    pairs) run one launch each (one synchronisation per round), rounds 3..20
    (2^17 pairs and fewer) in one resident launch (one synchronisation at its
    end): the failure hits a per-round synchronisation (nth = 2) or the
    resident launch's (nth = 3)."""
    from hyperplonk_gb300.transcript import IOPTranscript
    nv = 20
    gm = [gpu.mle_from_evaluations(nv, t) for t in _tables(oracle, nv, 66)]

    def transcript():
        t = IOPTranscript(b"poison")
        t.append_message(b"x", b"y")
        return t.native_merlin()

    expect = gpu.prove_rounds(gpu.prover_init(_degree2(gpu, gm)), transcript(), nv)  # also grows the mailbox
    s = gpu.prover_init(_degree2(gpu, gm))
    _native.inject_failure(SYNC, nth)
    with pytest.raises(InvalidState):
        gpu.prove_rounds(s, transcript(), nv)
    _native.inject_failure(NONE, 0)
    with pytest.raises(InvalidState):
        gpu.prove_rounds(s, transcript(), nv)
    fresh = gpu.prover_init(_degree2(gpu, gm))
    assert gpu.prove_rounds(fresh, transcript(), nv) == expect


def test_failed_destructor_aborts(tmp_path):
    """A handle whose destroy call fails (here: the retire of an address the
    context never handed out) aborts the process instead of passing silently."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = textwrap.dedent("""
        import sys
        sys.path.insert(0, %r)
        from hyperplonk_gb300.backend import CudaBackend, CudaMle
        be = CudaBackend(0)
        m = CudaMle(be.ctx, 0x1000, 4)
        del m
        print("not reached")
    """ % root)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=root)
    assert r.returncode != 0
    assert "buffer_retire failed while destroying a handle" in r.stderr
    assert "not reached" not in r.stdout


def test_prove_step_moves_no_table_across_the_link(gpu):
    """Witnesses resident: one proof step allocates only from the context's
    stream-ordered pool and copies only small values between host and
    device (challenges, points, commitments' partial sums, round messages
    through the mapped mailbox)."""
    nv = 14
    table = 32 << nv
    layers = gpu.generate_srs(nv, 0)
    sel, wit, perm, pub = snark.vanilla_fixture(nv, 2, wired=True)
    pk = snark.preprocess(gpu, nv, 16, sel, perm, layers, commit=False)
    del layers
    wm = gpu.mle_from_evaluations_many(nv, wit)
    snark.prove(gpu, pk, pub, None, witness_mles=wm)  # warm-up: mailbox, worker streams, events
    c0 = _native.runtime_counters()
    proof = snark.prove(gpu, pk, pub, None, witness_mles=wm).to_bytes()
    c1 = _native.runtime_counters()
    d = {k: c1[k] - c0[k] for k in c0}
    print("runtime calls in one proof step:", d)
    assert d["device_allocs"] == 0 and d["host_allocs"] == 0
    assert d["other_copies"] == 0
    assert d["h2d_bytes"] < table // 4, d
    assert d["d2h_bytes"] < table // 4, d
    assert d["pool_allocs"] > 0
    assert len(proof) > 0
