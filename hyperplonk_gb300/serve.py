"""Continuous-batching HyperPlonk prove server on one GPU.

A request is (num_vars, witness tables, public inputs) for the vanilla-plonk
circuit of that size.  The server keeps, per lane, one device context with
the SRS of nv_max variables prepared in HBM (commits and openings of every
smaller circuit use its layers nv_max - nv.., exactly what the reference's
trimmed prover parameters hold) and the selector / permutation oracles of
each circuit size; witness MLEs and every derived table stay on the device
for the life of a proof.

Admission: a request is admitted to the lane with the fewest proofs in flight
when its device memory fits the budget and the lane has a free slot;
otherwise it waits in arrival order.  A request's memory is the measured
high-water mark of one proof of its size alone (ProofServer.prepare with
measure=True: the lane context's pool high-water mark over one proof, minus
the memory in use before it), else a table-count upper estimate.  Requests that arrive while others are
on the GPU start as soon as memory and slots free up.

Coalescing: each in-flight proof runs the unchanged prover driver
(snark.prove) in its own host thread against the lane's CoalescingBackend.
MSM commitments and sumcheck rounds do not run when called: the call waits
until every proof thread of the lane is waiting on such a call (or has
finished), and then all pending calls of the lane run together -- every
pending commitment in one multi_commit (concurrent MSMs on the context's
worker streams) and every pending sumcheck round in one batch_prove_round.
Other backend calls run at once, one at a time per context.  Several lanes
overlap one lane's host work (transcript, serialisation) and latency-bound
phases with another's device work; a lane's proofs wait for each other at
every coalesced step, so few slots per lane and several lanes serve a
mixed-size stream best (measured on GB300, nv 16..22 at 1.5x the plain
capacity with pinned request witnesses: 4 lanes x 2 slots 1.09x the plain
throughput; with 2 lanes x 6 slots about the same as plain).

Each proof is byte-identical to the same request proven alone: the device
work of a proof does not depend on what it is batched with (tests check it).
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

from . import snark
from .backend import CudaBackend
from .errors import InvalidParameters

# Device bytes one in-flight proof of 2^nv gates may hold, in Fr tables of 2^nv,
# for sizes whose use has not been measured: 3 witnesses, 6 nums/denoms,
# frac, prod, 2 product factors, eq tables, the sumcheck fold slots of both
# zero-checks and the batch opening, merged opening polynomials and MSM
# scratch -- an upper estimate (prepare(measure=True) replaces it by the
# measured high-water mark of one proof).
TABLES_PER_PROOF = 64


def proof_hbm_estimate(num_vars: int) -> int:
    return TABLES_PER_PROOF * 32 * (1 << num_vars)


class _Op:
    __slots__ = ("kind", "payload", "result", "error", "done")

    def __init__(self, kind: str, payload):
        self.kind, self.payload = kind, payload
        self.result = self.error = None
        self.done = threading.Event()


class Lane:
    """One device context with its prepared SRS, circuit keys and the
    coalescing scheduler of the proof threads bound to it."""

    def __init__(self, backend, nv_max: int, srs_layers: list):
        self.backend = backend
        self.nv_max = nv_max
        self.param = backend.prepare_prover_param(nv_max, srs_layers)
        self.keys: dict = {}
        self.keys_lock = threading.Lock()
        self.mutex = threading.RLock()      # one host thread at a time on the context
        if hasattr(backend, "ctx"):
            backend.ctx.lock = self.mutex   # handle destructors of proof threads take it too
        self.cond = threading.Condition()   # scheduling state below
        self.running = 0                    # proof threads not waiting on a coalesced call
        self.pending: list[_Op] = []
        self.inflight = 0
        self.flushes = 0
        self.coalesced_calls = 0
        self.view = CoalescingBackend(self)

    # -- proof threads ----------------------------------------------------
    def enter(self) -> None:
        with self.cond:
            self.running += 1

    def leave(self) -> None:
        with self.cond:
            self.running -= 1
            ops = self._take_if_idle()
        if ops:
            self._execute(ops)

    def immediate(self, fn, *args):
        with self.mutex:
            return fn(*args)

    def coalesce(self, kind: str, payload):
        op = _Op(kind, payload)
        with self.cond:
            self.pending.append(op)
            self.running -= 1
            ops = self._take_if_idle()
        if ops:
            self._execute(ops)
        op.done.wait()
        if op.error is not None:
            raise op.error
        return op.result

    def _take_if_idle(self) -> list:
        if self.running == 0 and self.pending:
            ops, self.pending = self.pending, []
            return ops
        return []

    def _execute(self, ops: list) -> None:
        be = self.backend
        with self.mutex:
            self.flushes += 1
            self.coalesced_calls += len(ops)
            msm = [o for o in ops if o.kind == "msm"]
            rounds = [o for o in ops if o.kind == "round"]
            if msm:
                param = msm[0].payload[0]
                flat = [m for o in msm for m in o.payload[1]]
                try:
                    out = be.multi_commit(param, flat) if all(o.payload[0] is param for o in msm) else None
                except Exception:  # attribute the failure to its own call below
                    out = None
                if out is None:
                    for o in msm:
                        self._run_alone(o, lambda p=o.payload: be.multi_commit(p[0], p[1]))
                else:
                    k = 0
                    for o in msm:
                        o.result = out[k:k + len(o.payload[1])]
                        k += len(o.payload[1])
            if rounds:
                out = None
                if hasattr(be, "batch_prove_round"):
                    try:
                        out = be.batch_prove_round([o.payload[0] for o in rounds], [o.payload[1] for o in rounds])
                    except Exception:  # nothing advanced: run each alone to report its own error
                        out = None
                if out is None:
                    for o in rounds:
                        self._run_alone(o, lambda p=o.payload: be.prove_round_and_update_state(p[0], p[1]))
                else:
                    for o, r in zip(rounds, out):
                        o.result = r
        with self.cond:
            self.running += len(ops)
        for o in ops:
            o.done.set()

    @staticmethod
    def _run_alone(op: _Op, fn) -> None:
        try:
            op.result = fn()
        except Exception as e:  # noqa: BLE001 -- re-raised in the proof thread
            op.error = e

    def measure_proof_memory(self, num_vars: int, circuit_seed: int, num_pub: int) -> int:
        """Device bytes one proof of this size takes on this lane's context at
        its peak: the pool's high-water mark over one proof of the circuit's
        own witness, run alone, minus the bytes in use before it."""
        pk = self.proving_key(num_vars, circuit_seed, num_pub)
        wit = snark.vanilla_witness(num_vars, circuit_seed, circuit_seed)
        pub = [int.from_bytes(wit[0][32 * i:32 * i + 32].tobytes(), "little") for i in range(pk.num_pub_input)]
        with self.mutex:
            ctx = self.backend.ctx
            before, _, _ = ctx.memory(reset_high=True)
            snark.prove(self.backend, pk, pub, wit)
            _, high, _ = ctx.memory()
        return max(0, high - before)

    # -- circuits -----------------------------------------------------------
    def proving_key(self, num_vars: int, circuit_seed: int, num_pub: int) -> snark.ProvingKey:
        key = (num_vars, circuit_seed, num_pub)
        with self.keys_lock:
            return self._proving_key(key)

    def _proving_key(self, key) -> snark.ProvingKey:
        num_vars, circuit_seed, num_pub = key
        if key not in self.keys:
            if not 0 < num_vars <= self.nv_max:
                raise InvalidParameters(f"num_vars {num_vars} outside 1..{self.nv_max}")
            sel, _, perm, _ = snark.vanilla_fixture(num_vars, circuit_seed, num_pub)
            with self.mutex:
                sels = [self.backend.mle_from_evaluations(num_vars, s) for s in sel]
                perms = [self.backend.mle_from_evaluations(num_vars, p) for p in perm]
            self.keys[key] = snark.ProvingKey(num_vars, min(num_pub, 1 << num_vars), snark.VANILLA_GATE,
                                              self.param, sels, perms)
        return self.keys[key]


class CoalescingBackend:
    """The backend trait surface the prover driver uses, bound to one lane:
    commitments and sumcheck rounds are coalesced, the rest runs at once."""

    _IMMEDIATE = ("mle_from_evaluations", "linear_combination", "evaluate_mle", "build_eq_x_r",
                  "compute_frac_poly", "compute_product_poly", "compute_nums_and_denoms",
                  "compute_product_factors", "prover_init", "final_evaluations", "open")

    def __init__(self, lane: Lane):
        self._lane = lane
        for name in self._IMMEDIATE:
            fn = getattr(lane.backend, name)
            setattr(self, name, lambda *a, _fn=fn: lane.immediate(_fn, *a))

    def multi_commit(self, prover_param, polynomials):
        if not polynomials:
            return []
        return self._lane.coalesce("msm", (prover_param, list(polynomials)))

    def commit(self, prover_param, polynomial):
        return self._lane.coalesce("msm", (prover_param, [polynomial]))[0]

    def prove_round_and_update_state(self, state, challenge):
        return self._lane.coalesce("round", (state, challenge))


@dataclass
class Ticket:
    num_vars: int
    witnesses: list
    pub: list
    submitted: float
    admitted: float | None = None
    finished: float | None = None
    proof: bytes | None = None
    error: BaseException | None = None
    lane: int | None = None
    done: threading.Event = field(default_factory=threading.Event)


class ProofServer:
    """submit() / poll() / wait() prove server (the serve API: create,
    submit, poll) over `lanes` device contexts of one GPU."""

    def __init__(self, device: int = 0, nv_max: int = 22, lanes: int = 4, hbm_budget_bytes: int | None = None,
                 slots_per_lane: int = 2, circuit_seed: int = 2, srs_seed: int = 0, num_pub: int = 16,
                 srs_layers: list | None = None, backend_factory=None, transcript_cls=None):
        """`backend_factory()` makes one lane's backend (default: a CudaBackend
        context on `device`); `srs_layers` default to the testing SRS of
        nv_max variables from `srs_seed`, generated on the device."""
        if backend_factory is None:
            backend_factory = lambda: CudaBackend(device)  # noqa: E731
        if srs_layers is None:
            srs_layers = CudaBackend(device).generate_srs(nv_max, srs_seed)
        self.lanes = [Lane(backend_factory(), nv_max, srs_layers) for _ in range(lanes)]
        self.nv_max, self.circuit_seed, self.num_pub = nv_max, circuit_seed, num_pub
        if transcript_cls is None:
            from .transcript import IOPTranscript as transcript_cls
        self.transcript_cls = transcript_cls
        self.slots_per_lane = slots_per_lane
        if hbm_budget_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info(device)
            hbm_budget_bytes = free // 2
        self.stats = {"flushes": 0, "coalesced_calls": 0}
        self.budget = hbm_budget_bytes
        self.measured: dict[int, int] = {}  # num_vars -> device bytes of one proof (prepare(measure=True))
        self.in_use = 0
        self.lock = threading.Lock()
        self.queue: list[Ticket] = []
        self.tickets: list[Ticket] = []
        self.threads: list[threading.Thread] = []

    def prepare(self, num_vars_list, measure: bool = False) -> None:
        """Upload the circuit oracles of these sizes to every lane ahead of
        requests; with `measure`, also measure each size's device memory per
        proof (one proof alone on the first lane) for admission."""
        for lane in self.lanes:
            for nv in num_vars_list:
                lane.proving_key(nv, self.circuit_seed, self.num_pub)
        if measure:
            for nv in sorted(set(num_vars_list)):
                self.measured[nv] = self.lanes[0].measure_proof_memory(nv, self.circuit_seed, self.num_pub)

    def proof_bytes(self, num_vars: int) -> int:
        """Device memory admission counts for one proof of this size."""
        return self.measured.get(num_vars) or proof_hbm_estimate(num_vars)

    def submit(self, num_vars: int, witnesses: list, pub: list) -> int:
        if not 0 < num_vars <= self.nv_max:
            raise InvalidParameters(f"num_vars {num_vars} outside 1..{self.nv_max}")
        if self.proof_bytes(num_vars) > self.budget:
            raise InvalidParameters("request does not fit the HBM budget")
        t = Ticket(num_vars, witnesses, pub, time.perf_counter())
        with self.lock:
            self.tickets.append(t)
            self.queue.append(t)
            self._admit()
        return len(self.tickets) - 1

    def poll(self, ticket: int) -> bytes | None:
        t = self.tickets[ticket]
        if t.error is not None:
            raise t.error
        return t.proof

    def wait(self, ticket: int, timeout: float | None = None) -> bytes:
        t = self.tickets[ticket]
        if not t.done.wait(timeout):
            raise TimeoutError(f"ticket {ticket} not done")
        return self.poll(ticket)

    def ticket(self, ticket: int) -> Ticket:
        return self.tickets[ticket]

    def close(self) -> None:
        for th in list(self.threads):
            th.join()

    # -- admission (called with self.lock held) -----------------------------
    def _admit(self) -> None:
        while self.queue:
            t = self.queue[0]
            need = self.proof_bytes(t.num_vars)
            lane_i = min(range(len(self.lanes)), key=lambda i: self.lanes[i].inflight)
            lane = self.lanes[lane_i]
            if self.in_use + need > self.budget or lane.inflight >= self.slots_per_lane:
                return
            self.queue.pop(0)
            self.in_use += need
            lane.inflight += 1
            t.lane, t.admitted = lane_i, time.perf_counter()
            lane.enter()
            th = threading.Thread(target=self._prove, args=(t, lane, need), daemon=True)
            self.threads.append(th)
            th.start()

    def _prove(self, t: Ticket, lane: Lane, need: int) -> None:
        try:
            pk = lane.proving_key(t.num_vars, self.circuit_seed, self.num_pub)
            t.proof = snark.prove(lane.view, pk, t.pub, t.witnesses, transcript_cls=self.transcript_cls).to_bytes()
        except BaseException as e:  # noqa: BLE001 -- reported through poll()
            t.error = e
        finally:
            t.finished = time.perf_counter()
            lane.leave()
            with self.lock:
                self.in_use -= need
                lane.inflight -= 1
                self._admit()
            t.done.set()
