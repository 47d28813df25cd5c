#!/usr/bin/env python3
"""Benchmark of the GB300 HyperPlonk prover hot path.

Workloads (--workload):

  prove  (default) -- full HyperPlonk prove of the vanilla-plonk circuit of
         2^nv gates (q_L, q_R, q_M, q_C, w1, w2 uniform, q_O
         = -1, w3 solving the gate, identity permutation over 3 columns, 16
         public inputs, fixture seed 2, testing SRS of nv variables).  One step
         = one proof through the reference-facing C ABI (witness commits,
         gate zero-check, permutation check, 22 evaluations, batch opening),
         proof serialized to bytes.  Metric: HyperPlonk proofs/s, with p50/p99
         proof latency.  The MSM pts/s of a 2^nv commit on the same SRS is
         reported beside it ("msm").
  commit -- one multilinear-KZG commit of a 2^nv-point MLE (the nv = 16
         commit of stream-0 scalars is the commit workload's stated size).
         Metric: MSM pts/s.

  value : inputs already resident in HBM (witness MLEs uploaded before the
          timed loop);
  e2e   : the same through the C ABI from pinned host buffers every step
          (upload of the inputs + the work + results back on the host); for
          prove, a stream of proofs whose next witness upload overlaps the
          current proof (hp_cuda_v1_mle_upload_async), the blocking
          upload-then-prove form beside it as e2e_serial.

Timing: W warm-up steps, then K steps each bracketed by CUDA events on the
backend's own stream (hp_cuda_v1_context_stream), a barrier and
torch.cuda.synchronize() on both sides of the timed loop; a 256 MiB buffer is
written between steps to flush L2 (the prepared SRS, ~2.6 GB at nv=20, is
larger than L2 anyway).  The dominant kernel (k_msm_accumulate) is timed by
the library's own CUDA-event hooks on the same stream.  --impl reference
times the CPU restatement of the reference's CPU path (the oracle: its C
backend, its own prover driver oracle/prover.py and its Python transcript,
all host threads) on one full step of the same workload at the same size per
step, with the oracle's own fixture and SRS generators; it loads nothing of
the product package.

--gpus N without a launcher runs N local ranks through torch.distributed.run
(replicas, one process per GPU).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FQ_MUL_IMAD = 588  # 32-bit-limb CIOS, n = 12: 2n^2 + 2n^2 + n
FR_MUL_IMAD = 264
FQ_MUL_WIDE = 252  # wide multiply-adds of the library's Fq product: 3 x 36 (Karatsuba) + 12 x 12 (reduction rows)
PROVE_SEED = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["prove", "commit", "sumcheck", "batch", "serve"], default="prove")
    ap.add_argument("--requests", type=int, default=28, help="serve workload: requests per offered load")
    ap.add_argument("--lanes", type=int, default=4, help="serve workload: device contexts of the server")
    ap.add_argument("--slots", type=int, default=2, help="serve workload: proofs in flight per lane")
    ap.add_argument("--num-vars", type=int, default=None,
                    help="default 20 (prove, commit, sumcheck); the batch workload's SRS has 22")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="prove workload: skip the batch and serve workloads run beside it (child processes)")
    ap.add_argument("--msm-tuning", default=None, metavar="FILE",
                    help="load an MSM tuning table (hp_cuda_v1_msm_tuning_load) before preparing the SRS")
    ap.add_argument("--autotune", action="store_true",
                    help="prove / commit / batch: run the MSM autotuner on the workload's MSM sizes; prove / "
                         "sumcheck: the sumcheck round-route tuner on the workload's sumcheck shapes; before warm-up")
    return ap.parse_args()


def window_bits(n: int) -> int:
    """Window width the library uses for an n-point layer (size rule or tuned entry)."""
    from hyperplonk_gb300 import tuning
    return tuning.query(tuning.ALONE, n)[0]


# MSM geometry of this run: the tuning file loaded and the autotuner's entries
TUNING_INFO: dict = {}


def load_tuning(args, local: int) -> None:
    if args.msm_tuning:
        import torch
        from hyperplonk_gb300 import tuning
        tuning.load(args.msm_tuning, device=torch.cuda.get_device_name(local))
        TUNING_INFO["file"] = args.msm_tuning


def autotune(args, be, params, alone_nvs, shared_nvs) -> None:
    """--autotune: measure the geometry of the workload's MSM sizes (alone)
    and of its shared launch of small MSMs, untimed, before the warm-up."""
    if not args.autotune:
        return
    from hyperplonk_gb300 import tuning
    t0 = time.perf_counter()
    entries = tuning.autotune(be, params, sorted(set(alone_nvs)))
    if shared_nvs:
        entries += tuning.autotune(be, params, list(shared_nvs)[:64], mode=tuning.SHARED)
    TUNING_INFO["autotune_s"] = round(time.perf_counter() - t0, 2)
    TUNING_INFO["autotune"] = [
        {"mode": "alone" if e.mode == tuning.ALONE else "shared", "size": e.size, "window_bits": e.window_bits,
         "segment": e.segment, "chunk": e.chunk, "model_ms": round(e.model_ms, 4), "tuned_ms": round(e.tuned_ms, 4)}
        for e in entries]


def autotune_sumcheck(args, be, run_once) -> None:
    """--autotune: tune the sumcheck round routes of every sumcheck shape one
    untimed run of the workload meets (run_once(backend_view)), before the
    warm-up."""
    if not args.autotune:
        return
    from hyperplonk_gb300 import tuning
    t0 = time.perf_counter()
    view = tuning.SumcheckTuningBackend(be)
    run_once(view)
    TUNING_INFO["sumcheck_autotune_s"] = round(time.perf_counter() - t0, 2)
    TUNING_INFO["sumcheck_routes"] = [
        {"shape_nv_arity_slots": list(key), "pairs": r.pairs, "kernel": r.kernel, "blocks_per_sm": r.blocks_per_sm,
         "default_kernel": r.default_kernel, "default_us": round(r.default_us, 2), "tuned_us": round(r.tuned_us, 2)}
        for key, recs in view.tuned.items() for r in recs]


def shared_mix(nvs) -> list:
    """The sizes that run_msms puts into the shared launch: fewer than 2^22
    (window, point) records."""
    return [k for k in nvs if math.ceil(256 / window_bits(1 << k)) * (1 << k) < (1 << 22)]


def accumulate_imad(n: int) -> int:
    """Algorithmic work of k_msm_accumulate for one n-point MSM: one XYZZ
    mixed addition (10 Fq muls) per (point, window) record."""
    return math.ceil(256 / window_bits(n)) * n * 10 * FQ_MUL_IMAD


def msm_accounting_imad(n: int) -> float:
    """Fixed algorithmic work of an n-point MSM: min_c ceil(255/c)(10n + 14*2^c)
    Fq multiplications at 588 IMAD each."""
    best = min(math.ceil(255 / c) * (10 * n + 14 * (1 << c)) for c in range(8, 21))
    return best * FQ_MUL_IMAD


def sumcheck_work(nv: int) -> tuple[int, int]:
    """Algorithmic (IMAD, HBM bytes) of one degree-2 sumcheck prove over six
    2^nv tables: 12 Fr muls per pair in round 1, 24 (fold + message) per pair
    in every later round; six tables read in round 1, then each round reads
    the previous round's tables and writes the folded halves."""
    n = 1 << nv
    muls = 12 * (n // 2) + 24 * (n // 2 - 1)
    return muls * FR_MUL_IMAD, 192 * n + 192 * (n - 2) + 192 * (n // 2 - 1)


def prove_msm_sizes(nv: int) -> list:
    """MSMs of one proof: 3 witness commits, frac and prod commits (2^nv each)
    and the batch opening's nv quotient MSMs (2^(nv-1) .. 1)."""
    return [1 << nv] * 5 + [1 << (nv - 1 - i) for i in range(nv)]


# ---------------------------------------------------------------------------
# distributed plumbing
# ---------------------------------------------------------------------------

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baselines (oracle restatement of the reference CPU path)
# ---------------------------------------------------------------------------

def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc
    return orc


class CpuMsmSample:
    """The oracle's multithreaded Pippenger MSM (the CPU restatement of ark-ec
    msm_unchecked as used by backend/src/cpu/multilinear_kzg.rs:40-59): one
    multilinear-KZG commit of 2^nv stream-0 scalars over layer 0 of the
    oracle's testing SRS of nv variables (seed 0) -- the commit workload at
    its own size."""

    def __init__(self, nv: int):
        orc = _oracle()
        self.orc, self.nv = orc, nv
        self.threads = orc.set_threads(0)
        self.bases = orc.srs_layers(nv, 0)[0]
        self.scalars = orc.random_fr(0, 1 << nv)

    def step(self) -> float:
        t0 = time.perf_counter()
        self.orc.msm(self.bases, self.scalars)
        return time.perf_counter() - t0


class CpuProveSample:
    """The oracle's own prover (oracle/prover.py: the reference's prover
    driver restated over the C restatement of backend/src/cpu, with the
    oracle's Python transcript) proving the full-prove workload's circuit of
    2^nv gates; fixture and testing SRS from the oracle's generators (or the
    SRS layers passed in, 96-byte affine).  No product code runs."""

    def __init__(self, nv: int, srs_layers=None, wired: bool = False):
        orc = _oracle()
        import prover as oprover  # oracle/prover.py (path set by _oracle)
        self.op, self.nv = oprover, nv
        self.threads = orc.set_threads(0)
        self.cpu = orc.CpuBackend()
        sel, self.wit, perm, self.pub = oprover.vanilla_fixture(nv, PROVE_SEED, wired=wired)
        layers = srs_layers if srs_layers is not None else orc.srs_layers(nv, 0)
        self.pk = oprover.ProvingKey(self.cpu, nv, min(16, 1 << nv), sel, perm, layers)

    def step(self) -> float:
        t0 = time.perf_counter()
        self.proof = self.op.prove(self.cpu, self.pk, self.pub, self.wit)
        return time.perf_counter() - t0


class CpuSumcheckSample:
    """The oracle's sumcheck prover (backend/src/cpu/sum_check.rs restated)
    driven by oracle/prover.py with the oracle's Python transcript, on the
    degree-2 instance at 2^nv (seed 1)."""

    def __init__(self, nv: int, seed: int = 1):
        orc = _oracle()
        import prover as oprover
        self.op, self.nv, self.seed = oprover, nv, seed
        self.threads = orc.set_threads(0)
        self.instance = oprover.sumcheck_instance(nv, seed)

    def step(self) -> float:
        t0 = time.perf_counter()
        self.op.sumcheck_prove_instance(self.nv, self.seed, self.instance)
        return time.perf_counter() - t0


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------

class Session:
    def __init__(self, local: int):
        import torch
        from hyperplonk_gb300.backend import CudaBackend
        self.torch = torch
        torch.cuda.set_device(local)
        self.local = local
        self.be = CudaBackend(local)
        self.lib = self.be.lib
        self.stream = torch.cuda.ExternalStream(self.be.ctx.stream(), device=torch.device("cuda", local))
        self.flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def check(self, status, op):
        from hyperplonk_gb300.errors import check_status
        check_status(status, op)

    def launches(self) -> int:
        c = ctypes.c_uint64()
        self.check(self.lib.hp_cuda_v1_kernel_launch_count(ctypes.byref(c)), "kernel_launch_count")
        return c.value

    def profile(self, on: bool):
        self.check(self.lib.hp_cuda_v1_context_profile(self.be.ctx.raw, 1 if on else 0), "context_profile")

    def profile_read(self, name: bytes):
        ms, cnt = ctypes.c_double(), ctypes.c_uint64()
        self.check(self.lib.hp_cuda_v1_context_profile_read(self.be.ctx.raw, name, ctypes.byref(ms),
                                                            ctypes.byref(cnt)), "profile_read")
        return ms.value, cnt.value

    def timed(self, fn, steps):
        torch = self.torch
        per = []
        with torch.cuda.stream(self.stream):
            for _ in range(steps):
                self.flush_buf.fill_(1)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(self.stream)
                fn()
                b.record(self.stream)
                b.synchronize()
                per.append(a.elapsed_time(b) / 1e3)
        return per

    def srs_layers(self, nv: int, seed: int):
        import numpy as np
        from hyperplonk_gb300 import _native
        total = (1 << (nv + 1)) - 1
        packets = np.empty(total * 97, dtype=np.uint8)
        self.check(self.lib.hp_cuda_v1_srs_generate(self.be.ctx.raw, nv, seed, _native.buf(packets), total),
                   "srs_generate")
        layers, off = [], 0
        for i in range(nv + 1):
            cnt = 1 << (nv - i) if i < nv else 1
            layers.append(packets[97 * off:97 * (off + cnt)])
            off += cnt
        return layers

    def pinned(self, arr):
        t = self.torch.empty(arr.nbytes, dtype=self.torch.uint8, pin_memory=True)
        t.numpy()[:] = arr.reshape(-1)
        return t

    def wide_rate(self) -> float:
        """mad.wide.u32 (32x32->64 multiply-add) issues per second on this GPU."""
        probe = ctypes.CDLL(str(ROOT / "bench_probe" / "_build" / "libhp_probe.so"))
        probe.hp_probe_wide_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        w = ctypes.c_double()
        rc = probe.hp_probe_wide_rate(self.local, ctypes.byref(w))
        if rc != 0:
            raise RuntimeError(f"wide-multiply probe failed ({rc})")
        return w.value

    def integer_rates(self):
        probe = ctypes.CDLL(str(ROOT / "bench_probe" / "_build" / "libhp_probe.so"))
        probe.hp_probe_integer_rates.argtypes = [ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 3
        imad, fqm, frm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rc = probe.hp_probe_integer_rates(self.local, ctypes.byref(imad), ctypes.byref(fqm), ctypes.byref(frm))
        if rc != 0:
            raise RuntimeError(f"integer probe failed ({rc})")
        return imad.value, fqm.value, frm.value


def measure(s: Session, pg, steps: int, value_fn, e2e_fn, profile: bool = True, hooks=()):
    """Timed loops; returns (value step seconds list, e2e list, launches, clocks, accumulate ms/launches,
    msm ms/launches).  With `profile`, the library's event hooks time the value loop only; the totals
    of the hook names in `hooks` are stored in s.hook_totals."""
    if profile:
        s.profile(True)
    clocks = ClockSampler(s.local)
    barrier(pg)
    s.torch.cuda.synchronize()
    clocks.start()
    l0 = s.launches()
    s.torch.cuda.nvtx.range_push("timed_value")  # ncu --nvtx --nvtx-include "timed_value/" selects this loop
    per = s.timed(value_fn, steps)
    s.torch.cuda.synchronize()
    s.torch.cuda.nvtx.range_pop()
    l1 = s.launches()
    barrier(pg)
    clk = clocks.stop()
    acc = s.profile_read(b"msm_accumulate")
    msm = s.profile_read(b"msm")
    s.hook_totals = {h: s.profile_read(h.encode()) for h in hooks}
    if profile:
        s.profile(False)
    barrier(pg)
    s.torch.cuda.synchronize()
    s.torch.cuda.nvtx.range_push("timed_e2e")  # the second loop (e2e, or the batch workload's plain run)
    per_e2e = s.timed(e2e_fn, steps)
    s.torch.cuda.synchronize()
    s.torch.cuda.nvtx.range_pop()
    barrier(pg)
    return per, per_e2e, l1 - l0, clk, acc, msm


def common_fields(args, world, metric, value, unit, step_s, workload, config, e2e, nl, clk) -> dict:
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 limbs (Fr 8x32, Fq 12x32 Montgomery)",
            "data": "synthetic: ChaCha20 fixture streams, device-generated testing SRS",
            "config": dict({"workload": workload, "l2": "256 MiB flush between steps; inputs > L2",
                            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}, **config),
            "e2e": e2e, "gpu_launches": int(nl), "clocks": clk,
            **({"msm_tuning": dict(TUNING_INFO)} if TUNING_INFO else {})}


def run_sumcheck(args, world, rank, local, pg):
    """Sumcheck prove of the degree-2 instance (6 tables, 4 arity-2 products,
    seed 1) with the host transcript; value: tables resident; e2e: a stream of
    proves, each from its own upload of the six tables from pinned host
    memory, the upload of prove i+1 queued on the context's ingress stream
    before prove i runs; e2e_serial: upload, then prove, one at a time."""
    from hyperplonk_gb300 import protocol, workloads
    from hyperplonk_gb300.transcript import IOPTranscript
    s = Session(local)
    be = s.be
    nv = args.num_vars or 20
    tables = [s.pinned(t).numpy() for t in workloads.sumcheck_tables(nv, 1)]
    coefs = workloads.sumcheck_coefficients(1)
    resident = [be.mle_from_evaluations(nv, t) for t in tables]
    out = {}
    autotune_sumcheck(args, be, lambda view: protocol.sumcheck_prove(
        view, workloads.sumcheck_polynomial(nv, resident, coefs), IOPTranscript(workloads.SUMCHECK_LABEL), []))

    def value_fn():
        vp = workloads.sumcheck_polynomial(nv, resident, coefs)
        finals = []
        out["proof"] = protocol.sumcheck_prove(be, vp, IOPTranscript(workloads.SUMCHECK_LABEL), finals)
        out["finals"] = finals

    def e2e_fn():
        m = be.mle_from_evaluations_many(nv, tables)
        vp = workloads.sumcheck_polynomial(nv, m, coefs)
        protocol.sumcheck_prove(be, vp, IOPTranscript(workloads.SUMCHECK_LABEL), [])

    for _ in range(args.warmup):
        value_fn()
        e2e_fn()
    per, per_e2e, nl, clk, _, _ = measure(s, pg, args.steps, value_fn, e2e_fn, hooks=("sumcheck_round",))
    rk_ms, rk_n = s.hook_totals["sumcheck_round"]
    step_s = max_over_ranks(pg, statistics.mean(per))
    e2e_s = max_over_ranks(pg, statistics.mean(per_e2e))

    def e2e_pipelined(steps: int) -> float:
        """`steps` proves, each from its own upload of the six tables, the
        upload of prove i+1 queued (hp_cuda_v1_mle_upload_async) before prove
        i runs, the L2 flush between proves inside the timed region; seconds
        per prove (CUDA events on the backend's stream around the loop)."""
        torch = s.torch
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s.stream):
            torch.cuda.synchronize()
            a.record(s.stream)
            nxt = be.mle_upload_async(nv, tables)
            for i in range(steps):
                cur = nxt
                if i + 1 < steps:
                    nxt = be.mle_upload_async(nv, tables)
                m = cur.wait()
                finals = []
                proof = protocol.sumcheck_prove(be, workloads.sumcheck_polynomial(nv, m, coefs),
                                                IOPTranscript(workloads.SUMCHECK_LABEL), finals)
                out["pipelined"] = (proof.to_bytes(), finals)
                s.flush_buf.fill_(1)
            b.record(s.stream)
            b.synchronize()
        return a.elapsed_time(b) / 1e3 / steps

    e2e_pipelined(2)  # warm-up
    pipe_s = max_over_ranks(pg, e2e_pipelined(args.steps))
    if out["pipelined"] != (out["proof"].to_bytes(), out["finals"]):
        raise RuntimeError("the pipelined end-to-end prove differs from the resident one")
    imad_work, hbm_bytes = sumcheck_work(nv)
    imad, _, _ = s.integer_rates()
    kernel_s = rk_ms / 1e3 / args.steps
    peaks = measured_peaks()
    result = common_fields(
        args, world, "sumcheck proofs/s", world / step_s, "proofs/s", step_s,
        f"sumcheck prove, degree 2: 6 MLEs of 2^{nv} Fr (seed 1), 4 arity-2 products (0,1),(2,3),(4,5),(0,3) "
        f"with uniform coefficients, host Merlin transcript, {nv} round messages + 6 final values",
        {"num_vars": nv},
        {"value": world / pipe_s, "unit": "proofs/s", "ms_per_step": pipe_s * 1e3,
         "h2d_bytes_per_step": 6 * 32 * (1 << nv), "d2h_bytes_per_step": 32 * (3 * nv + 6),
         "how": "table upload of prove i+1 (hp_cuda_v1_mle_upload_async, ingress stream) overlapping prove i; "
                "every prove's tables copied from pinned host memory and its messages read back inside the "
                "timed loop"}, nl, clk)
    result["e2e_serial"] = {"value": world / e2e_s, "unit": "proofs/s", "ms_per_step": e2e_s * 1e3,
                            "h2d_bytes_per_step": 6 * 32 * (1 << nv), "d2h_bytes_per_step": 32 * (3 * nv + 6),
                            "how": "each step uploads its tables (blocking) and then proves"}
    result["roofline"] = {
        "bound": "imad",
        "kernel": "sumcheck rounds: k_sumcheck_round_pp (round 1) and k_sumcheck_fold + k_sumcheck_round_pp "
                  "(round 2, p(0) from the claim), then one k_sumcheck_resident launch for rounds 3..20 (its "
                  "duration includes the host Merlin step of each of those rounds)",
        "achieved": imad_work / kernel_s / 1e12, "peak": imad / 1e12, "unit": "TIMAD/s",
        "frac": imad_work / kernel_s / imad, "traffic": None,
        "peak_source": "measured live: mad.lo.u32 issue rate on this GPU (libhp_probe)",
        "launches": rk_n // max(1, args.steps), "per_proof_kernel_ms": kernel_s * 1e3,
        "algorithmic_imad_per_proof": imad_work, "algorithmic_bytes_per_proof": hbm_bytes,
        "hbm": {"achieved_gbs": hbm_bytes / kernel_s / 1e9, "peak_gbs": peaks.get("hbm_gbs"),
                "frac": hbm_bytes / kernel_s / 1e9 / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}}
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline("sumcheck", nv)
    if rank == 0:
        print(json.dumps(result))


def run_batch(args, world, rank, local, pg):
    """The batch plan (64 MSMs of 2^12..2^22 points over prefixes of SRS
    layer 0 of nv=22, 32 degree-2 sumchecks of 14..22 variables, seed 3):
    value = the batched run (one batch_msm call; sumcheck rounds in lockstep,
    one batch_prove_round call per round) with inputs resident; the plain
    one-at-a-time run of the same inputs is timed beside it and must give the
    same results."""
    from hyperplonk_gb300 import workloads
    from hyperplonk_gb300.transcript import IOPTranscript
    s = Session(local)
    be = s.be
    nv_srs = args.num_vars or 22
    ks, nvs = workloads.batch_plan(3, msm_k=(12, nv_srs), sumcheck_nv=(14, nv_srs))
    layers = s.srs_layers(nv_srs, 0)
    params = be.prepare_prover_param(nv_srs, layers)
    del layers
    autotune(args, be, params, ks, shared_mix(ks))
    wl = workloads.BatchWorkload(be, params, ks, nvs)
    out = {}

    def value_fn():
        out["batched"] = wl.run_batched(IOPTranscript)

    def plain_fn():
        out["plain"] = wl.run_plain(IOPTranscript)

    for _ in range(args.warmup):
        value_fn()
    plain_fn()
    if out["plain"] != out["batched"]:
        raise RuntimeError("batched and plain runs of the batch plan differ")
    per, per_plain, nl, clk, _, _ = measure(s, pg, args.steps, value_fn, plain_fn, profile=False)
    step_s = max_over_ranks(pg, statistics.mean(per))
    plain_s = max_over_ranks(pg, statistics.mean(per_plain))
    points = sum(1 << k for k in ks)
    result = common_fields(
        args, world, "batch-plan runs/s", world / step_s, "runs/s", step_s,
        f"64 MSMs of 2^k points (k uniform in 12..{nv_srs}, {points} points, prefixes of SRS layer 0 nv={nv_srs}) "
        f"+ 32 degree-2 sumchecks (num_vars uniform in 14..{nv_srs}), seed 3, batched",
        {"num_vars": nv_srs, "msm_log_sizes": ks, "sumcheck_num_vars": nvs},
        {"value": None, "unit": "runs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
         "note": "inputs are resident by construction of this workload; see the prove workload for e2e"},
        nl, clk)
    result["plain"] = {"ms_per_run": plain_s * 1e3, "runs_per_s": world / plain_s,
                       "batched_over_plain": plain_s / step_s}
    result["msm_points_per_run"] = points
    if rank == 0:
        print(json.dumps(result))


def run_serve(args, world, rank, local, pg):
    """Poisson arrivals of vanilla-plonk prove requests (circuit of fixture
    seed 2 per size, num_vars uniform in 16..nv_max, independent witnesses
    per request from seed 4) at offered loads 0.5x..2x the plain path's
    capacity, served by ProofServer with the nv_max SRS resident.  The plain
    path proves each request alone, one at a time (its service times give
    the capacity and, replayed as a FIFO queue on the same arrivals, its
    latencies).  Every served proof must equal the request's plain proof."""
    import random
    from hyperplonk_gb300 import serve, snark
    s = Session(local)
    nv_max = args.num_vars or 22
    lo = min(16, nv_max)
    m = args.requests
    rng = random.Random(4)
    nvs = [rng.randint(lo, nv_max) for _ in range(m)]
    # request witnesses arrive in pinned host buffers (uploaded by each proof)
    pinned = [[s.pinned(t) for t in snark.vanilla_witness(nv, 2, (4 << 32) | i)] for i, nv in enumerate(nvs)]
    wits = [[t.numpy() for t in w] for w in pinned]
    pubs = [[int.from_bytes(w[0][32 * j:32 * j + 32].tobytes(), "little") for j in range(min(16, 1 << nv))]
            for nv, w in zip(nvs, wits)]
    layers = s.be.generate_srs(nv_max, 0)
    plain = serve.Lane(s.be, nv_max, layers)
    for nv in sorted(set(nvs)):
        snark.prove(s.be, plain.proving_key(nv, 2, 16), pubs[nvs.index(nv)], wits[nvs.index(nv)])  # warm-up
    service, alone = [], []
    for nv, w, pub in zip(nvs, wits, pubs):
        t0 = time.perf_counter()
        alone.append(snark.prove(s.be, plain.proving_key(nv, 2, 16), pub, w).to_bytes())
        service.append(time.perf_counter() - t0)
    mean_service = statistics.mean(service)
    srv = serve.ProofServer(local, nv_max=nv_max, lanes=args.lanes, slots_per_lane=args.slots, srs_layers=layers)
    srv.prepare(sorted(set(nvs)))
    for i in range(min(4, m)):  # warm-up of the lanes
        srv.wait(srv.submit(nvs[i], wits[i], pubs[i]))

    def pct(xs, q):
        xs = sorted(xs)
        return xs[min(len(xs) - 1, max(0, math.ceil(q * len(xs)) - 1))]

    loads = []
    clk_sampler = ClockSampler(local)
    clk_sampler.start()
    for k, rho in enumerate([0.5, 1.0, 1.5, 2.0]):
        rate = rho / mean_service
        arr_rng = random.Random(400 + k)
        arrivals, t = [], 0.0
        for _ in range(m):
            t += arr_rng.expovariate(rate)
            arrivals.append(t)
        tickets = []
        t0 = time.perf_counter()
        for i, a in enumerate(arrivals):
            delay = t0 + a - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            tickets.append(srv.submit(nvs[i], wits[i], pubs[i]))
        proofs = [srv.wait(tk) for tk in tickets]
        if proofs != alone:
            raise RuntimeError("a served proof differs from the same request proven alone")
        lat = [srv.ticket(tk).finished - srv.ticket(tk).submitted for tk in tickets]
        end = max(srv.ticket(tk).finished for tk in tickets)
        # plain path: FIFO single server over the same arrivals and measured service times
        finish, plat = 0.0, []
        for a, sv in zip(arrivals, service):
            finish = max(finish, a) + sv
            plat.append(finish - a)
        loads.append({"offered_load": rho, "offered_proofs_per_s": rate,
                      "served": {"proofs_per_s": m / (end - t0), "p50_ms": 1e3 * pct(lat, 0.5),
                                 "p99_ms": 1e3 * pct(lat, 0.99)},
                      "plain": {"proofs_per_s": m / finish, "p50_ms": 1e3 * pct(plat, 0.5),
                                "p99_ms": 1e3 * pct(plat, 0.99)}})
    clk = clk_sampler.stop()
    top = loads[-1]
    result = common_fields(
        args, world, "served HyperPlonk proofs/s", top["served"]["proofs_per_s"], "proofs/s",
        1.0 / top["served"]["proofs_per_s"],
        f"prove requests, vanilla-plonk circuits of 2^16..2^{nv_max} gates (num_vars uniform, seed 4), Poisson "
        f"arrivals at 0.5x..2x the plain path's capacity, {m} requests per load, SRS nv={nv_max} resident, "
        f"{args.lanes} lanes x {args.slots} slots",
        {"num_vars": nvs, "requests": m, "lanes": args.lanes, "slots_per_lane": args.slots},
        {"value": top["served"]["proofs_per_s"], "unit": "proofs/s",
         "h2d_bytes_per_step": int(statistics.mean(3 * 32 * (1 << nv) for nv in nvs)),
         "d2h_bytes_per_step": int(statistics.mean(len(b) for b in alone))},
        0, clk)
    result["gpu_launches"] = None
    result["latency_ms"] = {"p50": top["served"]["p50_ms"], "p99": top["served"]["p99_ms"]}
    result["plain_capacity_proofs_per_s"] = 1.0 / mean_service
    result["served_over_plain_at_2x"] = top["served"]["proofs_per_s"] / top["plain"]["proofs_per_s"]
    result["loads"] = loads
    result["coalescing"] = {"flushes": sum(l.flushes for l in srv.lanes),
                            "calls": sum(l.coalesced_calls for l in srv.lanes)}
    srv.close()
    if rank == 0:
        print(json.dumps(result))


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def run_gb300(args, world, rank, local, pg):
    load_tuning(args, local)
    if args.workload == "sumcheck":
        return run_sumcheck(args, world, rank, local, pg)
    if args.workload == "batch":
        return run_batch(args, world, rank, local, pg)
    if args.workload == "serve":
        return run_serve(args, world, rank, local, pg)
    s = Session(local)
    nv = args.num_vars or 20
    n = 1 << nv
    be = s.be
    layers = s.srs_layers(nv, 0)

    if args.workload == "commit":
        import numpy as np
        from hyperplonk_gb300 import _native
        params = be.prepare_prover_param(nv, layers)
        del layers
        autotune(args, be, params, [nv], [])
        hv = np.empty(32 * n, dtype=np.uint8)
        s.check(s.lib.hp_cuda_v1_fixture_random_fr(0, 0, n, _native.buf(hv)), "fixture_random_fr")
        host = s.pinned(hv)
        hvp = host.numpy()
        mle = be.mle_from_evaluations(nv, hvp)
        value_fn = lambda: be.commit(params, mle)  # noqa: E731

        def e2e_fn():
            m = be.mle_from_evaluations(nv, hvp)
            be.commit(params, m)

        for _ in range(args.warmup):
            value_fn()
            e2e_fn()
        per, per_e2e, nl, clk, acc, msm = measure(s, pg, args.steps, value_fn, e2e_fn)
        units, metric, unit = n, "MSM pts/s", "pts/s"
        acc_work = accumulate_imad(n) * acc[1]
        workload = f"multilinear-KZG commit of one MLE, num_vars={nv} (one 2^{nv}-point G1 MSM)"
        h2d, d2h = 32 * n, 97
        extra = {}
    else:
        from hyperplonk_gb300 import snark
        sel, wit, perm, pub = snark.vanilla_fixture(nv, PROVE_SEED)
        pk = snark.preprocess(be, nv, min(16, n), sel, perm, layers, commit=False)
        del sel, perm
        opening = [nv - 1 - i for i in range(nv)]  # the batch opening's quotient MSMs
        autotune(args, be, pk.pcs_param, [nv] + [k for k in opening if k >= 10], shared_mix(opening))
        pinned = [s.pinned(w) for w in wit]
        wit_host = [p.numpy() for p in pinned]
        resident = [be.mle_from_evaluations(nv, w) for w in wit_host]
        out = {}
        autotune_sumcheck(args, be, lambda view: snark.prove(view, pk, pub, None, witness_mles=resident))

        def value_fn():
            out["proof"] = snark.prove(be, pk, pub, None, witness_mles=resident).to_bytes()

        def e2e_fn():
            out["proof"] = snark.prove(be, pk, pub, wit_host).to_bytes()

        for _ in range(args.warmup):
            value_fn()
            e2e_fn()
        per, per_e2e, nl, clk, _, _ = measure(s, pg, args.steps, value_fn, e2e_fn)
        units, metric, unit = 1, "HyperPlonk proofs/s", "proofs/s"
        workload =(f"full HyperPlonk prove, vanilla-plonk circuit of 2^{nv} gates (q_O = -1, w3 solves the gate, "
                    f"identity permutation over 3 columns, 16 public inputs, seed {PROVE_SEED}), testing SRS nv={nv}")
        h2d, d2h = 3 * 32 * n, len(out["proof"])

        def e2e_pipelined(steps: int) -> float:
            """`steps` proofs, each from its own upload of the witnesses from
            pinned host memory, the upload of proof i+1 queued on the context's
            ingress stream before proof i runs (hp_cuda_v1_mle_upload_async),
            so the copies overlap the proof; the L2 flush between proofs stays
            inside the timed region.  Seconds per proof (CUDA events on the
            backend's stream around the whole loop)."""
            torch = s.torch
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s.stream):
                torch.cuda.synchronize()
                a.record(s.stream)
                nxt = be.mle_upload_async(nv, wit_host)
                for i in range(steps):
                    cur = nxt
                    if i + 1 < steps:
                        nxt = be.mle_upload_async(nv, wit_host)
                    mles = cur.wait()
                    out["proof_pipelined"] = snark.prove(be, pk, pub, None, witness_mles=mles).to_bytes()
                    s.flush_buf.fill_(1)
                b.record(s.stream)
                b.synchronize()
            return a.elapsed_time(b) / 1e3 / steps

        e2e_pipelined(2)  # warm-up
        pipe_s = max_over_ranks(pg, e2e_pipelined(args.steps))
        if out["proof_pipelined"] != out["proof"]:
            raise RuntimeError("the pipelined end-to-end proof differs from the resident one")
        lat = sorted(per)
        extra = {"latency_ms": {"p50": 1e3 * statistics.median(lat),
                                "p99": 1e3 * lat[min(len(lat) - 1, math.ceil(0.99 * len(lat)) - 1)],
                                "min": 1e3 * lat[0], "max": 1e3 * lat[-1]},
                 "proof_bytes": len(out["proof"])}
        # MSM pts/s of a 2^nv commit on the same prepared SRS (witness w1),
        # timed alone: inside a proof the MSMs overlap on worker streams, so
        # the dominant kernel's per-launch time is taken from this loop.
        commit = lambda: be.commit(pk.pcs_param, resident[0])  # noqa: E731
        for _ in range(3):
            commit()
        s.torch.cuda.synchronize()
        s.profile(True)
        cper = s.timed(commit, max(3, args.steps))
        acc = s.profile_read(b"msm_accumulate")
        msm = s.profile_read(b"msm")
        s.profile(False)
        extra["msm"] = {"metric": "MSM pts/s", "value": world * n / max_over_ranks(pg, statistics.mean(cper)),
                        "unit": "pts/s", "points": n, "ms_per_msm": 1e3 * statistics.mean(cper)}
        acc_work = accumulate_imad(n) * acc[1]
        # host wall time per prover phase, mean over a few untimed proofs
        phases = {}
        for _ in range(3):
            snark.prove(be, pk, pub, None, witness_mles=resident, phases=phases)
        extra["phases_ms"] = {k: 1e3 * v / 3 for k, v in phases.items()}
        # the same circuit with copy constraints that are not the identity:
        # frac and prod hold random fractions, so their commitments take the
        # full MSM (the identity permutation's 0/1 tables take the
        # sum-of-bases path); same SRS, witnesses resident
        wsel, wwit, wperm, wpub = snark.vanilla_fixture(nv, PROVE_SEED, wired=True)
        wpk = snark.ProvingKey(nv, min(16, n), snark.VANILLA_GATE, pk.pcs_param,
                               [be.mle_from_evaluations(nv, t) for t in wsel],
                               [be.mle_from_evaluations(nv, t) for t in wperm])
        wres = [be.mle_from_evaluations(nv, t) for t in wwit]
        del wsel, wwit, wperm
        wfn = lambda: snark.prove(be, wpk, wpub, None, witness_mles=wres).to_bytes()  # noqa: E731
        for _ in range(2):
            wfn()
        s.torch.cuda.synchronize()
        wper = s.timed(wfn, max(3, args.steps))
        extra["general_circuit"] = {
            "workload": "the same circuit with non-identity copy constraints (w2[i] = w1[wire(i)], "
                        "hp_cuda_v1_fixture_vanilla_plonk_wired), witnesses resident",
            "proofs_per_s": world / max_over_ranks(pg, statistics.mean(wper)),
            "ms_per_proof": 1e3 * statistics.mean(wper), "p50_ms": 1e3 * statistics.median(wper)}
        del wpk, wres

    step_s = max_over_ranks(pg, statistics.mean(per))
    e2e_s = max_over_ranks(pg, statistics.mean(per_e2e))
    imad, fqm, frm = s.integer_rates()
    acc_ms_total = acc[0]
    achieved = acc_work / (acc_ms_total / 1e3) / 1e12 if acc_ms_total > 0 else 0.0
    peak = imad / 1e12
    traffic = _profile_traffic(nv)
    result = {
        "metric": metric,
        "value": world * units / step_s,
        "unit": unit,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": step_s * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 limbs (Fr 8x32, Fq 12x32 Montgomery)",
        "data": "synthetic: ChaCha20 fixture streams (seed 0 SRS/scalars, seed 2 circuit), device-generated "
                "testing SRS",
        "config": {"workload": workload, "num_vars": nv, "window_bits": window_bits(n),
                   "l2": "256 MiB flush between steps; prepared SRS > L2",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        # prove: a stream of proofs through the C ABI, each from its own
        # witness upload (pinned host memory, ingress overlapping the
        # previous proof); e2e_serial: upload then prove, one at a time
        "e2e": ({"value": world / pipe_s, "unit": unit, "ms_per_step": pipe_s * 1e3, "h2d_bytes_per_step": h2d,
                 "d2h_bytes_per_step": d2h,
                 "how": "witness upload of proof i+1 (hp_cuda_v1_mle_upload_async, ingress stream) overlapping "
                        "proof i; every proof's inputs copied from pinned host memory and its proof bytes read "
                        "back inside the timed loop"}
                if args.workload == "prove" else
                {"value": world * units / e2e_s, "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}),
        **({"e2e_serial": {"value": world * units / e2e_s, "unit": unit, "ms_per_step": e2e_s * 1e3,
                           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                           "how": "each step uploads its witnesses (blocking) and then proves"}}
           if args.workload == "prove" else {}),
        "gpu_launches": int(nl),
        "roofline": {"bound": "imad", "kernel": "k_msm_accumulate", "achieved": achieved, "peak": peak,
                     "unit": "TIMAD/s", "frac": achieved / peak if peak else None, "traffic": traffic,
                     "traffic_source": ("dram__bytes_read.sum + dram__bytes_write.sum of one launch of this "
                                        "kernel at this size from a separate ncu capture of the commit workload "
                                        "(profiles/msm_accumulate_commit.md gives the command); not measured "
                                        "in this run, which no profiler may attach to"
                                        if traffic is not None else "no ncu capture at this size"),
                     "peak_source": "measured live: mad.lo.u32 issue rate on this GPU (libhp_probe)",
                     "launches": acc[1], "per_launch_ms": acc_ms_total / max(1, acc[1]),
                     "algorithmic_imad_per_launch": acc_work / max(1, acc[1])},
        "field_rates": {"fq_mul_per_s": fqm, "fr_mul_per_s": frm, "fq_mul_imad_equiv_tiimad_s": fqm * FQ_MUL_IMAD / 1e12},
        "clocks": clk,
    }
    result.update(extra)
    if TUNING_INFO:
        result["msm_tuning"] = dict(TUNING_INFO)
    # the same kernel against the pipe it actually fills: a Karatsuba Fq
    # product issues 108 + 144 wide multiply-adds, so the live mad.wide rate
    # / 252 caps the product rate before any addition, carry or load
    wide = s.wide_rate()
    if acc_ms_total > 0:
        fq_done = acc_work / FQ_MUL_IMAD / (acc_ms_total / 1e3)
        result["roofline"]["pipe"] = {
            "bound": "mad.wide.u32 issue (32x32->64 multiply-add)", "wide_per_s": wide,
            "wide_per_fq_mul": FQ_MUL_WIDE, "fq_mul_cap_per_s": wide / FQ_MUL_WIDE,
            "achieved_fq_mul_per_s": fq_done, "frac": fq_done / (wide / FQ_MUL_WIDE),
            "source": "measured live (libhp_probe: independent mad.wide.u32 chains)"}
    # the whole 2^nv MSM (sort, accumulation, reduction, host finish) against
    # the fixed accounting of the IMAD work, timed alone by the library hooks
    msm_ms = msm[0] / max(1, msm[1])
    result["msm_total"] = {"ms": msm_ms, "accounting_imad": msm_accounting_imad(n),
                           "frac_of_imad_peak": msm_accounting_imad(n) / (msm_ms / 1e3) / imad if msm_ms else None}
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.workload, nv, layers if args.workload == "prove" else None)
    if rank == 0 and world == 1 and args.workload == "prove" and not args.no_extras and args.num_vars is None:
        s.torch.cuda.synchronize()
        result["other_workloads"] = other_workloads()
    if rank == 0:
        print(json.dumps(result))


def other_workloads() -> dict:
    """The batch plan (64 MSMs + 32 sumchecks) and the serving stream
    (prove requests of 2^16..2^22 gates) measured in the same run, each in a child process of
    this script with its own timed region and clock record; their summaries
    go into the prove line."""
    out = {}
    runs = {"batch": ["--workload", "batch", "--steps", "3", "--warmup", "1"],
            "serve": ["--workload", "serve"]}
    for name, extra in runs.items():
        try:
            r = subprocess.run([sys.executable, str(pathlib.Path(__file__).resolve()), *extra, "--no-cpu-baseline"],
                               capture_output=True, text=True, timeout=1200, cwd=ROOT)
            lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
            if r.returncode != 0 or not lines:
                out[name] = {"error": f"exit {r.returncode}: {r.stderr.strip()[-300:]}"}
                continue
            d = json.loads(lines[-1])
        except (subprocess.TimeoutExpired, ValueError) as e:
            out[name] = {"error": str(e)[:300]}
            continue
        if name == "batch":
            out[name] = {"metric": d["metric"], "value": d["value"], "unit": d["unit"],
                         "ms_per_run": d["ms_per_step"], "plain_ms_per_run": d["plain"]["ms_per_run"],
                         "batched_over_plain": d["plain"]["batched_over_plain"],
                         "msm_points_per_run": d["msm_points_per_run"], "clocks": d["clocks"],
                         "workload": d["config"]["workload"]}
        else:
            out[name] = {"metric": d["metric"], "unit": d["unit"],
                         "plain_capacity_proofs_per_s": d["plain_capacity_proofs_per_s"],
                         "loads": d["loads"], "clocks": d["clocks"], "workload": d["config"]["workload"]}
    return out


def cpu_baseline(workload: str, nv: int, srs_layers=None) -> dict:
    """The oracle on this host's cores, on one step of the same workload at
    the same size (`srs_layers`: the SRS the GPU arm used, as packets, to skip
    regenerating it on the CPU; the oracle's own SRS is byte-identical)."""
    if workload == "commit":
        sample = CpuMsmSample(nv)
        per = statistics.median([sample.step() for _ in range(3)])
        return {"value": (1 << nv) / per, "unit": "pts/s", "cores": sample.threads, "kind": "port",
                "sample": f"oracle Pippenger MSM of 2^{nv} points (the commit at its size), median of 3, "
                          f"{per:.3f} s each"}
    if workload == "sumcheck":
        sample = CpuSumcheckSample(nv)
        per = statistics.median([sample.step() for _ in range(3)])
        return {"value": 1.0 / per, "unit": "proofs/s", "cores": sample.threads, "kind": "port",
                "sample": f"oracle sumcheck prove of the same instance at 2^{nv}, median of 3 = {per:.2f} s"}
    orc = _oracle()
    layers = None if srs_layers is None else [orc.packets_to_affine(l) for l in srs_layers]
    sample = CpuProveSample(nv, layers)
    per = sample.step()
    return {"value": 1.0 / per, "unit": "proofs/s", "cores": sample.threads, "kind": "port",
            "sample": f"one oracle proof of the same circuit at 2^{nv} gates ({per:.2f} s): oracle/prover.py over "
                      f"the oracle's C backend, Python transcript"}


def _profile_traffic(nv: int):
    """DRAM bytes (read + write) of one k_msm_accumulate launch of a 2^nv
    commit, from the committed ncu summary of that kernel at that size
    (profiles/msm_accumulate_commit.md, line 'traffic_bytes_per_launch
    nv=<k>: <bytes>'); None when no capture at this size exists."""
    p = ROOT / "profiles" / "msm_accumulate_commit.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(f"traffic_bytes_per_launch nv={nv}:"):
            try:
                return float(line.split(":")[1].strip().split()[0])
            except (IndexError, ValueError):
                return None
    return None


def run_reference(args, world, rank):
    """The reference arm: the oracle (the C restatement of the reference's
    CPU backend with the oracle's own prover driver and transcript; the
    reference's Rust/arkworks path cannot be built here) on every host core,
    one full step of the workload at its stated size per step, fixtures and
    SRS from the oracle's own generators.  Imports nothing of the product."""
    if rank != 0:
        return
    nv = args.num_vars or (22 if args.workload == "batch" else 16 if args.workload == "commit" else 20)
    t_setup = time.perf_counter()
    if args.workload == "batch":
        sample, units, metric, unit = CpuBatchSample(nv), 1, "batch-plan runs/s", "runs/s"
        desc = f"the whole batch plan (seed 3, SRS nv={nv}) on the oracle per step"
    elif args.workload == "commit":
        sample, units, metric, unit = CpuMsmSample(nv), 1 << nv, "MSM pts/s", "pts/s"
        desc = f"oracle Pippenger MSM of 2^{nv} points (one commit) per step"
    elif args.workload == "sumcheck":
        sample, units, metric, unit = CpuSumcheckSample(nv), 1, "sumcheck proofs/s", "proofs/s"
        desc = f"oracle sumcheck prove of the degree-2 instance at 2^{nv} per step"
    else:
        sample, units, metric, unit = CpuProveSample(nv), 1, "HyperPlonk proofs/s", "proofs/s"
        desc = f"one oracle proof of the vanilla-plonk circuit (seed 2) at 2^{nv} gates per step"
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        sample.step()
    per = [sample.step() for _ in range(args.steps)]
    step = sum(per) / len(per)
    v = units / step
    print(json.dumps({
        "impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 limbs (Montgomery)",
        "data": "synthetic: ChaCha20 fixture streams, oracle testing SRS",
        "config": {"workload": f"{args.workload}, num_vars={nv}, full size", "num_vars": nv},
        "latency_ms": {"p50": 1e3 * statistics.median(per), "min": 1e3 * min(per), "max": 1e3 * max(per)},
        "setup_s": round(setup_s, 2),
        "product_code_loaded": sorted(m for m in sys.modules if m.startswith("hyperplonk_gb300")),
        "cpu_baseline": {"value": v, "unit": unit, "cores": sample.threads, "kind": "port",
                         "sample": desc + " (the reference's Rust/arkworks CPU path cannot be built here: no cargo, "
                                          "arkworks not vendored)"},
        "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


class CpuBatchSample:
    """The batch plan on the oracle: every MSM over its prefix of layer 0 of
    the oracle's SRS of nv_srs variables and every sumcheck prove, one after
    another (the oracle parallelises inside each)."""

    def __init__(self, nv_srs: int):
        orc = _oracle()
        import prover as oprover
        self.orc, self.op = orc, oprover
        self.threads = orc.set_threads(0)
        self.layer0 = orc.srs_layers(nv_srs, 0)[0]
        self.ks, self.nvs = oprover.batch_plan(3, msm_k=(12, nv_srs), sumcheck_nv=(14, nv_srs))
        self.scalars = oprover.batch_msm_scalars(self.ks, 3)
        self.instances = [oprover.sumcheck_instance(v, 103 + i) for i, v in enumerate(self.nvs)]

    def step(self) -> float:
        t0 = time.perf_counter()
        for k, sc in zip(self.ks, self.scalars):
            self.orc.msm(self.layer0[:96 << k], sc)
        for i, (v, inst) in enumerate(zip(self.nvs, self.instances)):
            self.op.sumcheck_prove_instance(v, 103 + i, inst)
        return time.perf_counter() - t0


def relaunch(n: int) -> int:
    """`--gpus N` without a launcher: run this command as N local ranks
    (torch.distributed.run on 127.0.0.1, one process per GPU) and return the
    launcher's exit status."""
    import socket
    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(pathlib.Path(__file__).resolve()),
           *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    args = parse()
    launched = os.environ.get("WORLD_SIZE")
    if launched is None and args.gpus > 1:
        sys.exit(relaunch(args.gpus))
    if launched is not None and int(launched) != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} under a launcher of WORLD_SIZE {launched}")
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gb300(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
