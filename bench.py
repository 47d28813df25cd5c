#!/usr/bin/env python3
"""Benchmark of the GB300 HyperPlonk prover hot path.

Workloads (--workload):

  prove  (default) -- full HyperPlonk prove of the vanilla-plonk circuit of
         2^nv gates (configuration 3: q_L, q_R, q_M, q_C, w1, w2 uniform, q_O
         = -1, w3 solving the gate, identity permutation over 3 columns, 16
         public inputs, fixture seed 2, testing SRS of nv variables).  One step
         = one proof through the reference-facing C ABI (witness commits,
         gate zero-check, permutation check, 22 evaluations, batch opening),
         proof serialized to bytes.  Metric: HyperPlonk proofs/s, with p50/p99
         proof latency.  The MSM pts/s of a 2^nv commit on the same SRS is
         reported beside it ("msm").
  commit -- one multilinear-KZG commit of a 2^nv-point MLE (configuration 1
         shape; nv = 16 is configuration 1 itself).  Metric: MSM pts/s.

  value : inputs already resident in HBM (witness MLEs uploaded before the
          timed loop);
  e2e   : the same through the C ABI from pinned host buffers every step
          (mle_upload of the inputs + the work + results back on the host).

Timing: W warm-up steps, then K steps each bracketed by CUDA events on the
backend's own stream (hp_cuda_v1_context_stream), a barrier and
torch.cuda.synchronize() on both sides of the timed loop; a 256 MiB buffer is
written between steps to flush L2 (the prepared SRS, ~2.6 GB at nv=20, is
larger than L2 anyway).  The dominant kernel (k_msm_accumulate) is timed by
the library's own CUDA-event hooks on the same stream.  --impl reference
times the CPU restatement of the reference's CPU path (oracle, all host
threads) on a bounded sample of the workload.
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
PROVE_SEED = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["prove", "commit"], default="prove")
    ap.add_argument("--num-vars", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def window_bits(n: int) -> int:
    """Window width the library picks for an n-point layer (msm.cu)."""
    env = os.environ.get("HP_MSM_WINDOW_BITS")
    if env and 4 <= int(env) <= 22:
        return int(env)
    best, best_cost = 4, float("inf")
    for c in range(4, 21):
        top_bits = 255 - c * (math.ceil(256 / c) - 1)
        top_buckets = float(1 << (top_bits - 1)) if top_bits >= 2 else 1.0
        if c > 4 and n / top_buckets > 2048.0:
            continue
        cost = math.ceil(256 / c) * 10.0 * n + 28.0 * (1 << (c - 1))
        if cost < best_cost:
            best, best_cost = c, cost
    return best


def accumulate_imad(n: int) -> int:
    """Algorithmic work of k_msm_accumulate for one n-point MSM: one XYZZ
    mixed addition (10 Fq muls) per (point, window) record."""
    return math.ceil(256 / window_bits(n)) * n * 10 * FQ_MUL_IMAD


def msm_accounting_imad(n: int) -> float:
    """Fixed algorithmic work of an n-point MSM: min_c ceil(255/c)(10n + 14*2^c)
    Fq multiplications at 588 IMAD each."""
    best = min(math.ceil(255 / c) * (10 * n + 14 * (1 << c)) for c in range(8, 21))
    return best * FQ_MUL_IMAD


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
    msm_unchecked as used by backend/src/cpu/multilinear_kzg.rs:40-59) on a
    2^log_n-point sample (testing SRS and fixture scalars, seed 0)."""

    def __init__(self, log_n: int = 16):
        orc = _oracle()
        self.orc, self.log_n = orc, log_n
        self.threads = orc.set_threads(0)
        self.bases = orc.srs_layers(log_n, 0)[0]
        self.scalars = orc.random_fr(0, 1 << log_n)

    def step(self) -> float:
        t0 = time.perf_counter()
        self.orc.msm(self.bases, self.scalars)
        return time.perf_counter() - t0


class CpuProveSample:
    """The oracle prover: the same driver over the oracle's CpuBackend
    (backend/src/cpu restated, multithreaded MSM) and the oracle's Python
    transcript, on the configuration-3 circuit at 2^nv gates."""

    def __init__(self, nv: int):
        from hyperplonk_gb300 import snark
        orc = _oracle()
        import transcript_ref as tref  # oracle/transcript_ref.py (path set by _oracle)
        self.snark, self.tcls = snark, tref.OracleIOPTranscript
        self.threads = orc.set_threads(0)
        self.cpu = orc.CpuBackend()
        self.nv = nv
        sel, self.wit, perm, self.pub = snark.vanilla_fixture(nv, PROVE_SEED)
        self.pk = snark.preprocess(self.cpu, nv, min(16, 1 << nv), sel, perm, orc.srs_layers(nv, 0))

    def step(self) -> float:
        t0 = time.perf_counter()
        self.snark.prove(self.cpu, self.pk, self.pub, self.wit, transcript_cls=self.tcls).to_bytes()
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

    def integer_rates(self):
        probe = ctypes.CDLL(str(ROOT / "hyperplonk_gb300" / "_build" / "libhp_probe.so"))
        probe.hp_probe_integer_rates.argtypes = [ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 3
        imad, fqm, frm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rc = probe.hp_probe_integer_rates(self.local, ctypes.byref(imad), ctypes.byref(fqm), ctypes.byref(frm))
        if rc != 0:
            raise RuntimeError(f"integer probe failed ({rc})")
        return imad.value, fqm.value, frm.value


def measure(s: Session, pg, steps: int, value_fn, e2e_fn):
    """Timed loops; returns (value step seconds list, e2e list, launches, clocks, accumulate ms/launches)."""
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
    s.profile(False)
    barrier(pg)
    s.torch.cuda.synchronize()
    per_e2e = s.timed(e2e_fn, steps)
    s.torch.cuda.synchronize()
    barrier(pg)
    return per, per_e2e, l1 - l0, clk, acc, msm


def run_gb300(args, world, rank, local, pg):
    s = Session(local)
    nv = args.num_vars
    n = 1 << nv
    be = s.be
    layers = s.srs_layers(nv, 0)

    if args.workload == "commit":
        import numpy as np
        from hyperplonk_gb300 import _native
        params = be.prepare_prover_param(nv, layers)
        del layers
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
        pk = snark.preprocess(be, nv, min(16, n), sel, perm, layers)
        del layers, sel, perm
        pinned = [s.pinned(w) for w in wit]
        wit_host = [p.numpy() for p in pinned]
        resident = [be.mle_from_evaluations(nv, w) for w in wit_host]
        out = {}

        def value_fn():
            out["proof"] = snark.prove(be, pk, pub, None, witness_mles=resident).to_bytes()

        def e2e_fn():
            out["proof"] = snark.prove(be, pk, pub, wit_host).to_bytes()

        for _ in range(args.warmup):
            value_fn()
            e2e_fn()
        per, per_e2e, nl, clk, acc, msm = measure(s, pg, args.steps, value_fn, e2e_fn)
        units, metric, unit = 1, "HyperPlonk proofs/s", "proofs/s"
        acc_work = sum(accumulate_imad(m) for m in prove_msm_sizes(nv)) * args.steps
        workload = (f"full HyperPlonk prove, vanilla-plonk circuit of 2^{nv} gates (q_O = -1, w3 solves the gate, "
                    f"identity permutation over 3 columns, 16 public inputs, seed {PROVE_SEED}), testing SRS nv={nv}")
        h2d, d2h = 3 * 32 * n, len(out["proof"])
        lat = sorted(per)
        extra = {"latency_ms": {"p50": 1e3 * statistics.median(lat),
                                "p99": 1e3 * lat[min(len(lat) - 1, math.ceil(0.99 * len(lat)) - 1)],
                                "min": 1e3 * lat[0], "max": 1e3 * lat[-1]},
                 "proof_bytes": len(out["proof"])}
        # MSM pts/s of a 2^nv commit on the same prepared SRS (witness w1)
        commit = lambda: be.commit(pk.pcs_param, resident[0])  # noqa: E731
        commit()
        cper = s.timed(commit, max(3, args.steps // 2))
        extra["msm"] = {"metric": "MSM pts/s", "value": world * n / max_over_ranks(pg, statistics.mean(cper)),
                        "unit": "pts/s", "points": n, "ms_per_msm": 1e3 * statistics.mean(cper)}

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
        "e2e": {"value": world * units / e2e_s, "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(nl),
        "roofline": {"bound": "imad", "kernel": "k_msm_accumulate", "achieved": achieved, "peak": peak,
                     "unit": "TIMAD/s", "frac": achieved / peak if peak else None, "traffic": traffic,
                     "peak_source": "measured live: mad.lo.u32 issue rate on this GPU (libhp_probe)",
                     "launches": acc[1], "per_launch_ms": acc_ms_total / max(1, acc[1]),
                     "algorithmic_imad_per_launch": acc_work / max(1, acc[1])},
        "msm_phase": {"ms_per_step": msm[0] / max(1, args.steps), "msm_launches": msm[1],
                      "share_of_step": (msm[0] / max(1, args.steps)) / (step_s * 1e3)},
        "field_rates": {"fq_mul_per_s": fqm, "fr_mul_per_s": frm, "fq_mul_imad_equiv_tiimad_s": fqm * FQ_MUL_IMAD / 1e12},
        "clocks": clk,
    }
    result.update(extra)
    if args.workload == "commit":
        result["msm_total"] = {"ms": msm[0] / max(1, msm[1]), "accounting_imad": msm_accounting_imad(n),
                               "frac_of_imad_peak": msm_accounting_imad(n) / (msm[0] / max(1, msm[1]) / 1e3) / imad}
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.workload, nv)
    if rank == 0:
        print(json.dumps(result))


def cpu_baseline(workload: str, nv: int) -> dict:
    if workload == "commit":
        sample = CpuMsmSample(16)
        per = statistics.median([sample.step() for _ in range(3)])
        return {"value": (1 << 16) / per, "unit": "pts/s", "cores": sample.threads, "kind": "port",
                "sample": f"oracle Pippenger MSM of 2^16 points (testing SRS nv=16, fixture seed 0), median of 3, "
                          f"{per:.3f} s each"}
    snv = min(nv, 16)  # oracle prove time is linear in gates from 2^16 up (2.9 s at 16, 11.4 s at 18)
    sample = CpuProveSample(snv)
    per = statistics.median([sample.step() for _ in range(2)])
    scale = 1 << (nv - snv)
    return {"value": 1.0 / (per * scale), "unit": "proofs/s", "cores": sample.threads, "kind": "port",
            "sample": f"oracle prover (CPU backend restatement + Python transcript) on the same circuit at 2^{snv} "
                      f"gates, median of 2 = {per:.2f} s, scaled linearly by {scale} to 2^{nv} gates"}


def _profile_traffic(nv: int):
    """DRAM bytes per k_msm_accumulate launch from the committed ncu summary
    (profiles/msm_accumulate.md, line 'traffic_bytes_per_launch nv=<k>: <bytes>'),
    scaled by the point count when captured at a smaller size; None if absent."""
    p = ROOT / "profiles" / "msm_accumulate.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch"):
            try:
                k = int(line.split("nv=")[1].split(":")[0])
                b = float(line.split(":")[1].strip().split()[0])
                return b * (1 << nv) / (1 << k)
            except (IndexError, ValueError):
                return None
    return None


def run_reference(args, world, rank):
    if rank != 0:
        return
    nv = args.num_vars
    if args.workload == "commit":
        sample, units, metric, unit, snv = CpuMsmSample(16), 1 << 16, "MSM pts/s", "pts/s", 16
        desc = "oracle Pippenger MSM of 2^16 points per step"
        scale = 1
    else:
        snv = min(nv, 16)  # oracle prove time is linear in gates from 2^16 up (2.9 s at 16, 11.4 s at 18)
        sample, units, metric, unit = CpuProveSample(snv), 1, "HyperPlonk proofs/s", "proofs/s"
        scale = 1 << (nv - snv)
        desc = (f"oracle prover on the configuration-3 circuit at 2^{snv} gates per step, throughput scaled "
                f"linearly by {scale} to 2^{nv} gates")
    for _ in range(args.warmup):
        sample.step()
    per = [sample.step() for _ in range(args.steps)]
    step = sum(per) / len(per) * scale
    v = units / step
    print(json.dumps({
        "impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 limbs (Montgomery)",
        "data": "synthetic: ChaCha20 fixture streams, oracle testing SRS",
        "config": {"workload": f"{args.workload}, num_vars={nv}: bounded CPU sample (2^{snv})", "num_vars": nv},
        "cpu_baseline": {"value": v, "unit": unit, "cores": sample.threads, "kind": "port",
                         "sample": desc + " (the reference's Rust/arkworks CPU path cannot be built here: no cargo, "
                                          "arkworks not vendored)"},
        "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    args = parse()
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gb300(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
