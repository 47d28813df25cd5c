#!/usr/bin/env python3
"""Benchmark of the GB300 HyperPlonk prover hot path: multilinear-KZG commit.

Workload (one step): commit one MLE of 2^nv uniform Fr (fixture stream seed 0)
against the prepared testing SRS of nv variables (fixture stream seed 0,
generated on the device) -- i.e. one 2^nv-point G1 MSM through the
reference-facing C ABI (hp_cuda_v1_multilinear_kzg_commit).  Default nv = 20,
the 2^20-point MSM of the reference's published MSM numbers; --num-vars 16 is
the configuration-1 size.  Metric: MSM pts/s (points per second).

  value : commit through the C ABI with the MLE already resident in HBM;
  e2e   : the same through the C ABI from a pinned host buffer each step
          (mle_upload H2D + commit + 97-byte result + retire).

Timing: W warm-up steps, then K steps each bracketed by CUDA events on the
backend's own stream (hp_cuda_v1_context_stream), a barrier and
torch.cuda.synchronize() on both sides of the timed loop; between steps a
256 MiB buffer is written to flush L2 (the MSM's precomputed base table,
~1.3 GB at nv=20, is larger than L2 anyway).  The dominant kernel
(msm_accumulate) is timed by the library's own event hooks on the same
stream.  --impl reference times the CPU restatement of the reference's CPU
path (oracle, all host threads) on a bounded sample of the workload.
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--num-vars", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def msm_accounting_imad(n: int) -> float:
    """Fixed algorithmic work of an n-point MSM: min_c ceil(255/c)(10n + 14*2^c)
    Fq multiplications at 588 IMAD each."""
    best = min(math.ceil(255 / c) * (10 * n + 14 * (1 << c)) for c in range(8, 21))
    return best * FQ_MUL_IMAD


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
# CPU baseline (oracle restatement of the reference CPU path)
# ---------------------------------------------------------------------------

class CpuMsmSample:
    """The oracle's multithreaded Pippenger MSM (the CPU restatement of ark-ec
    msm_unchecked as used by backend/src/cpu/multilinear_kzg.rs:40-59) on a
    2^log_n-point sample of the workload (testing SRS and fixture scalars,
    seed 0), prepared once."""

    def __init__(self, log_n: int = 16):
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as orc
        self.orc = orc
        self.log_n = log_n
        self.threads = orc.set_threads(0)
        self.bases = orc.srs_layers(log_n, 0)[0]
        self.scalars = orc.random_fr(0, 1 << log_n)

    def step(self) -> float:
        t0 = time.perf_counter()
        self.orc.msm(self.bases, self.scalars)
        return time.perf_counter() - t0


def cpu_msm_sample(steps: int, log_n: int = 16):
    """(pts/s, threads, median seconds per MSM) over `steps` timed MSMs."""
    s = CpuMsmSample(log_n)
    per = statistics.median([s.step() for _ in range(steps)])
    return (1 << log_n) / per, s.threads, per


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------

def run_gb300(args, world, rank, local, pg):
    import numpy as np
    import torch
    from hyperplonk_gb300 import _native
    from hyperplonk_gb300.backend import CudaBackend, CudaMle
    from hyperplonk_gb300.errors import check_status

    torch.cuda.set_device(local)
    nv = args.num_vars
    n = 1 << nv
    be = CudaBackend(local)
    lib = be.lib
    stream = torch.cuda.ExternalStream(be.ctx.stream(), device=torch.device("cuda", local))

    # SRS (device-generated testing SRS, seed 0) -> prepared params
    total = (1 << (nv + 1)) - 1
    packets = np.empty(total * 97, dtype=np.uint8)
    check_status(lib.hp_cuda_v1_srs_generate(be.ctx.raw, nv, 0, _native.buf(packets), total), "srs_generate")
    layers, off = [], 0
    for i in range(nv + 1):
        cnt = 1 << (nv - i) if i < nv else 1
        layers.append(packets[97 * off:97 * (off + cnt)])
        off += cnt
    params = be.prepare_prover_param(nv, layers)
    del packets, layers

    # scalars: fixture stream seed 0, in pinned host memory
    host = torch.empty(32 * n, dtype=torch.uint8, pin_memory=True)
    hv = host.numpy()
    check_status(lib.hp_cuda_v1_fixture_random_fr(0, 0, n, _native.buf(hv)), "fixture_random_fr")
    mle = be.mle_from_evaluations(nv, hv)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def launches() -> int:
        c = ctypes.c_uint64()
        check_status(lib.hp_cuda_v1_kernel_launch_count(ctypes.byref(c)), "kernel_launch_count")
        return c.value

    def timed(fn, steps):
        per = []
        with torch.cuda.stream(stream):
            for _ in range(steps):
                flush.fill_(1)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                b.synchronize()
                per.append(a.elapsed_time(b) / 1e3)
        return per

    commit_once = lambda: be.commit(params, mle)  # noqa: E731

    def e2e_once():
        m = be.mle_from_evaluations(nv, hv)
        be.commit(params, m)
        del m

    for _ in range(args.warmup):
        commit_once()
        e2e_once()

    # ---- value: device-resident input ----
    check_status(lib.hp_cuda_v1_context_profile(be.ctx.raw, 1), "context_profile")
    clocks = ClockSampler(local)
    barrier(pg)
    torch.cuda.synchronize()
    clocks.start()
    l0 = launches()
    t0 = time.perf_counter()
    per = timed(commit_once, args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    l1 = launches()
    barrier(pg)
    clk = clocks.stop()
    step_s = max_over_ranks(pg, sum(per) / len(per))
    ms = ctypes.c_double()
    cnt = ctypes.c_uint64()
    check_status(lib.hp_cuda_v1_context_profile_read(be.ctx.raw, b"msm_accumulate", ctypes.byref(ms),
                                                     ctypes.byref(cnt)), "profile_read")
    acc_ms = ms.value / max(1, cnt.value)
    check_status(lib.hp_cuda_v1_context_profile_read(be.ctx.raw, b"msm", ctypes.byref(ms), ctypes.byref(cnt)),
                 "profile_read")
    msm_ms = ms.value / max(1, cnt.value)
    check_status(lib.hp_cuda_v1_context_profile(be.ctx.raw, 0), "context_profile")

    # ---- e2e: host buffer in, result out, every step ----
    barrier(pg)
    torch.cuda.synchronize()
    per_e2e = timed(e2e_once, args.steps)
    torch.cuda.synchronize()
    barrier(pg)
    e2e_s = max_over_ranks(pg, sum(per_e2e) / len(per_e2e))

    # ---- integer-pipe ceilings on this GPU ----
    probe = ctypes.CDLL(str(ROOT / "hyperplonk_gb300" / "_build" / "libhp_probe.so"))
    probe.hp_probe_integer_rates.argtypes = [ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 3
    imad, fqm, frm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    rc = probe.hp_probe_integer_rates(local, ctypes.byref(imad), ctypes.byref(fqm), ctypes.byref(frm))
    if rc != 0:
        raise RuntimeError(f"integer probe failed ({rc})")

    # dominant kernel roofline: W*n point-window records x one XYZZ mixed add
    # (10 Fq muls) each
    c_bits = next(c for c in range(4, 21) if c == _window_bits(n))
    windows = math.ceil(256 / c_bits)
    acc_imad = windows * n * 10 * FQ_MUL_IMAD
    achieved = acc_imad / (acc_ms / 1e3) / 1e12
    peak = imad.value / 1e12
    traffic = _profile_traffic(nv)

    result = {
        "metric": "MSM pts/s",
        "value": world * n / step_s,
        "unit": "pts/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": step_s * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 limbs (Fr 8x32, Fq 12x32 Montgomery)",
        "data": "synthetic: ChaCha20 fixture stream seed 0, device-generated testing SRS (seed 0)",
        "config": {"workload": f"multilinear-KZG commit of one MLE, num_vars={nv} (one 2^{nv}-point G1 MSM)",
                   "num_vars": nv, "points": n, "window_bits": c_bits, "windows": windows,
                   "l2": "256 MiB flush between steps; base table > L2",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "e2e": {"value": world * n / e2e_s, "unit": "pts/s", "h2d_bytes_per_step": 32 * n,
                "d2h_bytes_per_step": 97},
        "gpu_launches": int(l1 - l0),
        "roofline": {"bound": "imad", "kernel": "k_msm_accumulate", "achieved": achieved, "peak": peak,
                     "unit": "TIMAD/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "measured live: mad.lo.u32 issue rate on this GPU (libhp_probe)",
                     "per_launch_ms": acc_ms, "algorithmic_imad_per_launch": acc_imad},
        "msm_total": {"ms": msm_ms, "accounting_imad": msm_accounting_imad(n),
                      "achieved_tiimad_s": msm_accounting_imad(n) / (msm_ms / 1e3) / 1e12,
                      "frac_of_imad_peak": msm_accounting_imad(n) / (msm_ms / 1e3) / imad.value},
        "field_rates": {"fq_mul_per_s": fqm.value, "fr_mul_per_s": frm.value,
                        "fq_mul_imad_equiv_tiimad_s": fqm.value * FQ_MUL_IMAD / 1e12},
        "clocks": clk,
        "wall_s_timed_loop": wall,
    }
    if rank == 0 and not args.no_cpu_baseline:
        v, threads, per_s = cpu_msm_sample(3)
        result["cpu_baseline"] = {"value": v, "unit": "pts/s", "cores": threads, "kind": "port",
                                  "sample": f"oracle Pippenger MSM of 2^16 points (testing SRS nv=16, "
                                            f"fixture seed 0), median of 3, {per_s:.3f} s each"}
    if rank == 0:
        print(json.dumps(result))


def _window_bits(n: int) -> int:
    best, best_cost = 4, float("inf")
    for c in range(4, 21):
        cost = math.ceil(256 / c) * 10.0 * n + 28.0 * (1 << (c - 1))
        if cost < best_cost:
            best, best_cost = c, cost
    return best


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
    sample = CpuMsmSample(16)
    for _ in range(args.warmup):
        sample.step()
    per = [sample.step() for _ in range(args.steps)]
    step = sum(per) / len(per)
    v = (1 << 16) / step
    print(json.dumps({
        "impl": "reference", "metric": "MSM pts/s", "value": v, "unit": "pts/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 limbs (Montgomery)",
        "data": "synthetic: ChaCha20 fixture stream seed 0, oracle testing SRS nv=16",
        "config": {"workload": f"multilinear-KZG commit, num_vars={args.num_vars}: bounded sample of 2^16 points "
                               "per step", "num_vars": args.num_vars},
        "cpu_baseline": {"value": v, "unit": "pts/s", "cores": sample.threads, "kind": "port",
                         "sample": "oracle Pippenger MSM of 2^16 points per step (the reference's Rust/arkworks "
                                   "CPU path cannot be built here: no cargo, arkworks not vendored)"},
        "e2e": {"value": v, "unit": "pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
