"""MSM autotuner: the Python face of hp_cuda_v1_msm_autotune and the tuning
table entries of include/hp_cuda.h (csrc/tune.cu).

The MSM's window width c, reduction segment length and accumulation chunk
length come from a process-wide table of measured entries, else from the size
rules in csrc/msm.cu.  `autotune` measures them on the device (an MSM alone,
keyed by ceil(log2 points), or one launch shared by a mix of MSMs, keyed by
ceil(log2 records)); `save` / `load` keep the table in a text file, and the
file named by HP_CUDA_MSM_TUNING is merged at the first lookup.  A tuned
geometry never changes a result: the tuner checks every candidate's point
against the size rule's.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Optional, Sequence

from . import _native
from .errors import check_status

ALONE = 0
SHARED = 1


@dataclasses.dataclass(frozen=True)
class Tuning:
    size: int          # points (ALONE) or records of the shared launch (SHARED)
    mode: int
    window_bits: int   # ALONE only
    segment: int       # ALONE only
    chunk: int
    model_ms: float    # median device time with the size rule's geometry
    tuned_ms: float    # median device time with the chosen geometry

    @property
    def speedup(self) -> float:
        return self.model_ms / self.tuned_ms if self.tuned_ms > 0 else 1.0


def autotune(backend, prover_param, num_vars: Sequence[int], mode: int = ALONE) -> list[Tuning]:
    """Measure MSMs of 2^nv points (nv in num_vars) over the first bases of
    layer 0 of `prover_param` and record the fastest geometry.  ALONE: one
    entry per size, and prover_param's layers are re-prepared with it.
    SHARED: one entry for a launch shared by all the sizes (at most 64)."""
    lib = _native.load()
    count = len(num_vars)
    if count == 0:
        return []
    nvs = (ctypes.c_size_t * count)(*num_vars)
    out = (_native.MsmTuning * (count if mode == ALONE else 1))()
    check_status(lib.hp_cuda_v1_msm_autotune(backend.ctx.raw, prover_param.raw, nvs, count, mode, out),
                 "msm_autotune")
    return [Tuning(int(t.size), int(t.mode), int(t.window_bits), int(t.segment), int(t.chunk),
                   float(t.model_ms), float(t.tuned_ms)) for t in out]


def query(mode: int, size: int) -> tuple[int, int, int]:
    """(window bits, segment, chunk) a new layer of `size` points (ALONE) or
    (0, 0, chunk) a shared launch of `size` records (SHARED) would use now."""
    lib = _native.load()
    out = (ctypes.c_uint32 * 3)()
    check_status(lib.hp_cuda_v1_msm_tuning_query(mode, size, out), "msm_tuning_query")
    return int(out[0]), int(out[1]), int(out[2])


def save(path: str | os.PathLike) -> None:
    check_status(_native.load().hp_cuda_v1_msm_tuning_save(os.fsencode(path)), "msm_tuning_save")


def load(path: str | os.PathLike, device: Optional[str] = None) -> None:
    """Merge a saved table; with `device`, refuse one measured on another device."""
    dev = device.encode() if device is not None else None
    check_status(_native.load().hp_cuda_v1_msm_tuning_load(os.fsencode(path), dev), "msm_tuning_load")


def clear() -> None:
    check_status(_native.load().hp_cuda_v1_msm_tuning_clear(), "msm_tuning_clear")


def proof_opening_mix(num_vars: int) -> list[int]:
    """num_vars of the MSMs a HyperPlonk proof of 2^num_vars gates runs in
    one shared launch: the batch opening's quotient MSMs (2^(nv-1) .. 1
    points) below 2^22 (window, point) records (csrc/msm.cu msm_runs_alone)."""
    out = []
    for k in (num_vars - 1 - i for i in range(num_vars)):
        c = query(ALONE, 1 << k)[0]
        if -(-256 // c) * (1 << k) < 1 << 22:
            out.append(k)
    return out


def _parse_range(text: str) -> list[int]:
    if ":" in text:
        lo, hi = text.split(":")
        return list(range(int(lo), int(hi) + 1))
    return [int(x) for x in text.split(",") if x]


def main(argv=None) -> None:
    """Measure a tuning table on this device and write it to a file:

        python -m hyperplonk_gb300.tuning --srs-num-vars 22 --alone 4:22 \\
            --shared proof:20 --shared 12,13,14 --out msm_tuning.txt

    --alone lo:hi (or a comma list) tunes single MSMs of 2^k points;
    each --shared mix (a comma list of num_vars, or proof:NV for the opening
    mix of a 2^NV-gate proof) tunes one shared launch.  The testing SRS of
    --srs-num-vars (seed 0) is generated on the device."""
    import argparse
    import json
    ap = argparse.ArgumentParser(prog="python -m hyperplonk_gb300.tuning")
    ap.add_argument("--srs-num-vars", type=int, default=22)
    ap.add_argument("--alone", default="4:22")
    ap.add_argument("--shared", action="append", default=[])
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--out", required=True)
    args = ap.parse_args(argv)
    from .backend import CudaBackend
    be = CudaBackend(args.device)
    nv = args.srs_num_vars
    params = be.prepare_prover_param(nv, be.generate_srs(nv, 0))
    alone = [k for k in _parse_range(args.alone) if k <= nv]
    for e in autotune(be, params, alone):
        print(json.dumps(dataclasses.asdict(e) | {"speedup": round(e.speedup, 4)}), flush=True)
    for mix in args.shared:
        nvs = proof_opening_mix(int(mix.split(":")[1])) if mix.startswith("proof:") else _parse_range(mix)
        nvs = [k for k in nvs if k <= nv][:64]
        if nvs:
            for e in autotune(be, params, nvs, mode=SHARED):
                print(json.dumps(dataclasses.asdict(e) | {"mix": mix, "speedup": round(e.speedup, 4)}), flush=True)
    save(args.out)


if __name__ == "__main__":
    main()
