"""Autotuners: the Python face of hp_cuda_v1_msm_autotune,
hp_cuda_v1_sumcheck_autotune and the tuning table entries of
include/hp_cuda.h (csrc/tune.cu, csrc/sumcheck.cu).

Sumcheck rounds: every round can run on several kernel families, each with
its own grid; `autotune_sumcheck` measures them for the rounds of one
virtual polynomial's shape (keyed by ceil(log2 pairs), the largest product
arity and the slot count) and records the fastest in the same table (saved
and loaded with the MSM entries).  A route never changes a round message:
the tuner compares every candidate's message with the built-in rule's.


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


ROUTE_KERNELS = {1: "one block", 2: "pair per thread", 3: "(slot, pair)", 4: "(slot, pair), fused fold",
                 5: "(product, pair)", 6: "(product, pair), fused fold", 7: "bulk-copied tiles", 8: "(node, pair) without the eq factor"}


@dataclasses.dataclass(frozen=True)
class RoundTuning:
    pairs: int
    kernel: int
    blocks_per_sm: int
    default_kernel: int
    default_blocks_per_sm: int
    default_us: float   # median device time of the built-in rule's route
    tuned_us: float     # median device time of the chosen route


def autotune_sumcheck(backend, polynomial) -> list[RoundTuning]:
    """Measure the round routes of `polynomial`'s shape on a throwaway prover
    state (the polynomial's MLEs are read, never changed) and record the
    fastest route of every round size in the tuning table."""
    lib = _native.load()
    state = backend.prover_init(polynomial)
    nv = polynomial.aux_info.num_variables
    out = (_native.RoundTuning * max(1, nv))()
    count = ctypes.c_size_t()
    check_status(lib.hp_cuda_v1_sumcheck_autotune(backend.ctx.raw, state.raw, out, nv, ctypes.byref(count)),
                 "sumcheck_autotune")
    return [RoundTuning(int(t.pairs), int(t.kernel), int(t.blocks_per_sm), int(t.default_kernel),
                        int(t.default_blocks_per_sm), float(t.default_us), float(t.tuned_us))
            for t in out[:count.value]]


class SumcheckTuningBackend:
    """A backend view that tunes the round routes of every new sumcheck shape
    it sees (autotune_sumcheck on a throwaway state) before the prover state
    is created; everything else goes to `backend` unchanged.  Running one
    proof through it tunes all of the proof's sumcheck shapes."""

    def __init__(self, backend):
        self._backend = backend
        self.tuned: dict = {}

    def __getattr__(self, name):
        return getattr(self._backend, name)

    def prover_init(self, polynomial):
        key = (polynomial.aux_info.num_variables,
               max(len(ix) for _, ix in polynomial.products) if polynomial.products else 0,
               sum(len(ix) + 1 for _, ix in polynomial.products))
        if polynomial.products and key not in self.tuned:
            self.tuned[key] = autotune_sumcheck(self._backend, polynomial)
        return self._backend.prover_init(polynomial)


def route(pairs: int, max_arity: int, slots: int, fold: bool = True) -> tuple[int, int]:
    """(kernel, blocks per SM) a round of `pairs` pairs of this shape takes now
    (fold: a round after the first, which folds the previous challenge in)."""
    out = (ctypes.c_uint32 * 2)()
    check_status(_native.load().hp_cuda_v1_sumcheck_route_query(pairs, max_arity, slots, 1 if fold else 0, out),
                 "sumcheck_route_query")
    return int(out[0]), int(out[1])


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
    ap.add_argument("--prove-num-vars", type=int, action="append", default=[],
                    help="tune the sumcheck round routes of a proof of 2^NV gates (repeatable)")
    ap.add_argument("--out", required=True)
    args = ap.parse_args(argv)
    from .backend import CudaBackend
    be = CudaBackend(args.device)
    nv = args.srs_num_vars
    for pnv in args.prove_num_vars:
        from . import snark
        sel, wit, perm, pub = snark.vanilla_fixture(pnv, 2)
        view = SumcheckTuningBackend(be)
        pk = snark.preprocess(be, pnv, min(16, 1 << pnv), sel, perm, be.generate_srs(pnv, 0), commit=False)
        snark.prove(view, pk, pub, wit)
        for key, recs in view.tuned.items():
            for r in recs:
                print(json.dumps({"shape": key} | dataclasses.asdict(r)), flush=True)
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
