"""Synthetic inputs of the measured workloads and their plain / batched runs.

Fixture tables come from the library's ChaCha20 fixture stream
(hp_cuda_v1_fixture_random_fr: seed -> key, keystream block index -> one
canonical Fr reduced from 64 bytes); they do not reproduce arkworks'
StdRng/Fr::rand streams.

  sumcheck instance (degree 2): 6 MLEs of 2^nv uniform Fr (stream `seed`,
      table j = elements [j 2^nv, (j+1) 2^nv) from `first`), 4 arity-2 products
      over factor pairs (0,1), (2,3), (4,5), (0,3) with uniform coefficients
      (stream 10 + seed).  nv = 20, seed 1 is the sumcheck-prove workload.
  batch plan: 64 MSM sizes 2^k, k uniform in {12..22}, and 32 sumcheck
      num_vars uniform in {14..22}, drawn by random.Random(seed) (seed 3);
      MSM i takes scalars [sum_{j<i} 2^{k_j}, ...) of stream `seed` and the
      first 2^{k_i} bases of SRS layer 0; sumcheck instance i is the instance
      above at its num_vars with stream seed 100 + seed + i.
"""
from __future__ import annotations

import ctypes
import random

import numpy as np

from . import protocol
from .virtual_polynomial import VirtualPolynomial

SUMCHECK_PAIRS = [(0, 1), (2, 3), (4, 5), (0, 3)]
SUMCHECK_LABEL = b"Initializing SumCheck transcript"


def fixture_fr(seed: int, count: int, first: int = 0) -> np.ndarray:
    """`count` canonical Fr (32-byte LE rows, flat uint8) of fixture stream `seed`."""
    from . import _native
    from .errors import check_status
    out = np.empty(32 * max(1, count), dtype=np.uint8)
    check_status(_native.load().hp_cuda_v1_fixture_random_fr(ctypes.c_uint64(seed), ctypes.c_uint64(first), count,
                                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
                 "fixture_random_fr")
    return out[:32 * count]


def fr_ints(table: np.ndarray) -> list[int]:
    raw = table.tobytes()
    return [int.from_bytes(raw[32 * i:32 * i + 32], "little") for i in range(len(raw) // 32)]


def sumcheck_tables(nv: int, seed: int) -> list[np.ndarray]:
    n = 1 << nv
    return [fixture_fr(seed, n, first=j * n) for j in range(6)]


def sumcheck_coefficients(seed: int) -> list[int]:
    return fr_ints(fixture_fr(10 + seed, len(SUMCHECK_PAIRS)))


def sumcheck_polynomial(nv: int, mles: list, coefs: list) -> VirtualPolynomial:
    vp = VirtualPolynomial(nv)
    for c, (a, b) in zip(coefs, SUMCHECK_PAIRS):
        vp.add_mle_list([mles[a], mles[b]], c)
    return vp


def batch_plan(seed: int = 3, msm_count: int = 64, msm_k=(12, 22), sumcheck_count: int = 32,
               sumcheck_nv=(14, 22)) -> tuple[list[int], list[int]]:
    rng = random.Random(seed)
    ks = [rng.randint(*msm_k) for _ in range(msm_count)]
    nvs = [rng.randint(*sumcheck_nv) for _ in range(sumcheck_count)]
    return ks, nvs


def batch_msm_scalars(ks: list[int], seed: int = 3) -> list[np.ndarray]:
    out, first = [], 0
    for k in ks:
        out.append(fixture_fr(seed, 1 << k, first=first))
        first += 1 << k
    return out


class BatchWorkload:
    """The batch plan's inputs resident on one backend: MSM scalar MLEs and
    each sumcheck instance's six MLEs with its coefficients."""

    def __init__(self, backend, pcs_param, ks: list[int], nvs: list[int], seed: int = 3):
        self.backend, self.pcs_param = backend, pcs_param
        self.ks, self.nvs, self.seed = ks, nvs, seed
        self.msm_mles = [backend.mle_from_evaluations(k, s) for k, s in zip(ks, batch_msm_scalars(ks, seed))]
        self.sc_mles, self.sc_coefs = [], []
        for i, nv in enumerate(nvs):
            s = 100 + seed + i
            self.sc_mles.append([backend.mle_from_evaluations(nv, t) for t in sumcheck_tables(nv, s)])
            self.sc_coefs.append(sumcheck_coefficients(s))

    def polynomials(self) -> list:
        return [sumcheck_polynomial(nv, m, c) for nv, m, c in zip(self.nvs, self.sc_mles, self.sc_coefs)]

    def run_batched(self, transcript_cls) -> tuple[list, list]:
        """All MSMs in one batch_msm call, all sumchecks advanced in lockstep
        (one batch_prove_round call per round)."""
        commits = self.backend.batch_msm(self.pcs_param, 0, self.msm_mles)
        finals = []
        proofs = protocol.batch_sumcheck_prove(self.backend, self.polynomials(),
                                               [transcript_cls(SUMCHECK_LABEL) for _ in self.nvs], finals)
        return commits, list(zip(proofs, finals))

    def run_plain(self, transcript_cls) -> tuple[list, list]:
        """One MSM per call, one sumcheck proof after another."""
        commits = [self.backend.batch_msm(self.pcs_param, 0, [m])[0] for m in self.msm_mles]
        out = []
        for vp in self.polynomials():
            finals = []
            proof = protocol.sumcheck_prove(self.backend, vp, transcript_cls(SUMCHECK_LABEL), finals)
            out.append((proof, finals))
        return commits, out
