"""TEST INFRASTRUCTURE ONLY -- Python face of the C oracle (hp_oracle.c).

CpuBackend restates the reference's CPU backend (backend/src/cpu/*.rs) with the
same method names and value conventions as hyperplonk_gb300.backend.CudaBackend
(Fr as ints, tables as canonical 32-byte packets, G1 as (x, y) / None), so
parity tests can drive both backends with one script.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
from typing import Iterable, Optional, Sequence

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libhp_oracle.so"

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
Q = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB

_u8p = ctypes.POINTER(ctypes.c_uint8)
_lib = None


class OracleInvalidParameters(Exception):
    pass


class OracleInvalidState(Exception):
    pass


def build() -> pathlib.Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        build()
    lib = ctypes.CDLL(str(LIB_PATH))
    lib.or_set_threads.argtypes = [ctypes.c_int]
    lib.or_set_threads.restype = ctypes.c_int
    lib.or_field_op.argtypes = [ctypes.c_int, ctypes.c_int, _u8p, _u8p, _u8p, ctypes.c_size_t]
    lib.or_field_op.restype = ctypes.c_size_t
    lib.or_fr_from_wide.argtypes = [_u8p, _u8p, ctypes.c_size_t]
    lib.or_g1_op.argtypes = [ctypes.c_int, _u8p, _u8p, ctypes.POINTER(ctypes.c_uint64), _u8p, ctypes.c_size_t]
    lib.or_g1_op.restype = ctypes.c_size_t
    lib.or_g1_on_curve.argtypes = [_u8p]
    lib.or_msm.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p]
    lib.or_mle_linear_combination.argtypes = [ctypes.c_size_t, ctypes.POINTER(_u8p), _u8p, ctypes.c_size_t, _u8p]
    lib.or_mle_evaluate.argtypes = [_u8p, ctypes.c_size_t, _u8p, _u8p]
    lib.or_mle_build_eq_x_r.argtypes = [_u8p, ctypes.c_size_t, _u8p]
    lib.or_eq_eval.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p]
    lib.or_mle_frac.argtypes = [ctypes.c_size_t, ctypes.POINTER(_u8p), ctypes.POINTER(_u8p), ctypes.c_size_t, _u8p]
    lib.or_mle_product_poly.argtypes = [_u8p, ctypes.c_size_t, _u8p]
    lib.or_mle_nums_denoms.argtypes = [ctypes.c_size_t, _u8p, _u8p, ctypes.POINTER(_u8p), ctypes.POINTER(_u8p),
                                       ctypes.POINTER(_u8p), ctypes.c_size_t, ctypes.POINTER(_u8p),
                                       ctypes.POINTER(_u8p)]
    lib.or_mle_product_factors.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p, _u8p]
    lib.or_sumcheck_create.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.POINTER(_u8p), ctypes.c_size_t,
                                       _u8p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_size_t,
                                       ctypes.POINTER(ctypes.c_size_t), ctypes.c_size_t]
    lib.or_sumcheck_create.restype = ctypes.c_void_p
    lib.or_sumcheck_round.argtypes = [ctypes.c_void_p, _u8p, _u8p]
    lib.or_sumcheck_final.argtypes = [ctypes.c_void_p, _u8p, _u8p]
    lib.or_sumcheck_destroy.argtypes = [ctypes.c_void_p]
    lib.or_kzg_commit.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p]
    lib.or_kzg_open.argtypes = [ctypes.POINTER(_u8p), _u8p, ctypes.c_size_t, _u8p, _u8p, _u8p]
    lib.or_chacha20_block.argtypes = [ctypes.c_uint64, ctypes.c_uint64, _u8p]
    lib.or_random_fr.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_size_t, _u8p]
    lib.or_srs_gen.argtypes = [ctypes.c_size_t, ctypes.c_uint64, _u8p]
    lib.or_g1_generator.argtypes = [_u8p]
    lib.or_set_threads(int(os.environ.get("HP_ORACLE_THREADS", "0")))
    _lib = lib
    return lib


def set_threads(n: int) -> int:
    return load().or_set_threads(n)


def _p(data) -> ctypes.POINTER(ctypes.c_uint8):
    if data is None:
        return None
    if isinstance(data, np.ndarray):
        return data.ctypes.data_as(_u8p)
    if isinstance(data, bytes):
        return ctypes.cast(ctypes.c_char_p(data), _u8p)
    arr = (ctypes.c_uint8 * len(data)).from_buffer(data)
    return ctypes.cast(arr, _u8p)


def _out(n: int):
    return (ctypes.c_uint8 * max(1, n))()


def _ptrs(items: Sequence[bytes]):
    arr = (_u8p * max(1, len(items)))()
    for i, it in enumerate(items):
        arr[i] = _p(it)
    return arr


def fr_bytes(x: int) -> bytes:
    return (x % R).to_bytes(32, "little")


def frs_bytes(xs: Iterable[int]) -> bytes:
    return b"".join(fr_bytes(x) for x in xs)


def fr_int(b) -> int:
    return int.from_bytes(bytes(b[:32]), "little")


def frs_ints(b) -> list[int]:
    b = bytes(b)
    return [int.from_bytes(b[i:i + 32], "little") for i in range(0, len(b), 32)]


def affine_to_point(b):
    b = bytes(b)
    if not any(b):
        return None
    return (int.from_bytes(b[:48], "little"), int.from_bytes(b[48:96], "little"))


def point_to_affine(p) -> bytes:
    if p is None:
        return bytes(96)
    return p[0].to_bytes(48, "little") + p[1].to_bytes(48, "little")


def packets_to_affine(packets) -> bytes:
    """97-byte G1 packets -> 96-byte affine (infinity -> zeros)."""
    a = np.frombuffer(bytes(packets), dtype=np.uint8).reshape(-1, 97)
    out = a[:, 1:].copy()
    out[a[:, 0] != 0] = 0
    return out.tobytes()


def affine_to_packets(affine) -> bytes:
    a = np.frombuffer(bytes(affine), dtype=np.uint8).reshape(-1, 96)
    n = a.shape[0]
    out = np.zeros((n, 97), dtype=np.uint8)
    out[:, 1:] = a
    inf = ~a.any(axis=1)
    out[inf, 0] = 1
    return out.tobytes()


# ---------------------------------------------------------------------------
# primitives
# ---------------------------------------------------------------------------

def field_op(field: int, op: int, a: bytes, b: Optional[bytes], n: int) -> bytes:
    width = 32 if field == 0 else 48
    out = _out(width * n)
    bad = load().or_field_op(field, op, _p(a), _p(b if b is not None else a), out, n)
    if bad:
        raise OracleInvalidParameters(f"non-canonical input at {bad - 1}")
    return bytes(out)[:width * n]


def fr_from_wide(wide: bytes) -> bytes:
    n = len(wide) // 64
    out = _out(32 * n)
    load().or_fr_from_wide(_p(wide), out, n)
    return bytes(out)[:32 * n]


def g1_op(op: int, a: bytes, b: Optional[bytes] = None, k: Optional[Sequence[int]] = None) -> bytes:
    n = len(a) // 96
    out = _out(96 * n)
    karr = (ctypes.c_uint64 * max(1, n))(*(k or [0] * n))
    bad = load().or_g1_op(op, _p(a), _p(b if b is not None else a), karr, out, n)
    if bad:
        raise OracleInvalidParameters(f"bad point at {bad - 1}")
    return bytes(out)[:96 * n]


def g1_generator() -> bytes:
    out = _out(96)
    load().or_g1_generator(out)
    return bytes(out)


def msm(bases_affine: bytes, scalars: bytes) -> bytes:
    """Sum scalars[i] * bases[i] (96-byte affine in/out)."""
    n = len(scalars) // 32
    out = _out(96)
    if load().or_msm(_p(bases_affine), _p(scalars), n, out):
        raise OracleInvalidParameters("non-canonical MSM input")
    return bytes(out)


def chacha20_block(seed: int, index: int) -> bytes:
    out = _out(64)
    load().or_chacha20_block(seed, index, out)
    return bytes(out)


def random_fr(seed: int, n: int, first: int = 0) -> bytes:
    """n canonical Fr of fixture stream `seed` (keystream blocks first..first+n)."""
    out = np.empty(32 * max(1, n), dtype=np.uint8)
    load().or_random_fr(seed, first, n, out.ctypes.data_as(_u8p))
    return out[:32 * n].tobytes()


def srs_layers(num_vars: int, seed: int) -> list[bytes]:
    """Testing SRS (srs.rs:158-235 restated): num_vars + 1 layers of 96-byte
    affine points, layer i holding 2^(num_vars - i) points."""
    total = (1 << (num_vars + 1)) - 1
    out = np.empty(96 * total, dtype=np.uint8)
    if load().or_srs_gen(num_vars, seed, out.ctypes.data_as(_u8p)):
        raise OracleInvalidParameters("bad SRS request")
    layers, off = [], 0
    for i in range(num_vars + 1):
        cnt = 1 << (num_vars - i) if i < num_vars else 1
        layers.append(out[96 * off:96 * (off + cnt)].tobytes())
        off += cnt
    return layers


# ---------------------------------------------------------------------------
# CpuBackend (backend/src/cpu)
# ---------------------------------------------------------------------------

class CpuMle:
    __slots__ = ("num_vars", "evaluations", "__weakref__")

    def __init__(self, num_vars: int, evaluations: bytes):
        self.num_vars = num_vars
        self.evaluations = bytes(evaluations)

    def id(self) -> int:
        return id(self)


def _table(evaluations) -> bytes:
    if isinstance(evaluations, (bytes, bytearray, memoryview)):
        return bytes(evaluations)
    if isinstance(evaluations, np.ndarray):
        return evaluations.astype(np.uint8).tobytes()
    return frs_bytes(evaluations)


class CpuPreparedProverParam:
    def __init__(self, num_vars: int, layers: list[bytes]):
        self.num_vars = num_vars
        self.layers = layers  # 96-byte affine


class CpuSumCheckState:
    def __init__(self, handle, degree: int, factor_count: int):
        self.handle = handle
        self.degree = degree
        self.factor_count = factor_count

    def __del__(self):
        if self.handle:
            load().or_sumcheck_destroy(self.handle)
            self.handle = None


class CpuBackend:
    def mle_from_evaluations(self, num_vars: int, evaluations) -> CpuMle:
        data = _table(evaluations)
        if num_vars >= 64 or len(data) != 32 * (1 << num_vars):
            raise OracleInvalidParameters("evaluation count does not match variables")
        if any(x >= R for x in frs_ints(data)) if num_vars <= 12 else False:
            raise OracleInvalidParameters("non-canonical evaluation")
        return CpuMle(num_vars, data)

    def download(self, mle: CpuMle) -> bytes:
        return mle.evaluations

    def linear_combination(self, polynomials, coefficients) -> CpuMle:
        if not polynomials or len(polynomials) != len(coefficients) or any(
                p.num_vars != polynomials[0].num_vars for p in polynomials):
            raise OracleInvalidParameters("linear combination requires matching counts and dimensions")
        nv = polynomials[0].num_vars
        out = _out(32 << nv)
        load().or_mle_linear_combination(nv, _ptrs([p.evaluations for p in polynomials]),
                                         _p(frs_bytes(coefficients)), len(polynomials), out)
        return CpuMle(nv, bytes(out)[:32 << nv])

    def evaluate_mle(self, mle: CpuMle, point: Sequence[int]) -> int:
        if len(point) != mle.num_vars:
            raise OracleInvalidParameters("wrong number of variables")
        out = _out(32)
        load().or_mle_evaluate(_p(mle.evaluations), mle.num_vars, _p(frs_bytes(point)) if point else None, out)
        return fr_int(bytes(out))

    def build_eq_x_r(self, r: Sequence[int]) -> CpuMle:
        if not r:
            raise OracleInvalidParameters("r length is 0")
        nv = len(r)
        out = _out(32 << nv)
        load().or_mle_build_eq_x_r(_p(frs_bytes(r)), nv, out)
        return CpuMle(nv, bytes(out)[:32 << nv])

    def compute_frac_poly(self, fxs, gxs) -> CpuMle:
        nv = fxs[0].num_vars
        out = _out(32 << nv)
        rc = load().or_mle_frac(nv, _ptrs([f.evaluations for f in fxs]), _ptrs([g.evaluations for g in gxs]),
                                len(fxs), out)
        if rc:
            raise OracleInvalidParameters("gxs has zero entries in the boolean hypercube")
        return CpuMle(nv, bytes(out)[:32 << nv])

    def compute_product_poly(self, frac: CpuMle) -> CpuMle:
        if frac.num_vars == 0:
            raise OracleInvalidParameters("product polynomial requires at least one variable")
        nv = frac.num_vars
        out = _out(32 << nv)
        load().or_mle_product_poly(_p(frac.evaluations), nv, out)
        return CpuMle(nv, bytes(out)[:32 << nv])

    def compute_nums_and_denoms(self, beta, gamma, fxs, gxs, perms):
        nv = fxs[0].num_vars
        k = len(fxs)
        outs_n = [_out(32 << nv) for _ in range(k)]
        outs_d = [_out(32 << nv) for _ in range(k)]
        pn = (_u8p * k)(*[ctypes.cast(o, _u8p) for o in outs_n])
        pd = (_u8p * k)(*[ctypes.cast(o, _u8p) for o in outs_d])
        load().or_mle_nums_denoms(nv, _p(fr_bytes(beta)), _p(fr_bytes(gamma)), _ptrs([f.evaluations for f in fxs]),
                                  _ptrs([g.evaluations for g in gxs]), _ptrs([p.evaluations for p in perms]), k, pn, pd)
        return ([CpuMle(nv, bytes(o)[:32 << nv]) for o in outs_n],
                [CpuMle(nv, bytes(o)[:32 << nv]) for o in outs_d])

    def compute_product_factors(self, frac: CpuMle, prod: CpuMle):
        nv = frac.num_vars
        if nv == 0 or prod.num_vars != nv:
            raise OracleInvalidParameters("product factors require matching positive dimensions")
        a, b = _out(32 << nv), _out(32 << nv)
        load().or_mle_product_factors(_p(frac.evaluations), _p(prod.evaluations), nv, a, b)
        return [CpuMle(nv, bytes(a)[:32 << nv]), CpuMle(nv, bytes(b)[:32 << nv])]

    # ---- KZG ----
    def prepare_prover_param(self, num_vars: int, powers_of_g) -> CpuPreparedProverParam:
        layers = []
        for layer in powers_of_g:
            if isinstance(layer, (bytes, bytearray, np.ndarray)):
                b = bytes(layer)
                layers.append(packets_to_affine(b) if len(b) % 97 == 0 and len(b) % 96 != 0 else b)
            else:
                layers.append(b"".join(point_to_affine(p) for p in layer))
        return CpuPreparedProverParam(num_vars, layers)

    def commit(self, pp: CpuPreparedProverParam, poly: CpuMle):
        if pp.num_vars < poly.num_vars:
            raise OracleInvalidParameters("MLE length exceeds param limit")
        out = _out(96)
        load().or_kzg_commit(_p(pp.layers[pp.num_vars - poly.num_vars]), _p(poly.evaluations), poly.num_vars, out)
        return affine_to_point(bytes(out))

    def multi_commit(self, pp, polys):
        return [self.commit(pp, p) for p in polys]

    def open(self, pp: CpuPreparedProverParam, poly: CpuMle, point: Sequence[int]):
        nv = poly.num_vars
        if nv > pp.num_vars or nv != len(point):
            raise OracleInvalidParameters("bad open dimensions")
        ignored = pp.num_vars - nv + 1
        layers = [pp.layers[ignored + i] for i in range(nv)]
        q = _out(96 * max(1, nv))
        ev = _out(32)
        load().or_kzg_open(_ptrs(layers), _p(poly.evaluations), nv, _p(frs_bytes(point)) if nv else None, q, ev)
        qb = bytes(q)
        return [affine_to_point(qb[96 * i:96 * i + 96]) for i in range(nv)], fr_int(bytes(ev))

    # ---- SumCheck ----
    def prover_init(self, poly) -> CpuSumCheckState:
        nv, d = poly.aux_info.num_variables, poly.aux_info.max_degree
        if nv == 0 or d == 0:
            raise OracleInvalidParameters("SumCheck requires positive variable count and degree.")
        factors = poly.flattened_ml_extensions()
        offsets, indices, coefs = [0], [], []
        for c, ix in poly.products:
            indices.extend(ix)
            offsets.append(len(indices))
            coefs.append(c)
        off = (ctypes.c_size_t * len(offsets))(*offsets)
        idx = (ctypes.c_size_t * max(1, len(indices)))(*indices)
        h = load().or_sumcheck_create(nv, d, _ptrs([f.evaluations for f in factors]), len(factors),
                                      _p(frs_bytes(coefs)) if coefs else None, off, len(coefs), idx, len(indices))
        if not h:
            raise OracleInvalidParameters("bad sumcheck description")
        return CpuSumCheckState(h, d, len(factors))

    def prove_round_and_update_state(self, state: CpuSumCheckState, challenge: Optional[int]):
        out = _out(32 * (state.degree + 1))
        rc = load().or_sumcheck_round(state.handle, _p(fr_bytes(challenge)) if challenge is not None else None, out)
        if rc == 2:
            raise OracleInvalidState("sumcheck round misuse")
        if rc:
            raise OracleInvalidParameters("bad challenge")
        return frs_ints(bytes(out)[:32 * (state.degree + 1)])

    def final_evaluations(self, state: CpuSumCheckState, challenge: int) -> list[int]:
        out = _out(32 * max(1, state.factor_count))
        rc = load().or_sumcheck_final(state.handle, _p(fr_bytes(challenge)), out)
        if rc:
            raise OracleInvalidState("final evaluations need all rounds")
        return frs_ints(bytes(out)[:32 * state.factor_count])
