"""CudaBackend: the reference's backend traits over the GB300 C ABI.

Mirrors, method for method, the Rust traits the reference's device backend
implements (backend/src/multilinear_polynomial.rs:33-121 MleBackend,
backend/src/multilinear_kzg.rs:20-55 MultilinearKzgBackend,
backend/src/sum_check.rs:17-38 SumCheckProver), the way
backend/src/ascend910b3/{multilinear_polynomial,multilinear_kzg,sum_check}.rs
wrap the Ascend bridge: argument validation, packet encoding, RAII handles.

Value conventions: Fr scalars are Python ints (canonical, reduced mod r on
input); MLE tables cross as canonical little-endian 32-byte packets
(bytes / bytearray / uint8 numpy arrays); G1 points are (x, y) int tuples,
None for the point at infinity.
"""
from __future__ import annotations

import contextlib
import os
import sys
import ctypes
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _native
from .errors import InvalidParameters, InvalidState, check_status
from .virtual_polynomial import R_MODULUS, VirtualPolynomial

Q_MODULUS = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB


# --------------------------------------------------------------------------
# packets (backend/src/ascend910b3/encoding.rs:12-108)
# --------------------------------------------------------------------------

def encode_fr(x: int) -> bytes:
    return (x % R_MODULUS).to_bytes(32, "little")


def decode_fr(b: bytes) -> int:
    v = int.from_bytes(bytes(b[:32]), "little")
    if v >= R_MODULUS:
        raise InvalidState("noncanonical Fr packet")
    return v


def encode_frs(xs: Sequence[int]) -> bytes:
    return b"".join(encode_fr(x) for x in xs)


def encode_g1(p) -> bytes:
    if p is None:
        return b"\x01" + bytes(96)
    x, y = p
    return b"\x00" + int(x).to_bytes(48, "little") + int(y).to_bytes(48, "little")


def decode_g1(b: bytes):
    """97-byte packet -> (x, y) or None.  Checks the tag, canonical
    coordinates and the curve equation y^2 = x^3 + 4."""
    b = bytes(b)
    if len(b) != 97:
        raise InvalidState("invalid G1 packet length")
    if b[0] == 1 and not any(b[1:]):
        return None
    if b[0] != 0:
        raise InvalidState("invalid G1 tag or infinity coordinates")
    x = int.from_bytes(b[1:49], "little")
    y = int.from_bytes(b[49:97], "little")
    if x >= Q_MODULUS or y >= Q_MODULUS or (y * y - x * x * x - 4) % Q_MODULUS != 0:
        raise InvalidState("invalid finite G1 packet")
    return (x, y)


def table_bytes(evaluations) -> bytes | np.ndarray:
    """Accept packets (bytes-like / uint8 array) or a sequence of ints."""
    if isinstance(evaluations, (bytes, bytearray, memoryview)):
        return evaluations
    if isinstance(evaluations, np.ndarray):
        if evaluations.dtype != np.uint8:
            raise InvalidParameters("evaluation array must be uint8 packets")
        return np.ascontiguousarray(evaluations).reshape(-1)
    return encode_frs(list(evaluations))


def _nbytes(data) -> int:
    return data.nbytes if isinstance(data, np.ndarray) else len(data)


# --------------------------------------------------------------------------
# handles
# --------------------------------------------------------------------------

def _destroy_or_abort(op: str, status) -> None:
    """A handle destructor's status: a failure is a contract violation that
    cannot be reported to a caller (destructors have none), so the process
    aborts after saying what failed, as the reference's device backend does
    (backend/src/ascend910b3/mod.rs:46-47, context.rs:126-128)."""
    if status.kind == 0:
        return
    sys.stderr.write(f"hyperplonk_gb300: {op} failed while destroying a handle (status kind {status.kind}, "
                     f"native code {status.native_code}); aborting\n")
    sys.stderr.flush()
    os.abort()


class CudaContext:
    """One device, one stream (bridge.h: single host thread, single stream)."""

    def __init__(self, device_id: int = 0):
        self.lib = _native.load()
        raw = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_context_create(int(device_id), ctypes.byref(raw)),
                     "context_create")
        self.raw = raw
        self.device_id = device_id
        # Set by a caller that drives this context from several host threads
        # (one at a time): handle destructors then take it too, so a retire
        # never overlaps another thread's call on the context.
        self.lock = None

    def held(self):
        return self.lock if self.lock is not None else contextlib.nullcontext()

    def stream(self) -> int:
        out = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_context_stream(self.raw, ctypes.byref(out)), "context_stream")
        return out.value or 0

    def memory(self, reset_high: bool = False) -> tuple[int, int, int]:
        """(bytes in use, high-water mark since the last reset, bytes held)
        of the context's memory pool (hp_cuda_v1_context_memory)."""
        out = (ctypes.c_uint64 * 3)()
        check_status(self.lib.hp_cuda_v1_context_memory(self.raw, 1 if reset_high else 0, out), "context_memory")
        return int(out[0]), int(out[1]), int(out[2])

    def close(self) -> None:
        if self.raw is not None and self.raw.value:
            check_status(self.lib.hp_cuda_v1_context_destroy(self.raw), "context_destroy")
        self.raw = None

    def __del__(self):
        raw = getattr(self, "raw", None)
        if raw is not None and raw.value:
            self.raw = None
            _destroy_or_abort("context_destroy", self.lib.hp_cuda_v1_context_destroy(raw))


class CudaMle:
    """Shared, immutable device-resident MLE (multilinear_polynomial.rs:22-27).
    Python references share the handle; the buffer is retired when the last
    reference goes away."""

    __slots__ = ("_ctx", "_addr", "num_vars", "__weakref__")

    def __init__(self, ctx: CudaContext, addr: int, num_vars: int):
        self._ctx = ctx
        self._addr = addr
        self.num_vars = num_vars

    def id(self) -> int:
        return self._addr

    @property
    def address(self) -> int:
        return self._addr

    def __del__(self):
        ctx = self._ctx
        addr, self._addr = self._addr, 0
        if ctx is not None and ctx.raw is not None and addr:
            with ctx.held():
                status = ctx.lib.hp_cuda_v1_buffer_retire(ctx.raw, ctypes.c_void_p(addr))
            _destroy_or_abort("buffer_retire", status)


class CudaPreparedProverParam:
    def __init__(self, ctx: CudaContext, raw: ctypes.c_void_p, num_vars: int):
        self._ctx, self.raw, self.num_vars = ctx, raw, num_vars

    def __del__(self):
        ctx = self._ctx
        raw, self.raw = self.raw, None
        if ctx is not None and ctx.raw is not None and raw is not None:
            with ctx.held():
                status = ctx.lib.hp_cuda_v1_multilinear_kzg_params_destroy(ctx.raw, raw)
            _destroy_or_abort("multilinear_kzg_params_destroy", status)


class CudaSumCheckProverState:
    def __init__(self, ctx: CudaContext, raw: ctypes.c_void_p, degree: int, factor_count: int):
        self._ctx, self.raw = ctx, raw
        self.round_evaluation_count = degree + 1
        self.factor_count = factor_count

    def __del__(self):
        ctx = self._ctx
        raw, self.raw = self.raw, None
        if ctx is not None and ctx.raw is not None and raw is not None:
            with ctx.held():
                status = ctx.lib.hp_cuda_v1_sumcheck_prover_state_destroy(ctx.raw, raw)
            _destroy_or_abort("sumcheck_prover_state_destroy", status)


class AsyncUpload:
    """Tables of one hp_cuda_v1_mle_upload_async call: `mles` are usable at
    once (device work waits for the copies); wait() blocks until the upload is
    complete, checks the encoding (InvalidParameters on a non-canonical
    element, the tables then released) and lets go of the host buffers."""

    def __init__(self, backend: "CudaBackend", mles: list, host_buffers: list):
        self.backend, self.mles, self._host = backend, mles, host_buffers

    def wait(self) -> list:
        if self._host is not None:
            arr = _addr_array(self.mles)
            try:
                check_status(self.backend.lib.hp_cuda_v1_mle_upload_wait(self.backend.ctx.raw, arr, len(self.mles)),
                             "mle_upload_wait")
            except InvalidParameters:
                for m in self.mles:  # the library released them
                    m._addr = 0
                self.mles = []
                raise
            finally:
                self._host = None
        return self.mles


def _addr_array(mles: Sequence[CudaMle]):
    arr = (ctypes.c_void_p * max(1, len(mles)))()
    for i, m in enumerate(mles):
        arr[i] = m.address
    return arr


# --------------------------------------------------------------------------
# backend
# --------------------------------------------------------------------------

class CudaBackend:
    """GB300 implementation of MleBackend + MultilinearKzgBackend + SumCheckProver."""

    def __init__(self, device_id: int = 0):
        self.ctx = CudaContext(device_id)
        self.lib = self.ctx.lib

    def _check_mle(self, mle: CudaMle) -> None:
        if not isinstance(mle, CudaMle) or mle._ctx is not self.ctx:
            raise InvalidParameters("MLE belongs to another backend context")

    def _new(self, addr: ctypes.c_void_p, num_vars: int) -> CudaMle:
        return CudaMle(self.ctx, addr.value, num_vars)

    # ---- MleBackend ----------------------------------------------------
    def mle_from_evaluations(self, num_vars: int, evaluations) -> CudaMle:
        data = table_bytes(evaluations)
        n = _nbytes(data)
        if num_vars >= 64 or n % 32 or n // 32 != (1 << num_vars):
            raise InvalidParameters(f"evaluation count {n // 32} does not match {num_vars} variables")
        out = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_mle_upload(self.ctx.raw, num_vars, _native.buf(data), n // 32,
                                                    ctypes.byref(out)), "mle_upload")
        return self._new(out, num_vars)

    def mle_from_evaluations_many(self, num_vars: int, tables: Sequence) -> list:
        """Several tables of the same size in one upload call (one validation
        synchronisation); equal to mle_from_evaluations of each."""
        datas = [table_bytes(t) for t in tables]
        for d in datas:
            n = _nbytes(d)
            if num_vars >= 64 or n % 32 or n // 32 != (1 << num_vars):
                raise InvalidParameters(f"evaluation count {n // 32} does not match {num_vars} variables")
        if not datas:
            return []
        ptrs = (_native.c_u8p * len(datas))(*[_native.buf(d) for d in datas])
        out = (ctypes.c_void_p * len(datas))()
        check_status(self.lib.hp_cuda_v1_mle_upload_many(self.ctx.raw, num_vars, ptrs, len(datas), 1 << num_vars,
                                                         out), "mle_upload_many")
        return [self._new(ctypes.c_void_p(a), num_vars) for a in out]

    def mle_upload_async(self, num_vars: int, tables: Sequence) -> "AsyncUpload":
        """Queue the upload of several tables of one size on the context's
        ingress stream and return at once (hp_cuda_v1_mle_upload_async): work
        queued later on the tables waits for the upload on the device, so the
        copies overlap whatever the context is computing.  The tables should
        be pinned host memory (else the copies are synchronous).  Call wait()
        on the result before trusting results computed from the tables: it
        checks the encoding and releases the host buffers."""
        datas = [table_bytes(t) for t in tables]
        for d in datas:
            n = _nbytes(d)
            if num_vars >= 64 or n % 32 or n // 32 != (1 << num_vars):
                raise InvalidParameters(f"evaluation count {n // 32} does not match {num_vars} variables")
        ptrs = (_native.c_u8p * max(1, len(datas)))(*[_native.buf(d) for d in datas])
        out = (ctypes.c_void_p * max(1, len(datas)))()
        check_status(self.lib.hp_cuda_v1_mle_upload_async(self.ctx.raw, num_vars, ptrs, len(datas), 1 << num_vars,
                                                          out), "mle_upload_async")
        return AsyncUpload(self, [self._new(ctypes.c_void_p(a), num_vars) for a in out[:len(datas)]], datas)

    def generate_srs(self, num_vars: int, seed: int) -> list:
        """Testing SRS of num_vars variables from fixture seed `seed`, computed
        on the device: num_vars + 1 layers of 97-byte packets (uint8 arrays),
        layer i holding 2^(num_vars - i) points."""
        total = (1 << (num_vars + 1)) - 1
        packets = np.empty(total * 97, dtype=np.uint8)
        check_status(self.lib.hp_cuda_v1_srs_generate(self.ctx.raw, num_vars, seed, _native.buf(packets), total),
                     "srs_generate")
        layers, off = [], 0
        for i in range(num_vars + 1):
            cnt = 1 << (num_vars - i) if i < num_vars else 1
            layers.append(packets[97 * off:97 * (off + cnt)])
            off += cnt
        return layers

    def download(self, mle: CudaMle) -> bytes:
        """Canonical table bytes of a resident MLE (test/debug helper)."""
        self._check_mle(mle)
        n = 1 << mle.num_vars
        out = (ctypes.c_uint8 * (32 * n))()
        check_status(self.lib.hp_cuda_v1_mle_download(self.ctx.raw, ctypes.c_void_p(mle.address), mle.num_vars,
                                                      out, n), "mle_download")
        return bytes(out)

    def linear_combination(self, polynomials: Sequence[CudaMle], coefficients: Sequence[int]) -> CudaMle:
        if not polynomials:
            raise InvalidParameters("linear combination requires nonempty polynomials")
        nv = polynomials[0].num_vars
        if len(polynomials) != len(coefficients) or any(p.num_vars != nv for p in polynomials):
            raise InvalidParameters("linear combination requires matching counts and dimensions")
        for p in polynomials:
            self._check_mle(p)
        coefs = encode_frs(coefficients)
        out = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_mle_linear_combination(
            self.ctx.raw, nv, _addr_array(polynomials), _native.buf(coefs), len(polynomials),
            ctypes.byref(out)), "mle_linear_combination")
        return self._new(out, nv)

    def evaluate_mle(self, mle: CudaMle, point: Sequence[int]) -> int:
        self._check_mle(mle)
        if len(point) != mle.num_vars:
            raise InvalidParameters(f"wrong number of variables {mle.num_vars} vs {len(point)}")
        pt = encode_frs(point) if point else None
        out = (ctypes.c_uint8 * 32)()
        check_status(self.lib.hp_cuda_v1_mle_evaluate(self.ctx.raw, ctypes.c_void_p(mle.address), mle.num_vars,
                                                      _native.buf(pt), out), "mle_evaluate")
        return decode_fr(bytes(out))

    def evaluate_many(self, mles: Sequence[CudaMle], points: Sequence[Sequence[int]]) -> list[int]:
        """evaluate_mle of every (mle, point) pair with one synchronisation."""
        if len(mles) != len(points):
            raise InvalidParameters("one point per polynomial")
        if not mles:
            return []
        for m, pt in zip(mles, points):
            self._check_mle(m)
            if len(pt) != m.num_vars:
                raise InvalidParameters(f"wrong number of variables {m.num_vars} vs {len(pt)}")
        nvs = (ctypes.c_size_t * len(mles))(*[m.num_vars for m in mles])
        flat = b"".join(encode_frs(pt) for pt in points)
        out = (ctypes.c_uint8 * (32 * len(mles)))()
        check_status(self.lib.hp_cuda_v1_mle_evaluate_many(self.ctx.raw, len(mles), _addr_array(mles), nvs,
                                                           _native.buf(flat) if flat else None, out),
                     "mle_evaluate_many")
        raw = bytes(out)
        return [decode_fr(raw[32 * i:32 * i + 32]) for i in range(len(mles))]

    def build_eq_x_r(self, r: Sequence[int]) -> CudaMle:
        if len(r) == 0:
            raise InvalidParameters("r length is 0")
        out = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_mle_build_eq_x_r(self.ctx.raw, _native.buf(encode_frs(r)), len(r),
                                                          ctypes.byref(out)), "mle_build_eq_x_r")
        return self._new(out, len(r))

    def compute_frac_poly(self, fxs: Sequence[CudaMle], gxs: Sequence[CudaMle]) -> CudaMle:
        if not fxs or len(fxs) != len(gxs):
            raise InvalidParameters("frac requires nonempty, equally sized lists")
        nv = fxs[0].num_vars
        if any(p.num_vars != nv for p in list(fxs) + list(gxs)):
            raise InvalidParameters("frac requires matching dimensions")
        for p in list(fxs) + list(gxs):
            self._check_mle(p)
        out = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_mle_compute_frac_poly(
            self.ctx.raw, nv, _addr_array(fxs), _addr_array(gxs), len(fxs), ctypes.byref(out)),
            "mle_compute_frac_poly")
        return self._new(out, nv)

    def compute_product_poly(self, frac_poly: CudaMle) -> CudaMle:
        self._check_mle(frac_poly)
        if frac_poly.num_vars == 0:
            raise InvalidParameters("product polynomial requires at least one variable")
        out = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_mle_compute_product_poly(
            self.ctx.raw, ctypes.c_void_p(frac_poly.address), frac_poly.num_vars, ctypes.byref(out)),
            "mle_compute_product_poly")
        return self._new(out, frac_poly.num_vars)

    def compute_nums_and_denoms(self, beta: int, gamma: int, fxs, gxs, perms):
        k = len(fxs)
        if k == 0 or len(gxs) != k or len(perms) != k:
            raise InvalidParameters("nums/denoms require nonempty, equally sized lists")
        nv = fxs[0].num_vars
        for p in list(fxs) + list(gxs) + list(perms):
            self._check_mle(p)
            if p.num_vars != nv:
                raise InvalidParameters("nums/denoms require matching dimensions")
        nums = (ctypes.c_void_p * k)()
        dens = (ctypes.c_void_p * k)()
        check_status(self.lib.hp_cuda_v1_mle_compute_nums_and_denoms(
            self.ctx.raw, nv, _native.buf(encode_fr(beta)), _native.buf(encode_fr(gamma)),
            _addr_array(fxs), _addr_array(gxs), _addr_array(perms), k, nums, dens),
            "mle_compute_nums_and_denoms")
        return ([CudaMle(self.ctx, nums[i], nv) for i in range(k)],
                [CudaMle(self.ctx, dens[i], nv) for i in range(k)])

    def compute_product_factors(self, frac_poly: CudaMle, prod_poly: CudaMle):
        self._check_mle(frac_poly)
        self._check_mle(prod_poly)
        nv = frac_poly.num_vars
        if nv == 0:
            raise InvalidParameters("product factors require at least one variable")
        if nv != prod_poly.num_vars:
            raise InvalidParameters("product factor inputs have different variable counts")
        a, b = ctypes.c_void_p(), ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_mle_compute_product_factors(
            self.ctx.raw, ctypes.c_void_p(frac_poly.address), ctypes.c_void_p(prod_poly.address), nv,
            ctypes.byref(a), ctypes.byref(b)), "mle_compute_product_factors")
        return [self._new(a, nv), self._new(b, nv)]

    # ---- MultilinearKzgBackend ---------------------------------------
    def prepare_prover_param(self, num_vars: int, powers_of_g: Iterable) -> CudaPreparedProverParam:
        """powers_of_g yields num_vars + 1 layers of decreasing size; a layer is
        either 97-byte packets (bytes-like) or a list of (x, y)/None points."""
        layers = list(powers_of_g)
        if len(layers) != num_vars + 1:
            raise InvalidParameters("SRS must contain num_vars + 1 layers")
        raw = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_multilinear_kzg_params_create(self.ctx.raw, num_vars, ctypes.byref(raw)),
                     "multilinear_kzg_params_create")
        params = CudaPreparedProverParam(self.ctx, raw, num_vars)
        for i, layer in enumerate(layers):
            count = 1 << (num_vars - i) if i < num_vars else 1
            if isinstance(layer, (bytes, bytearray, memoryview, np.ndarray)):
                packets = layer
            else:
                packets = b"".join(encode_g1(p) for p in layer)
            if _nbytes(packets) != 97 * count:
                raise InvalidParameters(f"SRS layer {i} has incorrect point count")
            check_status(self.lib.hp_cuda_v1_multilinear_kzg_params_upload_layer(
                self.ctx.raw, params.raw, i, _native.buf(packets), count), "multilinear_kzg_params_upload_layer")
        return params

    def commit(self, prover_param: CudaPreparedProverParam, polynomial: CudaMle):
        self._check_mle(polynomial)
        out = (ctypes.c_uint8 * 97)()
        check_status(self.lib.hp_cuda_v1_multilinear_kzg_commit(
            self.ctx.raw, prover_param.raw, ctypes.c_void_p(polynomial.address), polynomial.num_vars, out),
            "multilinear_kzg_commit")
        return decode_g1(bytes(out))

    def multi_commit(self, prover_param: CudaPreparedProverParam, polynomials: Sequence[CudaMle]):
        if not polynomials:
            return []
        for p in polynomials:
            self._check_mle(p)
        nvs = (ctypes.c_size_t * len(polynomials))(*[p.num_vars for p in polynomials])
        out = (ctypes.c_uint8 * (97 * len(polynomials)))()
        check_status(self.lib.hp_cuda_v1_multilinear_kzg_multi_commit(
            self.ctx.raw, prover_param.raw, _addr_array(polynomials), nvs, len(polynomials), out),
            "multilinear_kzg_multi_commit")
        raw = bytes(out)
        return [decode_g1(raw[97 * i:97 * i + 97]) for i in range(len(polynomials))]

    def open(self, prover_param: CudaPreparedProverParam, polynomial: CudaMle, point: Sequence[int]):
        self._check_mle(polynomial)
        nv = polynomial.num_vars
        if len(point) != nv:
            raise InvalidParameters(f"Polynomial num_vars {nv} does not match point len {len(point)}")
        q = (ctypes.c_uint8 * max(1, 97 * nv))()
        ev = (ctypes.c_uint8 * 32)()
        pt = encode_frs(point) if point else None
        check_status(self.lib.hp_cuda_v1_multilinear_kzg_open(
            self.ctx.raw, prover_param.raw, ctypes.c_void_p(polynomial.address), nv, _native.buf(pt), q, ev),
            "multilinear_kzg_open")
        raw = bytes(q)
        return [decode_g1(raw[97 * i:97 * i + 97]) for i in range(nv)], decode_fr(bytes(ev))

    # ---- SumCheckProver -------------------------------------------------
    def prover_init(self, polynomial: VirtualPolynomial) -> CudaSumCheckProverState:
        """Validates and encodes the product description exactly as
        backend/src/ascend910b3/sum_check.rs:32-90 does."""
        nv = polynomial.aux_info.num_variables
        d = polynomial.aux_info.max_degree
        if nv == 0 or d == 0:
            raise InvalidParameters("SumCheck requires positive variable count and maximum degree")
        factors = polynomial.flattened_ml_extensions()
        if any(f.num_vars != nv for f in factors):
            raise InvalidParameters("SumCheck factor dimensions do not match virtual polynomial metadata")
        offsets, indices, coefs = [0], [], []
        for c, ix in polynomial.products:
            if not ix or len(ix) > d:
                raise InvalidParameters("SumCheck product must have between one and max_degree multiplicands")
            if any(i >= len(factors) for i in ix):
                raise InvalidParameters("SumCheck product references an out-of-range factor")
            indices.extend(ix)
            offsets.append(len(indices))
            coefs.append(c)
        for f in factors:
            self._check_mle(f)
        off = (ctypes.c_size_t * len(offsets))(*offsets)
        idx = (ctypes.c_size_t * max(1, len(indices)))(*indices)
        cb = encode_frs(coefs) if coefs else None
        raw = ctypes.c_void_p()
        check_status(self.lib.hp_cuda_v1_sumcheck_prover_state_create(
            self.ctx.raw, nv, d, _addr_array(factors) if factors else None, len(factors), _native.buf(cb),
            off, len(coefs), idx if indices else None, len(indices), ctypes.byref(raw)),
            "sumcheck_prover_state_create")
        return CudaSumCheckProverState(self.ctx, raw, d, len(factors))

    def prove_round_and_update_state(self, state: CudaSumCheckProverState, challenge: Optional[int]):
        n = state.round_evaluation_count
        out = (ctypes.c_uint8 * (32 * n))()
        ch = _native.buf(encode_fr(challenge)) if challenge is not None else None
        check_status(self.lib.hp_cuda_v1_sumcheck_prover_state_round(self.ctx.raw, state.raw, ch, out, n),
                     "sumcheck_prover_state_round")
        raw = bytes(out)
        return [decode_fr(raw[32 * i:32 * i + 32]) for i in range(n)]

    def prove_rounds(self, state: CudaSumCheckProverState, transcript, rounds: int):
        """All rounds of a fresh state with the Fiat-Shamir step inside the
        library: `transcript` is a native MerlinTranscript.  Returns (round
        messages, challenges)."""
        d1 = state.round_evaluation_count
        msgs = (ctypes.c_uint8 * (32 * d1 * rounds))()
        chs = (ctypes.c_uint8 * (32 * rounds))()
        check_status(self.lib.hp_cuda_v1_sumcheck_prove_rounds(self.ctx.raw, state.raw, transcript.raw, rounds,
                                                              msgs, chs), "sumcheck_prove_rounds")
        mb, cb = bytes(msgs), bytes(chs)
        messages = [[int.from_bytes(mb[32 * (d1 * k + j):32 * (d1 * k + j) + 32], "little") for j in range(d1)]
                    for k in range(rounds)]
        return messages, [int.from_bytes(cb[32 * k:32 * k + 32], "little") for k in range(rounds)]

    # ---- batched execution (no counterpart in the reference traits) ----
    def batch_msm(self, prover_param: CudaPreparedProverParam, layer_index: int, scalars: Sequence[CudaMle]):
        """MSM i = sum_j scalars[i][j] * (layer `layer_index` base j) over the
        first 2^num_vars bases; all MSMs overlap on the device."""
        if not scalars:
            return []
        for m in scalars:
            self._check_mle(m)
        nvs = (ctypes.c_size_t * len(scalars))(*[m.num_vars for m in scalars])
        out = (ctypes.c_uint8 * (97 * len(scalars)))()
        check_status(self.lib.hp_cuda_v1_batch_msm(self.ctx.raw, prover_param.raw, layer_index, _addr_array(scalars),
                                                   nvs, len(scalars), out), "batch_msm")
        raw = bytes(out)
        return [decode_g1(raw[97 * i:97 * i + 97]) for i in range(len(scalars))]

    def batch_prove_round(self, states: Sequence[CudaSumCheckProverState], challenges: Sequence[Optional[int]]):
        """One round of every state (each with its own challenge or None),
        overlapped on the device, one synchronisation."""
        k = len(states)
        if k == 0:
            return []
        sp = (ctypes.c_void_p * k)(*[s.raw.value for s in states])
        keep = [encode_fr(c) if c is not None else None for c in challenges]
        cp = (ctypes.c_void_p * k)(*[ctypes.cast(ctypes.c_char_p(b), ctypes.c_void_p).value if b else None
                                     for b in keep])
        outs = [(ctypes.c_uint8 * (32 * s.round_evaluation_count))() for s in states]
        op = (ctypes.c_void_p * k)(*[ctypes.addressof(o) for o in outs])
        counts = (ctypes.c_size_t * k)(*[s.round_evaluation_count for s in states])
        check_status(self.lib.hp_cuda_v1_batch_sumcheck_round(self.ctx.raw, sp, cp, op, counts, k),
                     "batch_sumcheck_round")
        res = []
        for o, s in zip(outs, states):
            raw = bytes(o)
            res.append([decode_fr(raw[32 * i:32 * i + 32]) for i in range(s.round_evaluation_count)])
        return res

    def final_evaluations(self, state: CudaSumCheckProverState, challenge: int) -> list[int]:
        """Every distinct factor fixed at the full challenge point (after the
        last round), in factor order."""
        k = state.factor_count
        out = (ctypes.c_uint8 * max(1, 32 * k))()
        check_status(self.lib.hp_cuda_v1_sumcheck_prover_state_final_evaluations(
            self.ctx.raw, state.raw, _native.buf(encode_fr(challenge)), out, k),
            "sumcheck_prover_state_final_evaluations")
        raw = bytes(out)
        return [decode_fr(raw[32 * i:32 * i + 32]) for i in range(k)]
