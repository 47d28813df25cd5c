"""TEST INFRASTRUCTURE ONLY -- BLS12-381 G2 and pairing for the verifier.

Python face of the pairing section of hp_oracle.c.  The big integers the C
code takes as limbs are derived here from the curve's published parameters:
the base-field modulus p, the group order r and the curve parameter
z = -0xd201000000010000 (trace of Frobenius t = z + 1):
- the G2 cofactor #E'(Fq2) / r: over Fq2 the trace is t2 = t^2 - 2p; the
  sextic twists have traces +-t2 and (+-t2 +- 3f) / 2 with
  t2^2 - 4p^2 = -3 f^2, and exactly one twist other than E itself has an
  order divisible by r;
- the final exponent (p^12 - 1) / r.

The verifier parameter (multilinear_kzg/srs.rs:158-235: g, h, h_mask[i] =
t_i h) uses the same t_i and g as the testing SRS (oracle.srs_layers) and
h = s H0, with H0 the fixed point of or_g2_derive and s drawn from the same
ChaCha20 stream (block num_vars + 1).
"""
from __future__ import annotations

import ctypes
import functools
from math import isqrt

import oracle  # oracle/oracle.py

P = oracle.Q
R = oracle.R
Z = -0xd201000000010000

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def _limbs(x: int) -> "ctypes.Array":
    n = max(1, (x.bit_length() + 63) // 64)
    return (ctypes.c_uint64 * n)(*[(x >> (64 * i)) & (2**64 - 1) for i in range(n)])


@functools.lru_cache(maxsize=None)
def g2_cofactor() -> int:
    t = Z + 1
    t2 = t * t - 2 * P
    f2 = 4 * P * P - t2 * t2
    f = isqrt(f2 // 3)
    assert 3 * f * f == f2
    found = [P * P + 1 - tau for tau in (-t2, (t2 + 3 * f) // 2, (t2 - 3 * f) // 2, (-t2 + 3 * f) // 2,
                                         (-t2 - 3 * f) // 2) if (P * P + 1 - tau) % R == 0]
    assert len(found) == 1
    return found[0] // R


@functools.lru_cache(maxsize=None)
def final_exponent() -> int:
    assert (P**12 - 1) % R == 0
    return (P**12 - 1) // R


def _lib():
    lib = oracle.load()
    if not getattr(lib, "_pairing_ready", False):
        lib.or_g2_derive.argtypes = [_u64p, ctypes.c_size_t, _u8p]
        lib.or_g2_op.argtypes = [ctypes.c_int, _u8p, _u8p, _u8p, _u8p]
        lib.or_pairing_product_is_one.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u64p, ctypes.c_size_t]
        lib._pairing_ready = True
    return lib


def _buf(data: bytes):
    return ctypes.cast(ctypes.c_char_p(data), _u8p)


G2_INFINITY = bytes(192)


@functools.lru_cache(maxsize=None)
def g2_base() -> bytes:
    """H0: a fixed point of order r on E' (192 bytes: x.c0 x.c1 y.c0 y.c1)."""
    h = _limbs(g2_cofactor())
    out = (ctypes.c_uint8 * 192)()
    if _lib().or_g2_derive(h, len(h), out):
        raise RuntimeError("no G2 point found")
    return bytes(out)


def _g2_op(op: int, a: bytes, b: bytes = G2_INFINITY, k: int = 0) -> bytes:
    out = (ctypes.c_uint8 * 192)()
    kb = (k % R).to_bytes(32, "little")
    if _lib().or_g2_op(op, _buf(a), _buf(b), _buf(kb), out):
        raise oracle.OracleInvalidParameters("malformed G2 point")
    return bytes(out)


def g2_add(a: bytes, b: bytes) -> bytes:
    return _g2_op(0, a, b)


def g2_neg(a: bytes) -> bytes:
    return _g2_op(1, a)


def g2_mul(a: bytes, k: int) -> bytes:
    return _g2_op(2, a, k=k)


def g2_mul_unreduced(a: bytes, k: int) -> bytes:
    """k * a for 0 <= k < 2^256 without reducing k mod r (subgroup checks:
    r * a is the identity exactly for points of order r)."""
    out = (ctypes.c_uint8 * 192)()
    if _lib().or_g2_op(2, _buf(a), _buf(G2_INFINITY), _buf(k.to_bytes(32, "little")), out):
        raise oracle.OracleInvalidParameters("malformed G2 point")
    return bytes(out)


def g1_bytes(p) -> bytes:
    """G1 as (x, y) ints or None -> 96-byte affine packet."""
    if p is None:
        return bytes(96)
    return p[0].to_bytes(48, "little") + p[1].to_bytes(48, "little")


def pairing_product_is_one(pairs) -> bool:
    """prod e(P_i, Q_i) == 1 for (G1 (x, y) / None, G2 192-byte) pairs."""
    g1 = b"".join(g1_bytes(p) for p, _ in pairs)
    g2 = b"".join(q for _, q in pairs)
    fe = _limbs(final_exponent())
    res = _lib().or_pairing_product_is_one(_buf(g1 or b"\0"), _buf(g2 or b"\0"), len(pairs), fe, len(fe))
    if res < 0:
        raise oracle.OracleInvalidParameters("malformed pairing input")
    return res == 1


def srs_verifier_param(num_vars: int, seed: int) -> dict:
    """g (G1 (x, y)), h and h_mask (192-byte G2) of the testing SRS of
    oracle.srs_layers(num_vars, seed) (and of the device generator with the
    same seed): h_mask[i] = t_i h.  Needs only the seed's stream, not the
    layers."""
    def stream_fr(i: int) -> int:
        return oracle.fr_int(oracle.fr_from_wide(oracle.chacha20_block(seed, i)))

    # the SRS's last layer [g]: g = s_g G1 with s_g from block num_vars (or_srs_gen)
    g = oracle.affine_to_point(oracle.msm(oracle.g1_generator(), stream_fr(num_vars).to_bytes(32, "little")))
    ts = [stream_fr(i) for i in range(num_vars)]
    s = stream_fr(num_vars + 1)
    h = g2_mul(g2_base(), s)
    return {"num_vars": num_vars, "g": g, "h": h, "h_mask": [g2_mul(h, t) for t in ts]}
