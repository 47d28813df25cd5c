"""Canonical serialization of the values the prover appends to the transcript
and of the proof objects (ark-serialize 0.6.0 compressed conventions).

- usize / Vec length: u64 little-endian;
- Fr: 32-byte little-endian canonical integer;
- G1 affine (ark-bls12-381 0.6.0 compressed form): 48-byte big-endian x with
  flag bits in the first byte: 0x80 compressed, 0x40 point at infinity (all
  other bits zero), 0x20 set when y is the lexicographically larger root
  (y > (q-1)/2);
- VPAuxInfo: max_degree then num_variables (usize each); PhantomData is empty;
- IOPProverMessage: its Vec<Fr> of evaluations.

The reference's proof structs carry no serialization (HyperPlonkProof,
IOPProof); `proof_bytes` concatenates every field in declaration order with
the conventions above (hyperplonk/src/structs.rs:29-37).
"""
from __future__ import annotations

from .virtual_polynomial import R_MODULUS

Q_MODULUS = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB


def usize(n: int) -> bytes:
    return int(n).to_bytes(8, "little")


def fr(x: int) -> bytes:
    return (x % R_MODULUS).to_bytes(32, "little")


def vec_fr(xs) -> bytes:
    xs = list(xs)
    return usize(len(xs)) + b"".join(fr(x) for x in xs)


def g1_compressed(p) -> bytes:
    if p is None:
        out = bytearray(48)
        out[0] = 0xC0
        return bytes(out)
    x, y = p
    out = bytearray(x.to_bytes(48, "big"))
    out[0] |= 0x80
    if y > (Q_MODULUS - 1) // 2:
        out[0] |= 0x20
    return bytes(out)


def vec_g1(ps) -> bytes:
    ps = list(ps)
    return usize(len(ps)) + b"".join(g1_compressed(p) for p in ps)


def aux_info(max_degree: int, num_variables: int) -> bytes:
    return usize(max_degree) + usize(num_variables)
