"""TEST INFRASTRUCTURE ONLY -- independent pure-Python restatement of the
reference's transcript (transcript/src/lib.rs:30-131 over merlin 3.0.0):
Merlin 1.0 framing, STROBE-128, Keccak-f[1600] (FIPS 202).  Slow; used only
by the oracle prover in parity tests.  Keccak-f is pinned in the tests by
building SHA3-256 on it and comparing with hashlib.
"""
from __future__ import annotations

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
MASK = (1 << 64) - 1


def _round_constants():
    out = []
    for ir in range(24):
        c = 0
        for j in range(7):
            t = j + 7 * ir
            if t % 255 == 0:
                bit = 1
            else:
                r = 1
                for _ in range(t % 255):
                    r <<= 1
                    if r & 0x100:
                        r ^= 0x171
                bit = r & 1
            if bit:
                c |= 1 << ((1 << j) - 1)
        out.append(c)
    return out


def _rotations():
    rot = [[0] * 5 for _ in range(5)]
    x, y = 1, 0
    for t in range(24):
        rot[x][y] = ((t + 1) * (t + 2) // 2) % 64
        x, y = y, (2 * x + 3 * y) % 5
    return rot


RC = _round_constants()
ROT = _rotations()


def keccak_f1600(state: bytearray) -> None:
    a = [[int.from_bytes(state[8 * (x + 5 * y):8 * (x + 5 * y) + 8], "little") for y in range(5)] for x in range(5)]
    for rnd in range(24):
        c = [a[x][0] ^ a[x][1] ^ a[x][2] ^ a[x][3] ^ a[x][4] for x in range(5)]
        d = [c[(x - 1) % 5] ^ (((c[(x + 1) % 5] << 1) | (c[(x + 1) % 5] >> 63)) & MASK) for x in range(5)]
        a = [[a[x][y] ^ d[x] for y in range(5)] for x in range(5)]
        b = [[0] * 5 for _ in range(5)]
        for x in range(5):
            for y in range(5):
                r = ROT[x][y]
                v = a[x][y]
                b[y][(2 * x + 3 * y) % 5] = ((v << r) | (v >> (64 - r))) & MASK if r else v
        a = [[b[x][y] ^ ((~b[(x + 1) % 5][y]) & b[(x + 2) % 5][y]) for y in range(5)] for x in range(5)]
        a[0][0] ^= RC[rnd]
    for x in range(5):
        for y in range(5):
            state[8 * (x + 5 * y):8 * (x + 5 * y) + 8] = a[x][y].to_bytes(8, "little")


def sha3_256(msg: bytes) -> bytes:
    """FIPS 202 SHA3-256 on keccak_f1600 (rate 136, pad 0x06 ... 0x80)."""
    rate = 136
    st = bytearray(200)
    data = bytearray(msg) + b"\x06" + bytes((-len(msg) - 1) % rate)
    data[-1] |= 0x80
    for off in range(0, len(data), rate):
        for i in range(rate):
            st[i] ^= data[off + i]
        keccak_f1600(st)
    return bytes(st[:32])


STROBE_R = 166
I, A, C, T, M, K = 1, 2, 4, 8, 16, 32


class Strobe128:
    def __init__(self, label: bytes):
        self.st = bytearray(200)
        self.st[0:6] = bytes([1, STROBE_R + 2, 1, 0, 1, 96])
        self.st[6:18] = b"STROBEv1.0.2"
        keccak_f1600(self.st)
        self.pos = self.pos_begin = self.cur_flags = 0
        self.meta_ad(label, False)

    def _run_f(self):
        self.st[self.pos] ^= self.pos_begin
        self.st[self.pos + 1] ^= 0x04
        self.st[STROBE_R + 1] ^= 0x80
        keccak_f1600(self.st)
        self.pos = self.pos_begin = 0

    def _absorb(self, data: bytes):
        for byte in data:
            self.st[self.pos] ^= byte
            self.pos += 1
            if self.pos == STROBE_R:
                self._run_f()

    def _squeeze(self, n: int) -> bytes:
        out = bytearray(n)
        for i in range(n):
            out[i] = self.st[self.pos]
            self.st[self.pos] = 0
            self.pos += 1
            if self.pos == STROBE_R:
                self._run_f()
        return bytes(out)

    def _begin_op(self, flags: int, more: bool):
        if more:
            assert self.cur_flags == flags
            return
        assert flags & T == 0
        old = self.pos_begin
        self.pos_begin = self.pos + 1
        self.cur_flags = flags
        self._absorb(bytes([old, flags]))
        if flags & (C | K) and self.pos != 0:
            self._run_f()

    def meta_ad(self, data: bytes, more: bool):
        self._begin_op(M | A, more)
        self._absorb(data)

    def ad(self, data: bytes, more: bool):
        self._begin_op(A, more)
        self._absorb(data)

    def prf(self, n: int, more: bool) -> bytes:
        self._begin_op(I | A | C, more)
        return self._squeeze(n)


class Merlin:
    def __init__(self, label: bytes):
        self.s = Strobe128(b"Merlin v1.0")
        self.append_message(b"dom-sep", label)

    def append_message(self, label: bytes, msg: bytes):
        self.s.meta_ad(label, False)
        self.s.meta_ad(len(msg).to_bytes(4, "little"), True)
        self.s.ad(msg, False)

    def challenge_bytes(self, label: bytes, n: int) -> bytes:
        self.s.meta_ad(label, False)
        self.s.meta_ad(n.to_bytes(4, "little"), True)
        return self.s.prf(n, False)


class OracleIOPTranscript:
    """transcript/src/lib.rs:30-120."""

    def __init__(self, label: bytes):
        self.t = Merlin(label)
        self.is_empty = True

    def append_message(self, label: bytes, msg: bytes):
        self.t.append_message(label, msg)
        self.is_empty = False

    def append_field_element(self, label: bytes, x: int):
        self.append_message(label, (x % R).to_bytes(32, "little"))

    def append_serializable_element(self, label: bytes, data: bytes):
        self.append_message(label, data)

    def get_and_append_challenge(self, label: bytes) -> int:
        if self.is_empty:
            raise ValueError("transcript is empty")
        c = int.from_bytes(self.t.challenge_bytes(label, 64), "little") % R
        self.append_serializable_element(label, c.to_bytes(32, "little"))
        return c

    def get_and_append_challenge_vectors(self, label: bytes, n: int) -> list:
        if self.is_empty:
            raise ValueError("transcript is empty")
        return [self.get_and_append_challenge(label) for _ in range(n)]
