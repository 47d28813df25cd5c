"""IOPTranscript (transcript/src/lib.rs:30-131) over the native Merlin
transcript of libhp_cuda.so (csrc/transcript.cpp).

Challenges are 64 transcript bytes reduced mod r (Fr::from_le_bytes_mod_order)
and re-appended under the same label as their 32-byte canonical encoding.
"""
from __future__ import annotations

import ctypes

from . import _native
from .errors import check_status
from .virtual_polynomial import R_MODULUS


class TranscriptError(Exception):
    """transcript/src/errors.rs: InvalidTranscript."""


class MerlinTranscript:
    """Native Merlin 1.0 transcript (STROBE-128 / Keccak-f[1600])."""

    def __init__(self, label: bytes, _raw=None):
        self.lib = _native.load()
        if _raw is not None:
            self.raw = _raw
            return
        raw = ctypes.c_void_p()
        check_status(self.lib.hp_host_v1_merlin_new(_native.buf(label), len(label), ctypes.byref(raw)),
                     "merlin_new")
        self.raw = raw

    def append_message(self, label: bytes, message: bytes) -> None:
        check_status(self.lib.hp_host_v1_merlin_append(self.raw, _native.buf(label), len(label),
                                                       _native.buf(message) if message else None, len(message)),
                     "merlin_append")

    def challenge_bytes(self, label: bytes, n: int) -> bytes:
        out = (ctypes.c_uint8 * n)()
        check_status(self.lib.hp_host_v1_merlin_challenge(self.raw, _native.buf(label), len(label), out, n),
                     "merlin_challenge")
        return bytes(out)

    def clone(self) -> "MerlinTranscript":
        raw = ctypes.c_void_p()
        check_status(self.lib.hp_host_v1_merlin_clone(self.raw, ctypes.byref(raw)), "merlin_clone")
        return MerlinTranscript(b"", _raw=raw)

    def __del__(self):
        raw = getattr(self, "raw", None)
        if raw is not None and raw.value:
            self.raw = None
            from .backend import _destroy_or_abort
            _destroy_or_abort("merlin_free", self.lib.hp_host_v1_merlin_free(raw))


class IOPTranscript:
    def __init__(self, label: bytes, merlin_cls=MerlinTranscript):
        self._t = merlin_cls(label)
        self.is_empty = True

    def append_message(self, label: bytes, msg: bytes) -> None:
        self._t.append_message(label, msg)
        self.is_empty = False

    def native_merlin(self):
        """The underlying native transcript when it is one (library calls may
        then append and draw challenges on it directly), else None."""
        return self._t if isinstance(self._t, MerlinTranscript) and not self.is_empty else None

    def append_field_element(self, label: bytes, x: int) -> None:
        self.append_message(label, (x % R_MODULUS).to_bytes(32, "little"))

    def append_serializable_element(self, label: bytes, data: bytes) -> None:
        self.append_message(label, data)

    def get_and_append_challenge(self, label: bytes) -> int:
        if self.is_empty:
            raise TranscriptError("transcript is empty")
        buf = self._t.challenge_bytes(label, 64)
        c = int.from_bytes(buf, "little") % R_MODULUS
        self.append_serializable_element(label, c.to_bytes(32, "little"))
        return c

    def get_and_append_challenge_vectors(self, label: bytes, n: int) -> list[int]:
        if self.is_empty:
            raise TranscriptError("transcript is empty")
        return [self.get_and_append_challenge(label) for _ in range(n)]
