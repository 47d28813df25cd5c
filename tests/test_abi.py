"""CPU checks of the boundary: the library builds, loads and exports every
entry point declared in include/hp_cuda.h; the status mapping and packet
codecs mirror backend/src/ascend910b3/{status,encoding}.rs.  No device calls."""
import pathlib
import re

import pytest

from hyperplonk_gb300 import _native
from hyperplonk_gb300.backend import decode_g1, encode_g1, encode_fr, decode_fr
from hyperplonk_gb300.errors import InvalidParameters, InvalidState, check_status

ROOT = pathlib.Path(__file__).resolve().parent.parent
R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
G = (3685416753713387016781088315183077757961620795782546409894578378688607592378376318836054947676345821548104185464507,
     1339506544944476473020471379941921221584933875938349620426543736416511423956333506472724655353366534992391756441569)


def declared_entries():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"\b(hp_(?:cuda|host)_v1_\w+)\s*\(", h.read_text()))
    return sorted(names)


def test_library_exports_every_declared_entry(native_lib):
    declared = declared_entries()
    assert len(declared) >= 23
    missing = [n for n in declared if getattr(native_lib, n, None) is None]
    assert not missing, missing
    # the ctypes table binds every declared entry
    assert set(declared) <= set(_native.SIGNATURES)


def test_status_mapping():
    S = _native.Status
    check_status(S(0, 0), "op")
    for kind, code in [(0, 7), (2, 0), (2, -42), (3, 0), (3, 9), (-1, 0), (99, 0)]:
        with pytest.raises(InvalidState):
            check_status(S(kind, code), "op")
    for code in (0, -42, 7):
        with pytest.raises(InvalidParameters):
            check_status(S(1, code), "op")


def test_packets():
    assert decode_fr(encode_fr(R - 1)) == R - 1
    with pytest.raises(InvalidState):
        decode_fr(R.to_bytes(32, "little"))
    assert decode_g1(encode_g1(G)) == G
    assert decode_g1(encode_g1(None)) is None
    bad = bytearray(encode_g1(None))
    bad[5] = 1
    with pytest.raises(InvalidState):
        decode_g1(bytes(bad))
    off = bytearray(encode_g1(G))
    off[60] ^= 1
    with pytest.raises(InvalidState):
        decode_g1(bytes(off))
    with pytest.raises(InvalidState):
        decode_g1(b"\x02" + bytes(96))
