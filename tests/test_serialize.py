"""The compressed G1 encoding (ark-bls12-381 0.6.0, the zcash-style format:
48-byte big-endian x, flag bits 0x80 compressed / 0x40 infinity / 0x20 larger
y) pinned against the published encodings of the BLS12-381 G1 generator and
of the point at infinity, for both the product serializer and the oracle
prover's own one.  CPU only."""
import pytest

from hyperplonk_gb300 import serialize as ser

import prover as oprover  # oracle/prover.py

Q = ser.Q_MODULUS
# the standard BLS12-381 G1 generator, uncompressed big-endian x || y
G_UNCOMPRESSED = ("17f1d3a73197d7942695638c4fa9ac0fc3688c4f9774b905a14e3a3f171bac586c55e83ff97a1aeffb3af00adb22c6bb"
                  "08b3f481e3aaa0f1a09e30ed741d8ae4fcf5e095d5d00af600db18cb2c04b3edd03cc744a2888ae40caa232946c5e7e1")
# its published compressed encoding
G_COMPRESSED = "97f1d3a73197d7942695638c4fa9ac0fc3688c4f9774b905a14e3a3f171bac586c55e83ff97a1aeffb3af00adb22c6bb"
INFINITY_COMPRESSED = "c0" + "00" * 47

GX = int(G_UNCOMPRESSED[:96], 16)
GY = int(G_UNCOMPRESSED[96:], 16)

ENCODERS = [ser.g1_compressed, oprover.g1_compressed]


def test_generator_is_on_the_curve():
    assert (GY * GY - GX ** 3 - 4) % Q == 0


def test_oracle_generator_is_the_standard_one(oracle):
    assert oracle.affine_to_point(oracle.g1_generator()) == (GX, GY)


@pytest.mark.parametrize("enc", ENCODERS, ids=["product", "oracle"])
def test_generator_compressed(enc):
    assert enc((GX, GY)).hex() == G_COMPRESSED


@pytest.mark.parametrize("enc", ENCODERS, ids=["product", "oracle"])
def test_negated_generator_sets_the_sign_flag(enc):
    b = enc((GX, Q - GY))
    assert b[0] == int(G_COMPRESSED[:2], 16) | 0x20 and b[1:] == bytes.fromhex(G_COMPRESSED)[1:]


@pytest.mark.parametrize("enc", ENCODERS, ids=["product", "oracle"])
def test_infinity_compressed(enc):
    assert enc(None).hex() == INFINITY_COMPRESSED
