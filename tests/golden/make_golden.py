"""Regenerates the committed golden fixtures from the reference's own generator.

Runs backend/src/ascend910b3/native/tests/generate_golden.py of the reference
tree (stdlib Python, seeded; independent affine arithmetic) into a temporary
directory and packs the field, G1 and MSM cases used by the tests into
compact .npz files beside this script.  Large MSM inputs whose bases are the
consecutive multiples 1*G, 2*G, ... are stored as a marker plus the SHA-256
of the reference's bases file; the tests rebuild them and check the digest.

Usage: python tests/golden/make_golden.py --reference /path/to/reference
This is the only file in the repository that reads the reference tree.
"""
from __future__ import annotations

import argparse
import hashlib
import pathlib
import subprocess
import sys
import tempfile

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
GEN = "backend/src/ascend910b3/native/tests/generate_golden.py"
Q = 4002409555221667393417789825735904156556882819939007885332058136124031650490837864442687629129015664037894272559787
G = (3685416753713387016781088315183077757961620795782546409894578378688607592378376318836054947676345821548104185464507,
     1339506544944476473020471379941921221584933875938349620426543736416511423956333506472724655353366534992391756441569)

FIELD_CASES = ["case-0", "case-1", "case-2", "case-31", "case-32", "case-33", "case-47", "case-48", "case-49",
               "case-63", "case-64", "case-65", "case-95", "case-96", "case-97", "case-255", "case-256", "case-257",
               "case-513", "boundaries", "radix-boundaries"]
FIELD_FILES = ["lhs", "rhs", "add", "sub", "mul", "neg", "square", "inverse_input", "inverse"]
G1_FILES = ["affine_a", "affine_b", "mul_u64", "add", "double", "neg", "mul"]


def arr(path: pathlib.Path) -> np.ndarray:
    return np.frombuffer(path.read_bytes(), dtype=np.uint8)


def consecutive_digest(n: int) -> str:
    """SHA-256 of the 96-byte affine encoding of 1*G .. n*G (affine adds)."""
    h = hashlib.sha256()
    x, y = G
    px, py = None, None
    for i in range(n):
        if px is None:
            px, py = x, y
        else:
            if px == x:
                lam = 3 * px * px * pow(2 * py, -1, Q) % Q
            else:
                lam = (py - y) * pow((px - x) % Q, -1, Q) % Q
            nx = (lam * lam - px - x) % Q
            py = (lam * (x - nx) - y) % Q if px != x else (lam * (px - nx) - py) % Q
            px = nx
        h.update(px.to_bytes(48, "little") + py.to_bytes(48, "little"))
    return h.hexdigest()


def pack(out: pathlib.Path, ref: pathlib.Path) -> None:
    with tempfile.TemporaryDirectory() as tmp:
        tmp = pathlib.Path(tmp)
        subprocess.run([sys.executable, str(ref / GEN), "--output", str(tmp)], check=True)
        for name, root in (("fr", tmp), ("fq", tmp / "fq")):
            data = {}
            for case in FIELD_CASES:
                d = root / case
                if not d.exists():
                    continue
                for f in FIELD_FILES:
                    p = d / f"{f}.bin"
                    if p.exists():
                        data[f"{case}/{f}"] = arr(p)
            np.savez_compressed(out / f"{name}_ops.npz", **data)
        wide = {"fr/wide_input": arr(tmp / "wide_input.bin"), "fr/wide_result": arr(tmp / "wide_result.bin"),
                "fq/wide_input": arr(tmp / "fq" / "wide_input.bin"), "fq/wide_result": arr(tmp / "fq" / "wide_result.bin")}
        np.savez_compressed(out / "wide_reduction.npz", **wide)
        g1 = {"generator": arr(tmp / "g1" / "generator.bin")}
        for d in sorted((tmp / "g1").glob("case-*")):
            for f in G1_FILES:
                g1[f"{d.name}/{f}"] = arr(d / f"{f}.bin")
        for d in sorted((tmp / "g1" / "chain").iterdir()):
            for f in ("bases", "scalars", "expected"):
                g1[f"chain/{d.name}/{f}"] = arr(d / f"{f}.bin")
        np.savez_compressed(out / "g1_ops.npz", **g1)

        digests: dict[int, str] = {}
        msm = {}
        for d in sorted((tmp / "msm").iterdir()) + sorted((tmp / "msm-prepared").iterdir()):
            key = d.parent.name + "/" + d.name
            bases = (d / "bases.bin").read_bytes()
            scalars = (d / "scalars.bin").read_bytes()
            n = len(scalars) // 32
            msm[f"{key}/expected"] = arr(d / "expected.bin")
            if n > 300:
                if n not in digests:
                    digests[n] = hashlib.sha256(bases).hexdigest()
                if hashlib.sha256(bases).hexdigest() == consecutive_digest_cached(n, digests):
                    msm[f"{key}/bases_consecutive"] = np.array([n], dtype=np.int64)
                    msm[f"{key}/bases_sha256"] = np.frombuffer(bytes.fromhex(hashlib.sha256(bases).hexdigest()),
                                                               dtype=np.uint8)
                else:
                    msm[f"{key}/bases"] = np.frombuffer(bases, dtype=np.uint8)
            else:
                msm[f"{key}/bases"] = np.frombuffer(bases, dtype=np.uint8)
            if n > 8193:
                msm[f"{key}/scalars_sha256"] = np.frombuffer(hashlib.sha256(scalars).digest(), dtype=np.uint8)
                ints = [int.from_bytes(scalars[i:i + 32], "little") for i in range(0, len(scalars), 32)]
                if all(v == 1 for v in ints):
                    msm[f"{key}/scalars_ones"] = np.array([n], dtype=np.int64)
                else:
                    # uniform cases draw random.Random(20261103 + n).randrange(P) per
                    # scalar; the tests redraw them and check the digest
                    msm[f"{key}/scalars_pyrandom_seed"] = np.array([20261103 + n], dtype=np.int64)
            else:
                msm[f"{key}/scalars"] = np.frombuffer(scalars, dtype=np.uint8)
        np.savez_compressed(out / "msm.npz", **msm)


_consecutive_cache: dict[int, str] = {}


def consecutive_digest_cached(n: int, _unused) -> str:
    if n not in _consecutive_cache:
        _consecutive_cache[n] = consecutive_digest(n)
    return _consecutive_cache[n]


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--reference", required=True, type=pathlib.Path,
                    help="root of a checkout of the reference repository")
    args = ap.parse_args()
    pack(HERE, args.reference)


if __name__ == "__main__":
    main()
