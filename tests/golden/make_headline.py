"""Writes tests/golden/headline.json: the oracle's results for the measured
workloads at their stated sizes, for the GPU parity tests that compare the
GB300 results with them byte for byte.

Everything here runs on the oracle alone (oracle/oracle.py over
hp_oracle.c, the oracle's own prover oracle/prover.py and its pure-Python
transcript); nothing of the product package is imported.

  commit   one multilinear-KZG commit, num_vars = 16: stream-0 scalars
           [0, 2^16) over layer 0 of the testing SRS of nv = 16, seed 0
  sumcheck the degree-2 instance at nv = 20, seed 1: point, round messages
           and the six final folded values
  prove    the vanilla-plonk proof at nv = 20 (circuit seed 2, testing SRS
           nv = 20 seed 0), serialized
  wired    the same circuit with copy constraints that are not the identity
           at nv = 14 (SRS nv = 14 seed 0); wired20: the same at nv = 20
  batch    the batch plan (seed 3): 64 MSMs over prefixes of layer 0 of the
           nv = 22 SRS (seed 0) and 32 sumcheck instances of 14..22 variables
  serve    8 serving requests, num_vars 16..18 (seed 4), each proven against
           the trimmed nv = 18 SRS (seed 0)

SRS digests: SHA-256 of all layers' 96-byte affine points (x || y, 48-byte
little-endian each, (0, 0) for infinity), layer 0 first.

Usage: python tests/golden/make_headline.py [--only SECTION ...]
(about 15 minutes on 8 cores; existing sections are kept unless named).
"""
from __future__ import annotations

import argparse
import base64
import hashlib
import json
import pathlib
import sys
import time

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))

import oracle as orc  # noqa: E402
import prover as op  # noqa: E402

OUT = HERE / "headline.json"


def srs_digest(layers) -> str:
    h = hashlib.sha256()
    for layer in layers:
        h.update(layer)
    return h.hexdigest()


def commit_section():
    nv = 16
    layers = orc.srs_layers(nv, 0)
    scalars = orc.random_fr(0, 1 << nv)
    point = orc.affine_to_point(orc.msm(layers[0], scalars))
    return {"num_vars": nv, "srs_seed": 0, "scalar_seed": 0, "srs_sha256": srs_digest(layers),
            "commitment": op.g1_compressed(point).hex()}


def sumcheck_section():
    nv, seed = 20, 1
    point, msgs, finals = op.sumcheck_prove_instance(nv, seed)
    return {"num_vars": nv, "seed": seed, "point": [op.fr(x).hex() for x in point],
            "messages": [[op.fr(x).hex() for x in m] for m in msgs], "finals": [op.fr(x).hex() for x in finals]}


def prove_section(nv: int, wired: bool):
    layers = orc.srs_layers(nv, 0)
    proof = op.prove_fixture(nv, 2, wired=wired, srs_layers=layers)
    return {"num_vars": nv, "seed": 2, "srs_seed": 0, "wired": wired, "srs_sha256": srs_digest(layers),
            "proof_sha256": hashlib.sha256(proof).hexdigest(), "proof_len": len(proof),
            "proof_b64": base64.b64encode(proof).decode()}


def batch_section():
    nv_srs = 22
    layers = orc.srs_layers(nv_srs, 0)
    ks, nvs = op.batch_plan(3)
    commits = []
    for k, s in zip(ks, op.batch_msm_scalars(ks, 3)):
        commits.append(op.g1_compressed(orc.affine_to_point(orc.msm(layers[0][:96 << k], s))).hex())
    sums = [op.sumcheck_digest(*op.sumcheck_prove_instance(nv, 100 + 3 + i)) for i, nv in enumerate(nvs)]
    return {"srs_num_vars": nv_srs, "srs_seed": 0, "seed": 3, "msm_log_sizes": ks, "sumcheck_num_vars": nvs,
            "layer0_sha256": hashlib.sha256(layers[0]).hexdigest(), "commitments": commits, "sumchecks": sums}


def serve_section():
    nv_max = 18
    layers = orc.srs_layers(nv_max, 0)
    reqs = op.serve_requests(8, 16, nv_max, 4)
    out = []
    for nv, ws in reqs:
        proof = op.prove_fixture(nv, 2, srs_layers=layers[nv_max - nv:], witness_seed=ws)
        out.append({"num_vars": nv, "witness_seed": ws, "proof_sha256": hashlib.sha256(proof).hexdigest()})
    return {"nv_max": nv_max, "srs_seed": 0, "circuit_seed": 2, "requests": out}


SECTIONS = {
    "commit": commit_section,
    "sumcheck": sumcheck_section,
    "prove": lambda: prove_section(20, False),
    "wired": lambda: prove_section(14, True),
    "wired20": lambda: prove_section(20, True),
    "batch": batch_section,
    "serve": serve_section,
}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--only", nargs="*", choices=sorted(SECTIONS), default=None)
    args = ap.parse_args()
    data = json.loads(OUT.read_text()) if OUT.exists() else {}
    threads = orc.set_threads(0)
    for name in args.only or list(SECTIONS):
        t0 = time.perf_counter()
        data[name] = SECTIONS[name]()
        data[name]["oracle_seconds"] = round(time.perf_counter() - t0, 1)
        data[name]["oracle_threads"] = threads
        OUT.write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
        print(f"{name}: {data[name]['oracle_seconds']} s", flush=True)


if __name__ == "__main__":
    main()
