"""Generate the golden parity fixtures from the reference's own CPU path.

Runs in the container that holds the reference checkout: it needs
oracle/_ref/libref_cpu.so (built by oracle/build_ref.sh from the reference's
src/cpu/simpleBVH.cpp and src/utils/utils.cpp). For every case of cases.py it
builds one SimpleBVH per mesh, runs the reference detect over the case's
pairs (and over every extra frame after the reference refit), and stores

  * the inputs (or, for the large generated meshes, their SHA-256 digest),
  * the sorted int_tri_pair records {bvhA, bvhB, triA, triB} (original face
    indices) and the number of candidate leaf pairs, per frame,

in tests/golden/<case>.npz.  Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import CASES, REGENERATED  # noqa: E402
from oibvh_gb300.meshes import mesh_digest  # noqa: E402
from oracle.oracle import Reference, sort_pairs  # noqa: E402


def run_case(name: str):
    spec = CASES[name]()
    meshes, pairs, frames = spec["meshes"], spec["pairs"], spec["frames"]
    ref = Reference()
    ids = [ref.add_mesh(m.xyz, m.tri) for m in meshes]
    assert ids == list(range(len(meshes)))
    results = []
    hits, ncand = ref.detect(pairs)
    results.append((sort_pairs(hits), ncand))
    for fr in frames or []:
        for i, xyz in enumerate(fr):
            ref.set_positions(i, xyz)
        hits, ncand = ref.detect(pairs)
        results.append((sort_pairs(hits), ncand))
    out = {"n_meshes": np.int64(len(meshes)), "n_frames": np.int64(len(results))}
    if pairs is not None:
        out["pairs"] = np.asarray(pairs, dtype=np.uint32).reshape(-1, 2)
    for i, m in enumerate(meshes):
        out[f"digest_{i}"] = np.bytes_(mesh_digest(m.xyz, m.tri))
        if name not in REGENERATED:
            out[f"xyz_{i}"] = m.xyz
            out[f"tri_{i}"] = m.tri
    for f, fr in enumerate(frames or []):
        for i, xyz in enumerate(fr):
            out[f"frame{f + 1}_xyz_{i}"] = xyz
    for f, (h, c) in enumerate(results):
        out[f"hits_{f}"] = h
        out[f"candidates_{f}"] = np.int64(c)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return [(len(h), c) for h, c in results]


if __name__ == "__main__":
    if not Reference.available():
        sys.exit("oracle/_ref/libref_cpu.so is missing: run oracle/build_ref.sh first")
    for name in CASES:
        print(name, run_case(name))
