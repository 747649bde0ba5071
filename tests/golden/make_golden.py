"""Generates the golden fixtures under tests/golden/ from the reference's OWN
CPU code (oracle/_ref/libref_{moldyn,minimd}.so, built from the reference
sources by `make -C oracle ref`).

Run in a container that holds the reference tree:
    make -C oracle ref && python tests/golden/make_golden.py

Each fixture (npz) holds seeded inputs and the reference's outputs:
  pos      (n, 3) float64  node coordinates (all float32-representable)
  edges    (e, 2) int32    half list as passed to IrregularRuntime
  param    float64 blob    the reference's parameter block for the map
  map      str             "moldyn" (irregular.h map) or "minimd" (map1)
  f_ref    (n, 3) float32  FCPU::map over all edges into one Cobject
                           (moldyn/irregular.h:26-114, roc.cu:11-65)
  f_exec   (n, 3) float32  the reference's pthread executor compute_cpu with
                           4 workers (cpu_kernel.cu:13-70), merged per thread
The cases follow the configurations' shapes at sizes the oracle finishes in
well under a second.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def random_box(n: int, rho: float, seed: int):
    rng = np.random.Generator(np.random.PCG64(seed))
    L = np.float32((n / rho) ** (1.0 / 3.0))
    pos = (rng.random((n, 3), dtype=np.float32) * L).astype(np.float32)
    pos[pos >= L] = 0.0
    return pos, L


def case_moldyn_random(seed=20260001, n=2048, rho=0.4889, rc=2.5):
    pos32, L = random_box(n, rho, seed)
    edges = O.neighbor_half_list(pos32, float(L), np.float32(rc * rc))
    return dict(pos=pos32.astype(np.float64), edges=edges, map="moldyn",
                param=O.ref_param_bytes("moldyn", rc, float(L)), side=float(L), cutoff=rc)


def case_moldyn_fcc(m=6, rc=3.5, tol=1.2):
    # moldyn's lattice (moldyn.cu:596-626) and list rule rd <= (rc*1.2)^2 (:552-594)
    side = float(np.float32((4 * m ** 3 / 0.83134) ** 0.3333333))
    pos = O.fcc_moldyn(m, side).astype(np.float32)
    # a small seeded jitter so pairs are not all on lattice shells
    rng = np.random.Generator(np.random.PCG64(20260003))
    pos = (pos + rng.normal(0, 0.05, pos.shape).astype(np.float32)) % np.float32(side)
    pos = pos.astype(np.float32)
    edges = O.neighbor_half_list(pos, side, np.float32((rc * tol) ** 2))
    return dict(pos=pos.astype(np.float64), edges=edges, map="moldyn",
                param=O.ref_param_bytes("moldyn", rc, side), side=side, cutoff=rc)


def case_minimd_fcc(nx=6, rho=0.8442, cutforce=2.5, cutneigh=2.8):
    # miniMD lattice (setup.cpp:61-122), open boundaries, list at 2.8, force at 2.5
    pos = O.fcc_minimd(nx, nx, nx, rho).astype(np.float32)
    rng = np.random.Generator(np.random.PCG64(20260004))
    pos = (pos + rng.normal(0, 0.04, pos.shape).astype(np.float32)).astype(np.float32)
    edges = O.neighbor_half_list(pos, 0.0, np.float32(cutneigh * cutneigh))
    return dict(pos=pos.astype(np.float64), edges=edges, map="minimd",
                param=O.ref_param_bytes("minimd", cutforce), side=0.0, cutoff=cutforce)


def case_shuffled_dups(seed=20260005, n=1500, rho=0.6, rc=2.5):
    # unsorted edge order, swapped orientations and duplicated edges
    pos32, L = random_box(n, rho, seed)
    edges = O.neighbor_half_list(pos32, float(L), np.float32(rc * rc))
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    flip = rng.random(edges.shape[0]) < 0.5
    edges[flip] = edges[flip][:, ::-1]
    dup = edges[rng.integers(0, edges.shape[0], edges.shape[0] // 10)]
    edges = np.concatenate([edges, dup])
    edges = edges[rng.permutation(edges.shape[0])].astype(np.int32)
    return dict(pos=pos32.astype(np.float64), edges=edges, map="moldyn",
                param=O.ref_param_bytes("moldyn", rc, float(L)), side=float(L), cutoff=rc)


def case_ragged(seed=20260006):
    # isolated nodes, one hub node with a long row, a pair beyond the cutoff
    rng = np.random.Generator(np.random.PCG64(seed))
    n = 700
    L = np.float32(30.0)
    pos = (rng.random((n, 3), dtype=np.float32) * L).astype(np.float32)
    hub = 5
    near = rng.choice(np.arange(n), 400, replace=False)
    near = near[near != hub]
    pos[near] = (pos[hub] + rng.normal(0, 0.9, (near.size, 3)).astype(np.float32)) % L
    pos = pos.astype(np.float32)
    edges = [(hub, int(j)) for j in near] + [(1, 2), (3, 4)]
    edges = np.array(edges, np.int32)
    return dict(pos=pos.astype(np.float64), edges=edges, map="moldyn",
                param=O.ref_param_bytes("moldyn", 2.5, float(L)), side=float(L), cutoff=2.5)


CASES = {
    "moldyn_random_2048": case_moldyn_random,
    "moldyn_fcc_864": case_moldyn_fcc,
    "minimd_fcc_864": case_minimd_fcc,
    "moldyn_shuffled_dups_1500": case_shuffled_dups,
    "moldyn_ragged_700": case_ragged,
}


def main():
    for which in ("moldyn", "minimd"):
        if not O.ref_available(which):
            raise SystemExit(f"oracle/_ref/libref_{which}.so missing: run `make -C oracle ref`")
    for name, fn in CASES.items():
        c = fn()
        f_ref = O.ref_map_all(c["map"], c["pos"], c["edges"], c["param"])
        f_exec, _ = O.ref_compute_cpu(c["map"], c["pos"], c["edges"], c["param"], 4)
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, pos=c["pos"], edges=c["edges"], param=c["param"],
                            map=np.array(c["map"]), side=np.float64(c["side"]),
                            cutoff=np.float64(c["cutoff"]), f_ref=f_ref, f_exec=f_exec)
        print(f"{name}: n={c['pos'].shape[0]} e={c['edges'].shape[0]} -> {os.path.basename(out)}")


if __name__ == "__main__":
    main()
