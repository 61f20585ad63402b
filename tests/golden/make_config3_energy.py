"""Regenerate tests/golden/config3_oracle.json: the oracle's FP64 energies for
the N = 100 Heisenberg DMRG workload.

Workload: S=1/2 Heisenberg chain, N = 100, open boundaries, MPO bond dimension
5; random initial MPS of link dimension 16 from the Philox stream (seed 1236,
the same numbers itg.randomCuMPS draws); 10 sweeps with maxdim 16, 32, ...,
1024 (doubling, then 1024), cutoff 1e-12, Davidson krylovdim 3 / maxiter 2.
The oracle is the CPU restatement of ITensors 0.2's two-site dmrg
(oracle/itg_oracle.py, NumPy/LAPACK in FP64); the cutoff keeps every bond at or
below ~190, so the run takes minutes on a few cores.

Usage:  python tests/golden/make_config3_energy.py
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

N, LINKDIM, SEED, NSWEEP, CUTOFF = 100, 16, 1236, 10, 1e-12
MAXDIMS = [16, 32, 64, 128, 256, 512, 1024]


def main():
    from oracle import itg_oracle as O
    t0 = time.time()
    e, A, hist = O.dmrg(O.heisenberg_mpo(N), O.random_mps([2] * N, LINKDIM, SEED), MAXDIMS, [CUTOFF], NSWEEP,
                        return_sweeps=True)
    out = {"workload": "Heisenberg S=1/2 N=100 OBC, random MPS link 16 (Philox seed 1236), 10 sweeps, "
                       "maxdim 16->1024 doubling, cutoff 1e-12, Davidson krylovdim 3 maxiter 2",
           "N": N, "linkdim": LINKDIM, "seed": SEED, "nsweep": NSWEEP, "cutoff": CUTOFF, "maxdims": MAXDIMS,
           "energy": e, "sweep_energies": [h[0] for h in hist], "sweep_maxlinkdim": [h[1] for h in hist],
           "sweep_maxtruncerr": [h[2] for h in hist], "oracle_seconds": round(time.time() - t0, 1)}
    (HERE / "config3_oracle.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
