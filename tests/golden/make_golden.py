"""Regenerate tests/golden/reference_known_answers.json.

Reads the reference's own test files as text (they are Julia; nothing is run)
and extracts the known answers that pin the hot path:

* test/test_cutruncate.jl:9-17 — the three truncate! golden vectors;
* test/dmrg.jl:58-81 — the critical TFIM case (N, field, sweeps, cutoff and
  the closed-form energy with its relative tolerance);
* test/dmrg.jl:5-29 — the S=1 Heisenberg bound (N, sweeps, energy < -12).

It also adds exact-diagonalisation energies from the oracle (scipy eigsh in
the Sz = 0 sector) for the S=1/2 Heisenberg chains the DMRG tests use.

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))


def _floats(s):
    return [float(x) for x in re.findall(r"-?\d+\.?\d*(?:[eE]-?\d+)?", s)]


def parse_truncate(text: str):
    cases = []
    # zero spectrum: truncate!(CUDA.zeros(Float64, 10)) == (0., 0., CUDA.zeros(Float64, 1))
    m = re.search(r"truncate!\(CUDA\.zeros\(Float64,\s*(\d+)\)\)\s*==\s*\(([^,]+),\s*([^,]+),\s*CUDA\.zeros\(Float64,\s*(\d+)\)\)", text)
    if m:
        n = int(m.group(1))
        cases.append({"P": [0.0] * n, "kwargs": {}, "truncerr": float(m.group(2).rstrip('.') or 0),
                      "docut": float(m.group(3).rstrip('.') or 0), "kept": [0.0] * int(m.group(4)),
                      "source": "test/test_cutruncate.jl:9"})
    # trunc = ITensorsGPU.truncate!(CuArray([...]); kw...) followed by three @test lines
    for m in re.finditer(r"trunc = ITensorsGPU\.truncate!\(CuArray\(\[([^\]]*)\]\);\s*([^)]*)\)\s*\n"
                         r"\s*@test trunc\[1\] ≈ ([^\n]+)\n\s*@test trunc\[2\] ≈ ([^\n]+)\n"
                         r"\s*@test trunc\[3\] == CuArray\(\[([^\]]*)\]\)", text):
        P = _floats(m.group(1))
        kw = {}
        for part in m.group(2).split(","):
            if "=" in part:
                k, v = [x.strip() for x in part.split("=")]
                kw[k] = (v == "true") if v in ("true", "false") else float(v)
        line = text[: m.start()].count("\n") + 1
        cases.append({"P": P, "kwargs": kw, "truncerr": float(m.group(3)), "docut": float(m.group(4)),
                      "kept": _floats(m.group(5)), "source": f"test/test_cutruncate.jl:{line}-{line + 3}"})
    return cases


def parse_dmrg(text: str):
    out = {}
    tf = re.search(r'@testset "Transverse field Ising" begin(.*?@test abs[^\n]*\n)', text, re.S)
    if tf:
        body = tf.group(1)
        out["tfim"] = {
            "N": int(re.search(r"N = (\d+)", body).group(1)),
            "seed": int(re.search(r"Random\.seed!\((\d+)\)", body).group(1)),
            "J": -float(re.search(r'add!\(ampo,(-?[\d.]+),"Sz",j,"Sz",j\+1\)', body).group(1)),
            "h": -float(re.search(r'add!\(ampo,(-?[\d.]+),"Sx",j\)', body).group(1)),
            "nsweep": int(re.search(r"Sweeps\((\d+)\)", body).group(1)),
            "maxdim": [int(x) for x in re.search(r"maxdim!\(sweeps,([\d,]+)\)", body).group(1).split(",")],
            "cutoff": float(re.search(r"cutoff!\(sweeps,([\dEe.+-]+)\)", body).group(1)),
            "rel_tol": float(re.search(r"energy_exact\)/energy_exact\) < ([\dEe.+-]+)", body).group(1)),
            "source": "test/dmrg.jl:58-81",
        }
    s1 = re.search(r'@testset "Spin-one Heisenberg" begin(.*?@test energy[^\n]*\n)', text, re.S)
    if s1:
        body = s1.group(1)
        out["spin1_heisenberg"] = {
            "N": int(re.search(r"N = (\d+)", body).group(1)),
            "nsweep": int(re.search(r"Sweeps\((\d+)\)", body).group(1)),
            "maxdim": [int(x) for x in re.search(r"maxdim!\(sweeps,([\d,]+)\)", body).group(1).split(",")],
            "mindim": [int(x) for x in re.search(r"mindim!\(sweeps,([\d,]+)\)", body).group(1).split(",")],
            "cutoff": float(re.search(r"cutoff!\(sweeps,([\dEe.+-]+)\)", body).group(1)),
            "energy_below": float(re.search(r"@test energy < ([-\d.]+)", body).group(1)),
            "source": "test/dmrg.jl:5-29",
        }
    return out


def main(ref: Path):
    data = {
        "truncate": parse_truncate((ref / "test/test_cutruncate.jl").read_text()),
        "dmrg": parse_dmrg((ref / "test/dmrg.jl").read_text()),
    }
    from oracle import itg_oracle as O
    data["ed"] = {f"heisenberg_N{n}": O.heisenberg_ed_sz0(n) for n in (8, 10, 12, 20)}
    (HERE / "reference_known_answers.json").write_text(json.dumps(data, indent=1) + "\n")
    print(json.dumps(data, indent=1))


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference"))
