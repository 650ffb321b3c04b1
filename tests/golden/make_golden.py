"""Regenerates the golden fixtures in this folder from the reference's own recorded results.

Reads (as text) the reference project's multigrid convergence records:
  research/webgpu-bench/results/poisson-128-face.txt   CPU poisson.mjs study, 128^3, face ghosts
  research/webgpu-bench/results/result-new-mg.json     GPU V-cycle residual ratios (bench.js benchMG)
and writes poisson_128_face.json and mg_gpu_ratios.json.  Run from the repo root:
  python tests/golden/make_golden.py <path-to-reference>
The fixtures are committed; tests never read the reference tree.
"""
import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(ref: Path):
    txt = (ref / "research/webgpu-bench/results/poisson-128-face.txt").read_text()
    out = {"source": "research/webgpu-bench/results/poisson-128-face.txt", "N": 128, "ghost": "face", "lines": []}
    m = re.search(r"initial rms residual ([0-9.e+-]+)", txt)
    out["r0"] = m.group(1)
    for line in txt.splitlines():
        m = re.match(r"^(Jacobi w=([0-9.]+)|RB-SOR w=([0-9.]+)|MG V\((\d),(\d)\) RBGS, (\d+) lvls)\s+(.*?)\s+\(cost", line)
        if not m:
            continue
        pairs = re.findall(r"(\d+):([0-9.]+e[+-]\d+)", m.group(7))
        entry = {"label": m.group(1).strip(), "values": [v for _, v in pairs], "at": [int(k) for k, _ in pairs]}
        if m.group(2):
            entry.update(mode="jacobi", omega=float(m.group(2)))
        elif m.group(3):
            entry.update(mode="rbsor", omega=float(m.group(3)))
        else:
            entry.update(mode="mg", pre=int(m.group(4)), post=int(m.group(5)), levels=int(m.group(6)))
        out["lines"].append(entry)
    (HERE / "poisson_128_face.json").write_text(json.dumps(out, indent=1) + "\n")

    mg = json.loads((ref / "research/webgpu-bench/results/result-new-mg.json").read_text())["results"]["mg"]
    keep = {n: {k: v["residualRatioPerCycle"] for k, v in d.items() if isinstance(v, dict)} for n, d in mg.items()}
    (HERE / "mg_gpu_ratios.json").write_text(json.dumps(
        {"source": "research/webgpu-bench/results/result-new-mg.json", "ratios": keep}, indent=1) + "\n")
    print("wrote", len(out["lines"]), "poisson lines and", len(keep), "mg sizes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path-to-reference-checkout>")
    main(Path(sys.argv[1]))
