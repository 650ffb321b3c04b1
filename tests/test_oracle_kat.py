"""Pins the CPU oracle to the reference's own recorded multigrid study (poisson.mjs, 128^3, face ghosts).

research/webgpu-bench/poisson.mjs:8-124 printed residual histories that the reference committed as
results/poisson-128-face.txt; the oracle restates that program and must reproduce every printed value
(two significant digits) exactly, plus the initial RMS residual.
"""
import json
from pathlib import Path

import pytest

GOLD = json.loads((Path(__file__).parent / "golden" / "poisson_128_face.json").read_text())


def fmt(x: float, digits: int = 1) -> str:
    """JavaScript Number.prototype.toExponential(digits)."""
    m, e = f"{x:.{digits}e}".split("e")
    return f"{m}e{int(e):+d}"


def test_initial_residual(oracle_mod):
    r0, _ = oracle_mod.poisson_study(128, True, 2, cycles=1)
    assert fmt(r0, 3) == GOLD["r0"]


@pytest.mark.parametrize("line", GOLD["lines"], ids=[l["label"] for l in GOLD["lines"]])
def test_poisson_line(oracle_mod, line):
    if line["mode"] == "mg":
        _, hist = oracle_mod.poisson_study(128, True, 2, pre=line["pre"], post=line["post"], coarse=30,
                                           cycles=len(line["values"]))
    else:
        omega = 6.0 / 7.0 if line["label"].startswith("Jacobi w=0.857") else line["omega"]
        _, hist = oracle_mod.poisson_study(128, True, 0 if line["mode"] == "jacobi" else 1, omega=omega)
    got = [fmt(v) for v in hist]
    assert got == line["values"], (line["label"], got)
