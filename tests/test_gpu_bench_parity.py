"""Parity of the benchmarked configuration against the oracle in the same configuration.

bench.py times the 128x256x128 step at 5 mm (dt 1/240) with 6 seeded floor spots of 1-4 g/s (no logs, no
coal bed), vortEps 0.3, turbAmp 0.2, soot forming after a gas age of 20-60 ms, and the pressure solved to a
1e-5 relative residual with every multigrid sweep over-relaxed (omega 1.2).  At this grid the multigrid's
coarse end runs as the 8-CTA cluster tail from level 3 and forces runs its one-wave z-marching ranges, so
these tests exercise the code paths the benchmark times, from a developed fire (60 steps from rest):

  * every stage from identical inputs (the GPU state before the stage is copied into the oracle), at the
    per-stage tolerance of tests/test_gpu_stages.py; one over-relaxed V-cycle at 1e-4 relative;
  * one whole step as the benchmark runs it (CUDA graph, residual-driven WHILE loop, by-value parameter
    block), at the one-step tolerance of tests/test_gpu_step.py; the cycle count equals the oracle's
    tolerance loop, or exceeds it by one (the device skips the convergence test on the cycles the previous
    step predicts are needed, so it can run one more cycle, never fewer).
"""
import numpy as np
import pytest

import bench
import fire_cases as FC
import fire_sim as F
import oracle as O

pytestmark = pytest.mark.gpu

W = bench.WORKLOAD
RTOL, ATOL, OUTLIERS = 1e-4, 1e-5, 1e-3


@pytest.fixture(scope="module")
def developed():
    """The benchmark's simulation after 60 steps, and an oracle configured identically."""
    sim = bench.make_sim(F, 0)
    sim.step(W["dt"], 60)
    sim.sync()
    orc = O.OracleSim(W["res"], sim.dx)
    orc.set_tables(sim.download("noise").astype(np.float32), sim.download("curl").astype(np.float32))
    orc.set_logs(np.zeros(0, np.float32))
    orc.set_modes(omega=W["mg_omega"])
    yield sim, orc
    sim.close()


def _copy_state(sim, orc):
    for name in FC.FIELD_NAMES:
        orc.put(name, sim.download(name))
    for w in ("p", "b"):
        orc.put_level(0, w, sim.level(0, w))


def _check(sim, orc, names, what, rtol=RTOL, atol=ATOL, outliers=OUTLIERS):
    for name in names:
        g, o = sim.download(name), orc.get(name)
        for c in range(4):
            FC.compare(g[..., c], o[..., c], rtol, atol, outliers, what=f"{what}:{name}[{c}]")


def test_fire_is_developed(developed):
    sim, _ = developed
    assert sim.hrr() > 1.0
    assert 293.0 + 1000.0 * float(sim.download("S")[..., 0].max()) > 1000.0
    assert tuple(sim.info().res) == tuple(W["res"]) and sim.info().n_levels == 6


def test_stages_from_identical_inputs(developed):
    sim, orc = developed
    dt = W["dt"]
    _copy_state(sim, orc)
    FC.sync_block(sim, orc, dt)
    for stage, outs in (("adv1", ["velX", "SX", "S2X"]), ("adv2", ["velY", "SY", "S2Y"]), ("forces", ["velX", "S", "S2"])):
        sim.run_stage(stage, dt)
        sim.sync()
        if stage == "forces":
            orc.stage("curl")   # the GPU forces kernel computes the curl from velY itself
        orc.stage(stage)
        _check(sim, orc, outs, stage)
        _copy_state(sim, orc)   # the next stage starts from identical inputs
    sim.run_stage("div", dt)
    sim.sync()
    orc.stage("div")
    FC.compare(sim.level(0, "b"), orc.get_level(0, "b"), RTOL, ATOL, OUTLIERS, what="div")
    _copy_state(sim, orc)
    # one V-cycle with omega 1.2: level launches on 0-2, the cluster tail over levels 3-5
    sim.run_stage("vcycle", dt)
    sim.sync()
    orc.stage("vcycle")
    FC.compare(sim.level(0, "p"), orc.get_level(0, "p"), 1e-4, 1e-5, 0.0, what="vcycle omega 1.2")
    _copy_state(sim, orc)
    sim.run_stage("project", dt)
    sim.sync()
    orc.stage("project")
    _check(sim, orc, ["vel"], "project")


def test_one_benchmark_step(developed):
    sim, orc = developed
    dt = W["dt"]
    sim.step(dt, 2)   # restores a consistent step state after the stage test
    sim.sync()
    _copy_state(sim, orc)
    FC.sync_block(sim, orc, dt)
    sim.step(dt, 1)
    sim.sync()
    cycles_orc = orc.step_raw(False, -W["mg_max_cycles"], W["mg_tol"])
    info = sim.info()
    assert info.last_cycles in (cycles_orc, cycles_orc + 1), (info.last_cycles, cycles_orc)
    assert info.last_rel_residual <= W["mg_tol"]
    _check(sim, orc, ["vel", "S", "S2", "velX"], "bench step", 1e-3, 1e-4, 5e-3)
    FC.compare(sim.level(0, "p"), orc.get_level(0, "p"), 1e-3, 1e-4, 5e-3, what="bench step:p")
